// Host-side plumbing shared by the C ABI translation units: status codes,
// per-device workspace arena, error latch and timing.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/gqf.h"

namespace gqf {

#define GQF_CK(expr)                                   \
    do {                                               \
        cudaError_t e_ = (expr);                       \
        if (e_ != cudaSuccess) {                       \
            ::gqf::note_cuda_error(e_, #expr, __LINE__); \
            return GQF_ERR_CUDA;                       \
        }                                              \
    } while (0)

void note_cuda_error(cudaError_t e, const char *what, int line);

struct DeviceInfo {
    int sms = 0;
    int smem_optin = 0;
    int l2_bytes = 0;
};
const DeviceInfo &device_info(int dev);

// Grow-only scratch arena, one per (device, stream).  Calls on one stream
// are serialised by the arena mutex held for the duration of each entry
// point and run in stream order on the device.  The buffer comes from the
// device's stream-ordered pool on that stream, so growing it frees the old
// one behind the queued work instead of waiting for the device.
struct Arena {
    void *ptr = nullptr;
    size_t size = 0;
    cudaStream_t stream = nullptr;
    uint32_t *latch = nullptr;  // persistent per-device error latch
    uint32_t *err = nullptr;    // per-call device error word
    // two words of mapped pinned host memory: a synchronous call's error
    // word (and one more flag) land here from the device, so the host reads
    // them after the call's end event without a device-to-host copy
    volatile uint32_t *report = nullptr;
    uint32_t *report_dev = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // a side stream for work that can run beside the call's own kernels
    // (the in-place updates' table snapshot), forked from and joined back
    // into the call's stream by events
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    std::mutex mu;
};
// The side stream of the arena, created on first use (nullptr on failure).
cudaStream_t arena_side(Arena &a);
Arena &arena(int dev, cudaStream_t s);
// Frees the arena of (dev, s) after the stream drains.
int release_arena(int dev, cudaStream_t s);
// Ensures the arena holds `bytes`; returns its base (nullptr on failure).
void *arena_reserve(Arena &a, size_t bytes);

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Carves consecutive aligned sub-buffers out of a base pointer.
struct Carver {
    char *base;
    size_t off = 0;
    explicit Carver(void *b) : base(static_cast<char *>(b)) {}
    template <typename T>
    T *take(size_t count, size_t align = 256)
    {
        off = align_up(off, align);
        T *p = reinterpret_cast<T *>(base + off);
        off += count * sizeof(T);
        return p;
    }
};
// Same walk without a base, to size a request.
struct Sizer {
    size_t off = 0;
    template <typename T>
    T *take(size_t count, size_t align = 256)
    {
        off = align_up(off, align);
        off += count * sizeof(T);
        return nullptr;
    }
};

// Begins a timed / error-checked call on `stream`: clears the call's error
// word and records the start event when timing.
int call_begin(Arena &a, cudaStream_t s, bool timed);
// Ends the call: when `ms` is non-null waits, stores elapsed ms and maps the
// device error word to a status; otherwise ORs the error word into the
// device latch for gqf_stream_status.
int call_end(Arena &a, cudaStream_t s, float *ms);
// Synchronous end of a step of a call: the device copies the error word
// (and *extra, if given) into the arena's mapped host words, the host waits
// for the stream and returns them in out[0], out[1].
int call_report(Arena &a, cudaStream_t s, const uint32_t *extra, uint32_t out[2]);
int dev_err_to_status(uint32_t e);

int current_device();

// Kernel launches issued by this library (instrumentation for benchmarks).
void count_launches(unsigned n);

}  // namespace gqf
