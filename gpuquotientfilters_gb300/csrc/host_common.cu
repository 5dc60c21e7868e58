// Host plumbing: device info, arenas, error latch, timing, MT19937, hash.
#include "host_common.cuh"
#include "qf_device.cuh"

#include <atomic>
#include <cstring>
#include <map>
#include <memory>

namespace gqf {

static thread_local char g_last_error[256];

void note_cuda_error(cudaError_t e, const char *what, int line)
{
    snprintf(g_last_error, sizeof(g_last_error), "%s (%s) at line %d", cudaGetErrorString(e), what, line);
}

static std::atomic<unsigned long long> g_launches{0};
void count_launches(unsigned n) { g_launches += n; }

int current_device()
{
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) return 0;
    return d;
}

const DeviceInfo &device_info(int dev)
{
    static DeviceInfo info[64];
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    DeviceInfo &d = info[dev & 63];
    if (d.sms == 0) {
        cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&d.l2_bytes, cudaDevAttrL2CacheSize, dev);
        if (d.sms <= 0) d.sms = 1;
    }
    return d;
}

// One arena per (device, stream): calls on one stream run in order and
// reuse its scratch; calls on different streams get different scratch, so
// they may overlap on the device.
static std::mutex g_arena_mu;
static std::map<std::pair<int, cudaStream_t>, std::unique_ptr<Arena>> g_arenas;

Arena &arena(int dev, cudaStream_t s)
{
    std::lock_guard<std::mutex> lk(g_arena_mu);
    std::unique_ptr<Arena> &a = g_arenas[std::make_pair(dev, s)];
    if (!a) {
        a.reset(new Arena());
        a->stream = s;
    }
    return *a;
}

int release_arena(int dev, cudaStream_t s)
{
    std::unique_ptr<Arena> a;
    {
        std::lock_guard<std::mutex> lk(g_arena_mu);
        auto it = g_arenas.find(std::make_pair(dev, s));
        if (it == g_arenas.end()) return GQF_OK;
        std::lock_guard<std::mutex> lk2(it->second->mu);
        a = std::move(it->second);
        g_arenas.erase(it);
    }
    if (a->ptr) GQF_CK(cudaFreeAsync(a->ptr, s));
    GQF_CK(cudaStreamSynchronize(s));
    if (a->latch) GQF_CK(cudaFree(a->latch));
    if (a->report) GQF_CK(cudaFreeHost(const_cast<uint32_t *>(a->report)));
    if (a->ev0) cudaEventDestroy(a->ev0);
    if (a->ev1) cudaEventDestroy(a->ev1);
    if (a->side) {
        GQF_CK(cudaStreamSynchronize(a->side));
        cudaStreamDestroy(a->side);
        cudaEventDestroy(a->fork);
        cudaEventDestroy(a->join);
    }
    return GQF_OK;
}

cudaStream_t arena_side(Arena &a)
{
    if (!a.side) {
        if (cudaStreamCreateWithFlags(&a.side, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
        if (cudaEventCreateWithFlags(&a.fork, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        if (cudaEventCreateWithFlags(&a.join, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    }
    return a.side;
}

void *arena_reserve(Arena &a, size_t bytes)
{
    if (!a.latch) {
        uint32_t *p = nullptr;
        if (cudaMalloc(&p, 2 * sizeof(uint32_t)) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, 2 * sizeof(uint32_t)) != cudaSuccess) return nullptr;
        a.latch = p;
        a.err = p + 1;
        uint32_t *h = nullptr;
        if (cudaHostAlloc(reinterpret_cast<void **>(&h), 2 * sizeof(uint32_t), cudaHostAllocMapped) != cudaSuccess)
            return nullptr;
        h[0] = h[1] = 0;
        if (cudaHostGetDevicePointer(reinterpret_cast<void **>(&a.report_dev), h, 0) != cudaSuccess) return nullptr;
        a.report = h;
        cudaEventCreate(&a.ev0);
        cudaEventCreate(&a.ev1);
    }
    if (bytes <= a.size && a.ptr) return a.ptr;
    if (a.ptr) {
        // work queued on the stream may still use the old buffer: free it in
        // stream order, behind that work
        cudaFreeAsync(a.ptr, a.stream);
        a.ptr = nullptr;
        a.size = 0;
    }
    size_t want = align_up(bytes < (1u << 20) ? (1u << 20) : bytes, 1u << 20);
    if (cudaMallocAsync(&a.ptr, want, a.stream) != cudaSuccess) {
        a.ptr = nullptr;
        cudaGetLastError();
        return nullptr;
    }
    a.size = want;
    return a.ptr;
}

int dev_err_to_status(uint32_t e)
{
    if (e & DEV_ERR_TIMEOUT) return GQF_ERR_TIMEOUT;
    if (e & (DEV_ERR_FULL | DEV_ERR_BUCKET_CAP)) return GQF_ERR_FULL;
    return GQF_OK;
}

int call_begin(Arena &a, cudaStream_t s, bool timed)
{
    if (!arena_reserve(a, 0)) return GQF_ERR_NOMEM;
    GQF_CK(cudaMemsetAsync(a.err, 0, sizeof(uint32_t), s));
    if (timed) GQF_CK(cudaEventRecord(a.ev0, s));
    return GQF_OK;
}

__global__ void k_latch(uint32_t *latch, const uint32_t *err)
{
    if (*err) atomicOr(latch, *err);
}

__global__ void k_report(const uint32_t *err, const uint32_t *extra, uint32_t *host)
{
    host[0] = *err;
    host[1] = extra ? *extra : 0u;
    __threadfence_system();
}

int call_report(Arena &a, cudaStream_t s, const uint32_t *extra, uint32_t out[2])
{
    k_report<<<1, 1, 0, s>>>(a.err, extra, a.report_dev);
    count_launches(1);
    GQF_CK(cudaGetLastError());
    GQF_CK(cudaEventRecord(a.ev1, s));
    GQF_CK(cudaEventSynchronize(a.ev1));
    out[0] = a.report[0];
    out[1] = a.report[1];
    return GQF_OK;
}

int call_end(Arena &a, cudaStream_t s, float *ms)
{
    GQF_CK(cudaGetLastError());
    if (!ms) {
        k_latch<<<1, 1, 0, s>>>(a.latch, a.err);
        count_launches(1);
        GQF_CK(cudaGetLastError());
        return GQF_OK;
    }
    uint32_t rep[2];
    int st = call_report(a, s, nullptr, rep);
    if (st) return st;
    GQF_CK(cudaEventElapsedTime(ms, a.ev0, a.ev1));
    return dev_err_to_status(rep[0]);
}

}  // namespace gqf

using namespace gqf;

extern "C" {

const char *gqf_status_string(int st)
{
    switch (st) {
    case GQF_OK: return "ok";
    case GQF_ERR_ARG: return "invalid argument";
    case GQF_ERR_FULL: return "filter full: layout exceeds (1<<q)*1.1 slots";
    case GQF_ERR_CUDA: return g_last_error[0] ? g_last_error : "CUDA error";
    case GQF_ERR_TIMEOUT: return "device wait timed out";
    case GQF_ERR_NOMEM: return "workspace allocation failed";
    case GQF_ERR_MISMATCH: return "filters differ in q or r";
    case GQF_ERR_LIMIT: return "request exceeds the no-allocation entry point's fixed scratch (see GQF_NOALLOC_MAX_KEYS, GQF_NOALLOC_MAX_Q)";
    case GQF_ERR_FORMAT: return "filter image: bad magic, version, geometry, size or checksum";
    case GQF_ERR_IO: return "filter image file could not be opened, read or written";
    default: return "unknown status";
    }
}

int gqf_stream_status(void *stream)
{
    int dev = current_device();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Arena &a = arena(dev, s);
    std::lock_guard<std::mutex> lk(a.mu);
    if (!arena_reserve(a, 0)) return GQF_ERR_NOMEM;
    GQF_CK(cudaStreamSynchronize(s));
    uint32_t e = 0;
    GQF_CK(cudaMemcpy(&e, a.latch, sizeof(e), cudaMemcpyDeviceToHost));
    GQF_CK(cudaMemset(a.latch, 0, sizeof(uint32_t)));
    return dev_err_to_status(e);
}

unsigned long long gqf_kernel_launches(void) { return g_launches.load(); }

int gqf_workspace_reserve(void *stream, size_t bytes, size_t *reserved)
{
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Arena &a = arena(current_device(), s);
    std::lock_guard<std::mutex> lk(a.mu);
    if (!arena_reserve(a, bytes)) return GQF_ERR_NOMEM;
    if (reserved) *reserved = a.size;
    return GQF_OK;
}

int gqf_workspace_release(void *stream) { return release_arena(current_device(), static_cast<cudaStream_t>(stream)); }

unsigned int gqf_aphash(unsigned int value, unsigned int table_size)
{
    return aphash32(value) % table_size;
}

// MT19937 of Matsumoto & Nishimura (published algorithm), the generator
// the reference drivers seed with init_genrand (mt19937ar.cpp:57,102).
void gqf_mt19937_fill(uint32_t seed, uint64_t skip, uint32_t *out, uint64_t n)
{
    uint32_t mt[624];
    mt[0] = seed;
    for (int i = 1; i < 624; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
    int idx = 624;
    auto next = [&]() -> uint32_t {
        if (idx >= 624) {
            for (int k = 0; k < 624; k++) {
                uint32_t y = (mt[k] & 0x80000000u) | (mt[(k + 1) % 624] & 0x7fffffffu);
                mt[k] = mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
            }
            idx = 0;
        }
        uint32_t y = mt[idx++];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        return y;
    };
    for (uint64_t i = 0; i < skip; i++) (void)next();
    for (uint64_t i = 0; i < n; i++) out[i] = next();
}

}  // extern "C"
