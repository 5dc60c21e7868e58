// Device-side building blocks shared by the SQF and RSQF kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gqf.h"

#define QF_HD __host__ __device__ __forceinline__

namespace gqf {

// Device error word bits (latched per stream by the host layer).
enum : uint32_t {
    DEV_ERR_FULL = 1u,          // a layout ran past (1<<q)*1.1 slots
    DEV_ERR_TIMEOUT = 2u,       // a bounded spin-wait gave up
    DEV_ERR_BUCKET_OVER = 4u,   // speculative bucket capacity exceeded (host retries)
    DEV_ERR_BUCKET_CAP = 8u,    // a bucket is larger than one CTA can sort (host falls back)
};

// Normal_APHash without the final modulo (quotientFilter.cu:134-149):
// four byte rounds, most significant byte first.  Callers mask to q+r bits,
// which equals `% (1 << (q+r))`.
QF_HD uint32_t aphash32(uint32_t v)
{
    uint32_t h = 0xAAAAAAAAu;
    h ^= (h << 7) ^ (v >> 24) ^ (h >> 3);
    h ^= ~((h << 11) ^ ((v >> 16) & 0xFFu) ^ (h >> 5));
    h ^= (h << 7) ^ ((v >> 8) & 0xFFu) ^ (h >> 3);
    h ^= ~((h << 11) ^ (v & 0xFFu) ^ (h >> 5));
    return h;
}

// Slot element: rem << 3 | occupied << 2 | continuation << 1 | shifted
// (quotientFilter.cu:57-115).
QF_HD bool e_occ(uint32_t e) { return (e >> 2) & 1u; }
QF_HD bool e_cont(uint32_t e) { return (e >> 1) & 1u; }
QF_HD bool e_shift(uint32_t e) { return e & 1u; }
QF_HD bool e_empty(uint32_t e) { return (e & 7u) == 0; }

// ---- SWAR over 8 one-byte slots held in a little-endian u64 ----------
// bit k of the result = bit 0 of byte k
QF_HD uint32_t pack8(uint64_t x)
{
    x &= 0x0101010101010101ull;
    return (uint32_t)((x * 0x0102040810204080ull) >> 56);
}
struct Flags8 {
    uint32_t occ, cont, shift, nonempty;
};
QF_HD Flags8 flags8(uint64_t x)
{
    Flags8 f;
    f.occ = pack8(x >> 2);
    f.cont = pack8(x >> 1);
    f.shift = pack8(x);
    f.nonempty = pack8(x | (x >> 1) | (x >> 2));
    return f;
}

QF_HD int popc32(uint32_t x)
{
#ifdef __CUDA_ARCH__
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}
QF_HD int highest_bit(uint32_t x)  // x != 0
{
#ifdef __CUDA_ARCH__
    return 31 - __clz(x);
#else
    return 31 - __builtin_clz(x);
#endif
}
QF_HD int lowest_bit(uint32_t x)  // x != 0
{
#ifdef __CUDA_ARCH__
    return __ffs(x) - 1;
#else
    return __builtin_ctz(x);
#endif
}
// position of the j-th (0-based) set bit of m; m has more than j set bits
QF_HD int select_bit(uint32_t m, int j)
{
    for (int i = 0; i < j; i++) m &= m - 1;
    return lowest_bit(m);
}

// ---- byte-lane SWAR: one flag bit per byte of a u64 (slot k = byte k) ---
constexpr uint64_t BL_LO = 0x0101010101010101ull;  // bit 0 of every byte
constexpr uint64_t BL_HI = 0x8080808080808080ull;  // bit 7 of every byte
// bytes [0, n) set; n in [0, 8]
QF_HD uint64_t bytes_below(uint32_t n) { return n >= 8 ? ~0ull : ((1ull << (8 * n)) - 1ull); }
QF_HD int popc64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}
QF_HD uint32_t lowest_byte(uint64_t x)  // x != 0
{
#ifdef __CUDA_ARCH__
    return (uint32_t)(__ffsll((long long)x) - 1) >> 3;
#else
    return (uint32_t)__builtin_ctzll(x) >> 3;
#endif
}
QF_HD uint32_t highest_byte(uint64_t x)  // x != 0
{
#ifdef __CUDA_ARCH__
    return (uint32_t)(63 - __clzll((long long)x)) >> 3;
#else
    return (uint32_t)(63 - __builtin_clzll(x)) >> 3;
#endif
}
// per-slot flags of 8 one-byte slots, bit 0 of each byte
QF_HD uint64_t bl_unshifted(uint64_t x) { return ~x & BL_LO; }
// run starts: non-empty (metadata != 0) and not a continuation
QF_HD uint64_t bl_run_starts(uint64_t x) { return (x | (x >> 2)) & ~(x >> 1) & BL_LO; }

// ---- descriptor access for the decoupled look-back ----------------------
// A descriptor is one aligned 64-bit word holding both its flag and its
// value, and a reader uses nothing else its writer stored, so relaxed
// gpu-scope accesses suffice (no fence, no L1 invalidation on the reader).
#ifdef __CUDACC__
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
#endif

#ifdef __CUDACC__
// Runs of quotients below slot x0 still pending at x0 -- the lookup's walk
// back to the cluster start, for slot x0 -- by one warp: each round the 32
// lanes read the 32 words in front of the last ones, a ballot finds the
// nearest word holding an unshifted slot, and a warp sum adds #occupied -
// #run starts from that slot up to x0.  Words before the table read as
// empty, which ends the walk.  x0 is a multiple of 8; every lane returns D.
__device__ inline int pending_runs_warp(const uint8_t *table, uint32_t x0)
{
    const int lane = threadIdx.x & 31;
    if (x0 == 0 || !(__ldg(table + x0) & 1u)) return 0;
    constexpr uint64_t OCC = 0x0404040404040404ull;
    const unsigned long long *t64 = reinterpret_cast<const unsigned long long *>(table);
    int D = 0;
    for (int wend = (int)(x0 >> 3);; wend -= 32) {
        const int ww = wend - 1 - lane;
        const uint64_t y = ww >= 0 ? __ldg(t64 + ww) : 0ull;
        const uint64_t st = bl_unshifted(y);
        const unsigned stops = __ballot_sync(0xffffffffu, st != 0);
        const int nearest = stops ? __ffs(stops) - 1 : 32;
        uint64_t R = 0;
        if (lane < nearest) R = ~0ull;
        else if (lane == nearest) R = ~bytes_below(highest_byte(st));
        D += (int)__reduce_add_sync(0xffffffffu, (unsigned)(popc64(y & OCC & R) - popc64(bl_run_starts(y) & R)));
        if (stops) return D;
    }
}
#endif

// Look-back descriptor (64 bits): [63:62] flag, payload below.
//   AGG: [61:31] n (items), [30:0] F (end slot when entering at slot 0)
//   INC: [30:0] c_out (first slot after this bucket's items)
// A bucket's layout maps an entry slot c to max(c + n, F); composing two
// buckets (a then b) gives (n_a + n_b, max(F_a + n_b, F_b)).
constexpr unsigned long long LB_AGG = 1ull << 62;
constexpr unsigned long long LB_INC = 2ull << 62;
constexpr uint32_t LB_VMAX = 0x7FFFFFFFu;
QF_HD unsigned long long lb_pack_agg(uint32_t n, uint32_t F)
{
    return LB_AGG | ((unsigned long long)(n & LB_VMAX) << 31) | (F & LB_VMAX);
}
QF_HD unsigned long long lb_pack_inc(uint32_t c) { return LB_INC | (c & LB_VMAX); }

struct LayoutFn {
    uint32_t n, F;  // c -> max(c + n, F)
    QF_HD uint32_t apply(uint32_t c) const
    {
        uint32_t a = c + n;
        return a > F ? a : F;
    }
};
// first a, then b
QF_HD LayoutFn compose(LayoutFn a, LayoutFn b)
{
    LayoutFn r;
    r.n = a.n + b.n;
    uint32_t x = a.F + b.n;
    r.F = x > b.F ? x : b.F;
    return r;
}

}  // namespace gqf
