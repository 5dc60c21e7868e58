// Table -> sorted fingerprint list (the input side of insert, delete,
// insertViaMerge and mergeTwoFilters).
//
// The reference recovers each slot's fingerprint one thread per slot by
// walking back to its cluster start and forward counting runs
// (extractQuotients, quotientFilter.cu:1561-1600), then compacts with
// thrust::remove_if (:1627).  Here the recovery uses one global fact of a
// valid table: runs are stored in quotient order, one per occupied quotient,
// so the j-th run start (non-empty, not continuation) in slot order belongs
// to the j-th occupied slot.  Two passes over the table with tile-level
// prefix counts give, for every stored element, its run index and its
// output position; the fingerprint is (quotient of run j) << r | remainder.
// Canonical tables list their fingerprints in ascending order.
#pragma once

#include "qf_device.cuh"

namespace gqf {

constexpr int EXTRACT_THREADS = 256;
constexpr int EXTRACT_WPT = 4;  // 8-slot words per thread
constexpr uint32_t EXTRACT_TILE = EXTRACT_THREADS * EXTRACT_WPT * 8;  // slots per tile

struct Counts3 {
    uint32_t ne, rs, occ;  // non-empty, run starts, occupied
};

// Element values of 8 consecutive slots starting at slot s0 (zero past the
// logical end).  One 8-byte load per 8 one-byte slots; two for 2-byte slots.
template <int BPE>
__device__ __forceinline__ void load8_elems(const uint8_t *t, uint32_t nslots, uint32_t nbytes, uint32_t s0,
                                            uint32_t e[8])
{
    if (BPE == 1 && s0 + 8 <= nslots) {
        uint64_t x = __ldg(reinterpret_cast<const unsigned long long *>(t + s0));
#pragma unroll
        for (int k = 0; k < 8; k++) e[k] = (uint32_t)(x >> (8 * k)) & 0xFFu;
        return;
    }
    if (BPE == 2 && s0 + 8 <= nslots && (size_t)(s0 + 8) * 2 <= nbytes) {
        const unsigned long long *p = reinterpret_cast<const unsigned long long *>(t + (size_t)s0 * 2);
        uint64_t x0 = __ldg(p), x1 = __ldg(p + 1);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            e[k] = (((uint32_t)(x0 >> (16 * k)) & 0xFFu) << 8) | ((uint32_t)(x0 >> (16 * k + 8)) & 0xFFu);
            e[k + 4] = (((uint32_t)(x1 >> (16 * k)) & 0xFFu) << 8) | ((uint32_t)(x1 >> (16 * k + 8)) & 0xFFu);
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t sl = s0 + k;
        uint32_t v = 0;
        if (sl < nslots) {
            const uint8_t *p = t + (size_t)sl * BPE;
            v = p[0];
            if (BPE == 2) v = (v << 8) | p[1];
        }
        e[k] = v;
    }
}

__device__ __forceinline__ void masks_of(const uint32_t e[8], uint32_t &ne, uint32_t &rs, uint32_t &occ)
{
    ne = rs = occ = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        bool nonempty = (e[k] & 7u) != 0;
        ne |= (nonempty ? 1u : 0u) << k;
        rs |= ((nonempty && !(e[k] & 2u)) ? 1u : 0u) << k;
        occ |= ((e[k] >> 2) & 1u) << k;
    }
}

// A thread's EXTRACT_WPT words: element values and per-word masks.
template <int BPE>
struct ThreadSlots {
    uint32_t e[EXTRACT_WPT][8];
    uint32_t ne[EXTRACT_WPT], rs[EXTRACT_WPT], occ[EXTRACT_WPT];
    uint32_t s0;
    __device__ __forceinline__ void load(const uint8_t *t, uint32_t nslots, uint32_t nbytes)
    {
        s0 = blockIdx.x * EXTRACT_TILE + threadIdx.x * (EXTRACT_WPT * 8);
#pragma unroll
        for (int w = 0; w < EXTRACT_WPT; w++) load8_elems<BPE>(t, nslots, nbytes, s0 + 8 * w, e[w]);
#pragma unroll
        for (int w = 0; w < EXTRACT_WPT; w++) masks_of(e[w], ne[w], rs[w], occ[w]);
    }
    __device__ __forceinline__ Counts3 totals() const
    {
        Counts3 c{0, 0, 0};
#pragma unroll
        for (int w = 0; w < EXTRACT_WPT; w++) {
            c.ne += __popc(ne[w]);
            c.rs += __popc(rs[w]);
            c.occ += __popc(occ[w]);
        }
        return c;
    }
};

// Pass 1: per-tile counts.
// When `dups` is non-null it is set to 1 if the table stores a fingerprint
// twice: a continuation element whose remainder equals its predecessor's.
template <int BPE>
__global__ void __launch_bounds__(EXTRACT_THREADS) k_tile_counts(const uint8_t *__restrict__ t, uint32_t nslots,
                                                                uint32_t nbytes, Counts3 *__restrict__ tiles,
                                                                uint32_t *__restrict__ dups,
                                                                const uint32_t *__restrict__ gate = nullptr)
{
    if (gate && !*gate) return;
    ThreadSlots<BPE> ts;
    ts.load(t, nslots, nbytes);
    if (dups) {
        uint32_t prev = 0;
        if (ts.s0 > 0 && ts.s0 - 1 < nslots) {
            const uint8_t *p = t + (size_t)(ts.s0 - 1) * BPE;
            prev = p[0];
            if (BPE == 2) prev = (prev << 8) | p[1];
        }
        bool d = false;
#pragma unroll
        for (int w = 0; w < EXTRACT_WPT; w++)
#pragma unroll
            for (int k = 0; k < 8; k++) {
                uint32_t e = ts.e[w][k];
                d |= (e & 2u) && (e >> 3) == (prev >> 3);
                prev = e;
            }
        if (__any_sync(0xffffffffu, d) && (threadIdx.x & 31) == 0) atomicOr(dups, 1u);
    }
    Counts3 c = ts.totals();
    uint32_t a = c.ne, b = c.rs, d = c.occ;
    for (int o = 16; o; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        d += __shfl_xor_sync(0xffffffffu, d, o);
    }
    __shared__ uint32_t sw[3][EXTRACT_THREADS / 32];
    if ((threadIdx.x & 31) == 0) {
        sw[0][threadIdx.x >> 5] = a;
        sw[1][threadIdx.x >> 5] = b;
        sw[2][threadIdx.x >> 5] = d;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        Counts3 r{0, 0, 0};
        for (int w = 0; w < EXTRACT_THREADS / 32; w++) {
            r.ne += sw[0][w];
            r.rs += sw[1][w];
            r.occ += sw[2][w];
        }
        tiles[blockIdx.x] = r;
    }
}

// Exclusive scan of the tile counts by one CTA; total written at
// tiles[ntiles].  Each thread loads its run of tiles with independent loads.
__global__ void __launch_bounds__(1024) k_scan_counts3(Counts3 *tiles, uint32_t ntiles,
                                                       const uint32_t *__restrict__ gate = nullptr)
{
    if (gate && !*gate) return;
    __shared__ uint32_t sw[3][32];
    const uint32_t per = (ntiles + 1023) / 1024;
    const uint32_t beg = min(ntiles, threadIdx.x * per), end = min(ntiles, beg + per);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    Counts3 sum{0, 0, 0};
    for (uint32_t i = beg; i < end; i++) {
        Counts3 c = tiles[i];
        sum.ne += c.ne;
        sum.rs += c.rs;
        sum.occ += c.occ;
    }
    uint32_t a = sum.ne, b = sum.rs, d = sum.occ;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t x = __shfl_up_sync(0xffffffffu, a, o), y = __shfl_up_sync(0xffffffffu, b, o),
                 z = __shfl_up_sync(0xffffffffu, d, o);
        if (lane >= o) {
            a += x;
            b += y;
            d += z;
        }
    }
    if (lane == 31) {
        sw[0][wid] = a;
        sw[1][wid] = b;
        sw[2][wid] = d;
    }
    __syncthreads();
    if (wid == 0) {
        uint32_t x = sw[0][lane], y = sw[1][lane], z = sw[2][lane];
        uint32_t ix = x, iy = y, iz = z;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t p = __shfl_up_sync(0xffffffffu, ix, o), q = __shfl_up_sync(0xffffffffu, iy, o),
                     r = __shfl_up_sync(0xffffffffu, iz, o);
            if (lane >= o) {
                ix += p;
                iy += q;
                iz += r;
            }
        }
        sw[0][lane] = ix - x;
        sw[1][lane] = iy - y;
        sw[2][lane] = iz - z;
        if (lane == 31) tiles[ntiles] = Counts3{ix, iy, iz};
    }
    __syncthreads();
    Counts3 run{sw[0][wid] + a - sum.ne, sw[1][wid] + b - sum.rs, sw[2][wid] + d - sum.occ};
    for (uint32_t i = beg; i < end; i++) {
        Counts3 c = tiles[i];
        tiles[i] = run;
        run.ne += c.ne;
        run.rs += c.rs;
        run.occ += c.occ;
    }
}

// Block-exclusive prefix of three per-thread counts.
__device__ __forceinline__ Counts3 block_excl3(Counts3 c)
{
    __shared__ uint32_t sw[3][EXTRACT_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t ia = c.ne, ib = c.rs, ic = c.occ;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t va = __shfl_up_sync(0xffffffffu, ia, o);
        uint32_t vb = __shfl_up_sync(0xffffffffu, ib, o);
        uint32_t vc = __shfl_up_sync(0xffffffffu, ic, o);
        if (lane >= o) {
            ia += va;
            ib += vb;
            ic += vc;
        }
    }
    if (lane == 31) {
        sw[0][wid] = ia;
        sw[1][wid] = ib;
        sw[2][wid] = ic;
    }
    __syncthreads();
    Counts3 r{ia - c.ne, ib - c.rs, ic - c.occ};
    for (int w = 0; w < wid; w++) {
        r.ne += sw[0][w];
        r.rs += sw[1][w];
        r.occ += sw[2][w];
    }
    __syncthreads();
    return r;
}

// Copies a tile's outputs, staged in shared memory in output order, to
// out[base .. base + cnt) with coalesced stores.
__device__ __forceinline__ void flush_tile(const uint32_t *s_out, uint32_t cnt, uint32_t *__restrict__ out,
                                           uint32_t base)
{
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < cnt; i += EXTRACT_THREADS) out[base + i] = s_out[i];
}

// Pass 2: positions of occupied slots, in slot order (Q[j] = quotient of
// the j-th run).  A tile's entries are staged in shared memory and stored
// coalesced.
template <int BPE>
__global__ void __launch_bounds__(EXTRACT_THREADS) k_occ_list(const uint8_t *__restrict__ t, uint32_t nslots,
                                                             uint32_t nbytes, const Counts3 *__restrict__ tiles,
                                                             uint32_t *__restrict__ Q,
                                                             const uint32_t *__restrict__ gate = nullptr)
{
    if (gate && !*gate) return;
    __shared__ uint32_t s_out[EXTRACT_TILE];
    ThreadSlots<BPE> ts;
    ts.load(t, nslots, nbytes);
    const Counts3 ex = block_excl3(ts.totals());
    uint32_t o = ex.occ;
#pragma unroll
    for (int w = 0; w < EXTRACT_WPT; w++) {
        uint32_t m = ts.occ[w];
        while (m) {
            const int k = __ffs(m) - 1;
            m &= m - 1;
            s_out[o++] = ts.s0 + 8 * w + k;
        }
    }
    const uint32_t base = tiles[blockIdx.x].occ;
    flush_tile(s_out, tiles[blockIdx.x + 1].occ - base, Q, base);
}

// Pass 3: E[i] = fingerprint of the i-th stored element (staged per tile,
// stored coalesced).
template <int BPE>
__global__ void __launch_bounds__(EXTRACT_THREADS) k_extract(const uint8_t *__restrict__ t, uint32_t nslots,
                                                            uint32_t nbytes, uint32_t r,
                                                            const Counts3 *__restrict__ tiles,
                                                            const uint32_t *__restrict__ Q, uint32_t *__restrict__ E,
                                                            const uint32_t *__restrict__ gate = nullptr)
{
    if (gate && !*gate) return;
    __shared__ uint32_t s_out[EXTRACT_TILE];
    ThreadSlots<BPE> ts;
    ts.load(t, nslots, nbytes);
    const Counts3 ex = block_excl3(ts.totals());
    uint32_t o = ex.ne;
    uint32_t runs_before = tiles[blockIdx.x].rs + ex.rs;  // run starts strictly before this thread's slots
#pragma unroll
    for (int w = 0; w < EXTRACT_WPT; w++) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            if (!((ts.ne[w] >> k) & 1u)) continue;
            const uint32_t rs_upto = runs_before + __popc(ts.rs[w] & ((2u << k) - 1u));
            // rs_upto >= 1 in a valid table (the first element of a cluster starts a run)
            const uint32_t j = rs_upto ? rs_upto - 1 : 0;
            s_out[o++] = (Q[j] << r) | (ts.e[w][k] >> 3);
        }
        runs_before += __popc(ts.rs[w]);
    }
    const uint32_t base = tiles[blockIdx.x].ne;
    flush_tile(s_out, tiles[blockIdx.x + 1].ne - base, E, base);
}

// Bucket bounds of a sorted fingerprint list: base[b] = lower_bound(b << shift).
__global__ void k_sorted_bounds(const uint32_t *__restrict__ E, const uint32_t *__restrict__ m_ptr, uint32_t nb,
                                uint32_t shift, uint32_t *__restrict__ base, uint32_t *__restrict__ cnt,
                                const uint32_t *__restrict__ gate = nullptr)
{
    if (gate && !*gate) return;
    const uint32_t m = *m_ptr;
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b <= nb; b += gridDim.x * blockDim.x) {
        uint64_t key = (uint64_t)b << shift;
        uint32_t lo = 0, hi = m;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if ((uint64_t)E[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        base[b] = lo;
    }
}
__global__ void k_bounds_to_counts(const uint32_t *__restrict__ base, uint32_t nb, uint32_t *__restrict__ cnt,
                                   const uint32_t *__restrict__ gate = nullptr)
{
    if (gate && !*gate) return;
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
        cnt[b] = base[b + 1] - base[b];
}

}  // namespace gqf
