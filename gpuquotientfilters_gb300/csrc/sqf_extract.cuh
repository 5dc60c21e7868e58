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
constexpr uint32_t EXTRACT_TILE = EXTRACT_THREADS * 8;  // slots per tile

struct Counts3 {
    uint32_t ne, rs, occ;  // non-empty, run starts, occupied
};

template <int BPE>
__device__ __forceinline__ void load8_elems(const uint8_t *t, uint32_t nslots, uint32_t s0, uint32_t e[8])
{
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t s = s0 + k;
        uint32_t v = 0;
        if (s < nslots) {
            const uint8_t *p = t + (size_t)s * BPE;
            v = p[0];
            if (BPE == 2) v = (v << 8) | p[1];
        }
        e[k] = v;
    }
}

template <int BPE>
__device__ __forceinline__ void masks8(const uint8_t *t, uint32_t nslots, uint32_t s0, uint32_t &ne, uint32_t &rs,
                                       uint32_t &occ, uint32_t e[8])
{
    load8_elems<BPE>(t, nslots, s0, e);
    ne = rs = occ = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        bool nonempty = (e[k] & 7u) != 0;
        ne |= (nonempty ? 1u : 0u) << k;
        rs |= ((nonempty && !(e[k] & 2u)) ? 1u : 0u) << k;
        occ |= ((e[k] >> 2) & 1u) << k;
    }
}

// Pass 1: per-tile counts.
template <int BPE>
__global__ void __launch_bounds__(EXTRACT_THREADS) k_tile_counts(const uint8_t *__restrict__ t, uint32_t nslots,
                                                                Counts3 *__restrict__ tiles)
{
    const uint32_t s0 = blockIdx.x * EXTRACT_TILE + threadIdx.x * 8;
    uint32_t ne, rs, occ, e[8];
    masks8<BPE>(t, nslots, s0, ne, rs, occ, e);
    uint32_t a = __popc(ne), b = __popc(rs), c = __popc(occ);
    for (int o = 16; o; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    __shared__ uint32_t sw[3][EXTRACT_THREADS / 32];
    if ((threadIdx.x & 31) == 0) {
        sw[0][threadIdx.x >> 5] = a;
        sw[1][threadIdx.x >> 5] = b;
        sw[2][threadIdx.x >> 5] = c;
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

// Exclusive scan of the tile counts by one CTA (tiles <= a few 1e5);
// total written at tiles[ntiles].
__global__ void __launch_bounds__(1024) k_scan_counts3(Counts3 *tiles, uint32_t ntiles)
{
    __shared__ Counts3 s_part[1024];
    const uint32_t per = (ntiles + 1023) / 1024;
    const uint32_t beg = min(ntiles, threadIdx.x * per), end = min(ntiles, beg + per);
    Counts3 sum{0, 0, 0};
    for (uint32_t i = beg; i < end; i++) {
        sum.ne += tiles[i].ne;
        sum.rs += tiles[i].rs;
        sum.occ += tiles[i].occ;
    }
    s_part[threadIdx.x] = sum;
    __syncthreads();
    // Hillis-Steele over 1024 partials
    for (int o = 1; o < 1024; o <<= 1) {
        Counts3 v{0, 0, 0};
        if (threadIdx.x >= (unsigned)o) v = s_part[threadIdx.x - o];
        __syncthreads();
        s_part[threadIdx.x].ne += v.ne;
        s_part[threadIdx.x].rs += v.rs;
        s_part[threadIdx.x].occ += v.occ;
        __syncthreads();
    }
    Counts3 run{0, 0, 0};
    if (threadIdx.x) run = s_part[threadIdx.x - 1];
    for (uint32_t i = beg; i < end; i++) {
        Counts3 c = tiles[i];
        tiles[i] = run;
        run.ne += c.ne;
        run.rs += c.rs;
        run.occ += c.occ;
    }
    if (threadIdx.x == 1023) tiles[ntiles] = s_part[1023];
}

// Block-exclusive prefix of three per-thread counts.
__device__ __forceinline__ Counts3 block_excl3(uint32_t a, uint32_t b, uint32_t c)
{
    __shared__ uint32_t sw[3][EXTRACT_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t ia = a, ib = b, ic = c;
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
    Counts3 r{ia - a, ib - b, ic - c};
    for (int w = 0; w < wid; w++) {
        r.ne += sw[0][w];
        r.rs += sw[1][w];
        r.occ += sw[2][w];
    }
    __syncthreads();
    return r;
}

// Pass 2: positions of occupied slots, in slot order (Q[j] = quotient of
// the j-th run).
template <int BPE>
__global__ void __launch_bounds__(EXTRACT_THREADS) k_occ_list(const uint8_t *__restrict__ t, uint32_t nslots,
                                                             const Counts3 *__restrict__ tiles, uint32_t *__restrict__ Q)
{
    const uint32_t s0 = blockIdx.x * EXTRACT_TILE + threadIdx.x * 8;
    uint32_t ne, rs, occ, e[8];
    masks8<BPE>(t, nslots, s0, ne, rs, occ, e);
    Counts3 ex = block_excl3(__popc(ne), __popc(rs), __popc(occ));
    uint32_t o = tiles[blockIdx.x].occ + ex.occ;
    while (occ) {
        int k = __ffs(occ) - 1;
        occ &= occ - 1;
        Q[o++] = s0 + k;
    }
}

// Pass 3: E[i] = fingerprint of the i-th stored element.
template <int BPE>
__global__ void __launch_bounds__(EXTRACT_THREADS) k_extract(const uint8_t *__restrict__ t, uint32_t nslots, uint32_t r,
                                                            const Counts3 *__restrict__ tiles,
                                                            const uint32_t *__restrict__ Q, uint32_t *__restrict__ E)
{
    const uint32_t s0 = blockIdx.x * EXTRACT_TILE + threadIdx.x * 8;
    uint32_t ne, rs, occ, e[8];
    masks8<BPE>(t, nslots, s0, ne, rs, occ, e);
    Counts3 ex = block_excl3(__popc(ne), __popc(rs), __popc(occ));
    uint32_t o = tiles[blockIdx.x].ne + ex.ne;
    uint32_t runs_before = tiles[blockIdx.x].rs + ex.rs;  // run starts strictly before s0
#pragma unroll
    for (int k = 0; k < 8; k++) {
        if (!((ne >> k) & 1u)) continue;
        uint32_t rs_upto = runs_before + __popc(rs & ((2u << k) - 1u));
        // rs_upto >= 1 in a valid table (slot 0 of a cluster starts a run)
        uint32_t j = rs_upto ? rs_upto - 1 : 0;
        E[o++] = (Q[j] << r) | (e[k] >> 3);
    }
}

// Bucket bounds of a sorted fingerprint list: base[b] = lower_bound(b << shift).
__global__ void k_sorted_bounds(const uint32_t *__restrict__ E, const uint32_t *__restrict__ m_ptr, uint32_t nb,
                                uint32_t shift, uint32_t *__restrict__ base, uint32_t *__restrict__ cnt)
{
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
__global__ void k_bounds_to_counts(const uint32_t *__restrict__ base, uint32_t nb, uint32_t *__restrict__ cnt)
{
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
        cnt[b] = base[b + 1] - base[b];
}

}  // namespace gqf
