// Batched filters: the work lists shared by the pipeline kernels (batch.cu)
// and the persistent pipeline (batch_persist.cu).
#pragma once

#include <cstdint>

#include "sqf_build.cuh"
#include "sqf_lookup.cuh"

namespace gqf {

struct MfFilter {
    uint8_t *table;
    const uint32_t *keys;     // bulk build input (n_keys; 0 = no build)
    const uint32_t *queries;  // lookups (n_q)
    uint32_t *results;
    uint32_t q, r, nslots, T;
    uint32_t n_keys, n_q;
    uint32_t chunk0, bucket0, qchunk0, fix0;  // first work unit of each list
    uint32_t pchunk0;                         // first scatter chunk of the persistent kernel
    uint32_t nb, fix_cap;
};

struct MfParams {
    const MfFilter *f;
    uint32_t nf;
    uint32_t tb, cap_items;
    int nodup, bitmap_ok;
    uint32_t *bcnt, *bbase, *bfill;  // per global bucket
    uint32_t *items;                 // bucketed fingerprints of all filters
    unsigned long long *status;      // look-back descriptors, per global bucket
    uint32_t *ticket;
    uint32_t *fix_list, *fix_cnt;    // per-filter regions / counters
    uint32_t *err;
    uint32_t total_buckets;
};

// filter owning work unit x of a list whose per-filter starts are field F
template <uint32_t MfFilter::*F>
__device__ __forceinline__ uint32_t mf_owner(const MfFilter *f, uint32_t nf, uint32_t x)
{
    uint32_t lo = 0, hi = nf;  // last filter with start <= x
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (f[mid].*F <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ BucketGeom mf_geom(const MfFilter &f, uint32_t tb)
{
    BucketGeom g;
    g.q = f.q;
    g.r = f.r;
    g.tb = tb;
    g.nb = f.nb;
    g.shift = f.r + tb;
    g.fp_mask = (f.q + f.r >= 32) ? 0xFFFFFFFFu : ((1u << (f.q + f.r)) - 1u);
    return g;
}

// Occupied bits of filter f after its layout: from the fix-up list, or, when
// the list overflowed (a nearly full filter whose buckets mostly start in
// their predecessor's spill), from all of the filter's bucketed items (one
// atomic OR of bit 2 into each item's home slot).  The CTA strides over the
// work with THREADS threads; run after every layout of the filter is done.
template <int BPE>
__device__ __forceinline__ void mf_occupied_bits(const MfParams &p, const MfFilter &f, uint32_t fi, uint32_t tid,
                                                 uint32_t nthreads)
{
    const uint32_t nfix = p.fix_cnt[fi];
    if (nfix <= f.fix_cap) {
        for (uint32_t i = tid; i < nfix; i += nthreads) f.table[(size_t)p.fix_list[f.fix0 + i] * BPE + (BPE - 1)] |= 4u;
        return;
    }
    const uint32_t bl = f.bucket0 + f.nb - 1;
    const uint32_t i0 = p.bbase[f.bucket0], i1 = p.bbase[bl] + p.bcnt[bl];
    uint32_t *words = reinterpret_cast<uint32_t *>(f.table);  // 16-byte-aligned table
    for (uint32_t i = i0 + tid; i < i1; i += nthreads) {
        const size_t byte = (size_t)(p.items[i] >> f.r) * BPE + (BPE - 1);
        atomicOr(words + (byte >> 2), 4u << (8 * (byte & 3)));
    }
}

// Lookup work unit: MF_QCHUNK queries of one filter.
constexpr uint32_t MF_QCHUNK = LOOKUP_THREADS * LOOKUP_QPT;

// Persistent pipeline lists and its grid barrier words.
struct MfPersist {
    uint32_t total_chunks;   // scatter chunks of THREADS * IPT keys
    uint32_t total_buckets, total_qchunks;
    int any_build, any_lookup;
    uint32_t *bar;           // [0] arrivals, [1] generation, [2] abort (zeroed before each run)
};

// The compiled persistent kernel for (bytes per slot, CTA threads, keys per
// thread per scatter chunk, quotients per layout thread), or nullptr.
const void *mf_persistent_kernel(int bpe, int threads, int ipt, int qpt);

}  // namespace gqf
