// SQF bulk build: hash -> quotient-range buckets -> per-bucket layout.
//
// The reference (quotientFilter.cu:1446-1559) hashes, radix-sorts all
// fingerprints with Thrust, then iterates a host-driven fixpoint over
// 2^q/q segments until no segment overflows (:1516-1530), and finally
// scatters elements and read-modify-writes occupied bits.  Its result is a
// pure function of the sorted fingerprint multiset: item i of the sorted
// order lands at slot pos_i = max(quotient_i, pos_{i-1} + 1).  This build
// computes that layout directly:
//
//   k_hash_bucket   one pass over the keys: Normal_APHash, then a
//                   CTA-local counting sort by bucket (bucket = the top
//                   q - tb quotient bits) and coalesced runs into per-bucket
//                   regions (one global atomic per CTA and bucket).
//   k_bucket_layout one CTA per bucket (2^tb quotients): counting sort by
//                   quotient in shared memory, tiny per-quotient remainder
//                   sorts, then the slot recurrence as a block scan of
//                   c -> max(c + n, F) maps, chained across buckets with a
//                   decoupled look-back; every slot of the bucket's write
//                   range is produced in shared memory and stored once with
//                   16-byte stores (no read-modify-write of the table).
//   k_fixup_occ     occupied bits of quotients whose slot was written by an
//                   earlier bucket (the spill of a cluster that crosses a
//                   bucket boundary).
#pragma once

#include "qf_device.cuh"

namespace gqf {

struct BucketGeom {
    uint32_t q, r, tb, nb;  // S = 1 << tb quotients per bucket, nb = 2^(q - tb)
    uint32_t shift;         // r + tb: bucket index = fp >> shift
    uint32_t fp_mask;       // (1 << (q + r)) - 1
};

// Scatter CTA shapes: fingerprints only (build, insert, delete) take 32K
// keys per CTA, halving the per-(CTA, bucket) global reservations; pairs
// (sorted lookups) carry an index per key and take 16K.
constexpr int SCATTER_THREADS = 1024;
constexpr int SCATTER_IPT = 32;
constexpr int PAIR_THREADS = 512;
constexpr int PAIR_IPT = 32;
constexpr int LAYOUT_THREADS = 512;
constexpr uint32_t SPILL_SLOTS = 4096;  // tile buffer headroom past the bucket
constexpr uint32_t SPIN_LIMIT = 1u << 22;

// Exclusive scan of `cnt` (nvals entries of u32 in shared memory) in place,
// by a block of THREADS threads; returns the total.  Each thread owns a
// contiguous run of ceil(nvals / THREADS) entries.
template <int THREADS>
__device__ uint32_t block_exclusive_scan_u32(uint32_t *cnt, uint32_t nvals, uint32_t *s_warp)
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t per = (nvals + THREADS - 1) / THREADS;
    const uint32_t beg = min(nvals, tid * per), end = min(nvals, beg + per);
    uint32_t sum = 0;
    for (uint32_t i = beg; i < end; i++) sum += cnt[i];
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint32_t v = lane < THREADS / 32 ? s_warp[lane] : 0;
        uint32_t iv = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, iv, o);
            if (lane >= o) iv += t;
        }
        if (lane < THREADS / 32) s_warp[lane] = iv - v;  // exclusive warp offsets
        if (lane == THREADS / 32 - 1) s_warp[32] = iv;   // total
    }
    __syncthreads();
    uint32_t run = s_warp[wid] + incl - sum;
    for (uint32_t i = beg; i < end; i++) {
        uint32_t c = cnt[i];
        cnt[i] = run;
        run += c;
    }
    uint32_t total = s_warp[32];
    __syncthreads();
    return total;
}

// ---------------------------------------------------------------------
// K1: hash + bucket scatter.  out[base(b) + j] holds the j-th fingerprint
// of bucket b (order within a bucket is arbitrary).  base(b) = b * cap in
// speculative mode (bucket_base == nullptr); a bucket that would exceed cap
// sets DEV_ERR_BUCKET_OVER and the host reruns with exact bases.
// Dynamic smem: items[THREADS*IPT] + cursor[nb] + gbase[nb] (u32).
// With `vals` non-null the kernel scatters (fingerprint, index) pairs: the
// pair payload is the key's position in the input (sorted lookups).
// ---------------------------------------------------------------------
template <int THREADS, int IPT, bool PAIRS>
__device__ __forceinline__ void hash_bucket_chunk(
    uint32_t chunk, const uint32_t *__restrict__ keys, uint32_t n, const BucketGeom &g,
    const uint32_t *__restrict__ bucket_base, uint32_t cap,
    uint32_t *__restrict__ bucket_cnt, uint32_t *__restrict__ out,
    uint32_t *__restrict__ out_idx, uint32_t *__restrict__ err)
{
    extern __shared__ __align__(16) uint32_t smem_scatter[];
    constexpr uint32_t CHUNK = THREADS * IPT;
    uint32_t *s_items = smem_scatter;
    uint32_t *s_idx = s_items + CHUNK;  // only when PAIRS
    uint32_t *s_cur = s_items + (PAIRS ? 2 * CHUNK : CHUNK);
    uint32_t *s_gb = s_cur + g.nb;
    __shared__ uint32_t s_warp[33];
    const int tid = threadIdx.x;
    const uint64_t c0 = (uint64_t)chunk * CHUNK;
    const uint32_t cnt = (uint32_t)min((uint64_t)CHUNK, (uint64_t)n - c0);

    for (uint32_t i = tid; i < g.nb; i += THREADS) s_cur[i] = 0;
    __syncthreads();

    // all loads first (IPT keys in flight per thread), then hash + count.
    // A 16-byte aligned key array is read as 16-byte vectors: item k of the
    // thread is key 4 * ((k / 4) * THREADS + tid) + k % 4 of the chunk;
    // otherwise item k is key k * THREADS + tid.
    static_assert(IPT % 4 == 0, "IPT must be a multiple of 4");
    const bool vec = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0;
    auto jof = [&](int k) -> uint32_t {
        return vec ? 4u * ((uint32_t)(k >> 2) * THREADS + tid) + (uint32_t)(k & 3) : (uint32_t)k * THREADS + tid;
    };
    uint32_t fp[IPT];
    if (vec) {
#pragma unroll
        for (int k = 0; k < IPT / 4; k++) {
            const uint32_t j = 4u * ((uint32_t)k * THREADS + tid);
            if (j + 3 < cnt) {
                const uint4 v = __ldg(reinterpret_cast<const uint4 *>(keys + c0 + j));
                fp[4 * k] = v.x;
                fp[4 * k + 1] = v.y;
                fp[4 * k + 2] = v.z;
                fp[4 * k + 3] = v.w;
            } else {
#pragma unroll
                for (int e = 0; e < 4; e++) fp[4 * k + e] = j + e < cnt ? __ldg(keys + c0 + j + e) : 0u;
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const uint32_t j = (uint32_t)k * THREADS + tid;
            fp[k] = j < cnt ? __ldg(keys + c0 + j) : 0u;
        }
    }
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        fp[k] = aphash32(fp[k]) & g.fp_mask;
        if (jof(k) < cnt) atomicAdd(&s_cur[fp[k] >> g.shift], 1u);
    }
    __syncthreads();
    // one global reservation per non-empty bucket; a thread's reservations
    // (buckets tid, tid + THREADS, ...) are issued together so their round
    // trips overlap
    {
        constexpr uint32_t MAXPER = (4096 + THREADS - 1) / THREADS;  // nb <= 4096
        uint32_t c[MAXPER], r[MAXPER];
#pragma unroll
        for (uint32_t k = 0; k < MAXPER; k++) {
            const uint32_t b = tid + k * THREADS;
            c[k] = b < g.nb ? s_cur[b] : 0u;
        }
#pragma unroll
        for (uint32_t k = 0; k < MAXPER; k++) r[k] = c[k] ? atomicAdd(bucket_cnt + tid + k * THREADS, c[k]) : 0u;
#pragma unroll
        for (uint32_t k = 0; k < MAXPER; k++) {
            const uint32_t b = tid + k * THREADS;
            if (b < g.nb) s_gb[b] = r[k];
        }
    }
    block_exclusive_scan_u32<THREADS>(s_cur, g.nb, s_warp);
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        const uint32_t j = jof(k);
        if (j < cnt) {
            uint32_t p = atomicAdd(&s_cur[fp[k] >> g.shift], 1u);
            s_items[p] = fp[k];
            if (PAIRS) s_idx[p] = (uint32_t)(c0 + j);
        }
    }
    __syncthreads();
    // s_cur[b] is now the end of bucket b's run in s_items.  Per bucket:
    // item i of the run goes to out[i + delta(b)], delta(b) = base(b) +
    // reservation(b) - start(b), and overflows the speculative stride from
    // i = start(b) + cap - reservation(b) on (kept in s_cur).
    {
        constexpr uint32_t MAXPER = (4096 + THREADS - 1) / THREADS;
        uint32_t dl[MAXPER], lim[MAXPER];
#pragma unroll
        for (uint32_t k = 0; k < MAXPER; k++) {
            const uint32_t b = tid + k * THREADS;
            if (b < g.nb) {
                const uint32_t start = b ? s_cur[b - 1] : 0u, gb = s_gb[b];
                const size_t base = bucket_base ? (size_t)bucket_base[b] : (size_t)b * cap;
                dl[k] = (uint32_t)(base + gb - start);
                lim[k] = gb >= cap ? start : (cap - gb > 0xFFFFFFFFu - start ? 0xFFFFFFFFu : start + (cap - gb));
            }
        }
        __syncthreads();
        // (delta, limit) of bucket b as one 8-byte word over s_cur/s_gb
#pragma unroll
        for (uint32_t k = 0; k < MAXPER; k++) {
            const uint32_t b = tid + k * THREADS;
            if (b < g.nb) reinterpret_cast<uint2 *>(s_cur)[b] = make_uint2(dl[k], lim[k]);
        }
    }
    __syncthreads();
    for (uint32_t i = tid; i < cnt; i += THREADS) {
        const uint32_t v = s_items[i];
        const uint32_t b = v >> g.shift;
        const uint2 dlim = reinterpret_cast<const uint2 *>(s_cur)[b];
        if (i < dlim.y) {
            const uint32_t dst = i + dlim.x;
            out[dst] = v;
            if (PAIRS) out_idx[dst] = s_idx[i];
        } else {
            atomicOr(err, DEV_ERR_BUCKET_OVER);
        }
    }
}

template <int THREADS, int IPT, bool PAIRS>
__global__ void __launch_bounds__(THREADS) k_hash_bucket(
    const uint32_t *__restrict__ keys, uint32_t n, BucketGeom g,
    const uint32_t *__restrict__ bucket_base, uint32_t cap,
    uint32_t *__restrict__ bucket_cnt, uint32_t *__restrict__ out,
    uint32_t *__restrict__ out_idx, uint32_t *__restrict__ err)
{
    hash_bucket_chunk<THREADS, IPT, PAIRS>(blockIdx.x, keys, n, g, bucket_base, cap, bucket_cnt, out, out_idx, err);
}

// Histogram-only pass for exact bucket bases (used when a speculative
// bucket overflowed).
template <int THREADS, int IPT>
__device__ __forceinline__ void bucket_hist_chunk(uint32_t chunk, const uint32_t *__restrict__ keys, uint32_t n,
                                                  const BucketGeom &g, uint32_t *__restrict__ bucket_cnt)
{
    extern __shared__ __align__(16) uint32_t smem_hist[];
    constexpr uint32_t CHUNK = THREADS * IPT;
    const uint64_t c0 = (uint64_t)chunk * CHUNK;
    const uint32_t cnt = (uint32_t)min((uint64_t)CHUNK, (uint64_t)n - c0);
    for (uint32_t i = threadIdx.x; i < g.nb; i += THREADS) smem_hist[i] = 0;
    __syncthreads();
    uint32_t v[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        uint32_t j = k * THREADS + threadIdx.x;
        v[k] = j < cnt ? __ldg(keys + c0 + j) : 0u;
    }
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        uint32_t j = k * THREADS + threadIdx.x;
        if (j < cnt) atomicAdd(&smem_hist[(aphash32(v[k]) & g.fp_mask) >> g.shift], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < g.nb; b += THREADS)
        if (smem_hist[b]) atomicAdd(bucket_cnt + b, smem_hist[b]);
}

template <int THREADS, int IPT>
__global__ void __launch_bounds__(THREADS) k_bucket_hist(
    const uint32_t *__restrict__ keys, uint32_t n, BucketGeom g, uint32_t *__restrict__ bucket_cnt)
{
    bucket_hist_chunk<THREADS, IPT>(blockIdx.x, keys, n, g, bucket_cnt);
}

// ---------------------------------------------------------------------
// Decoupled look-back over bucket descriptors, one warp.  Each round issues
// the loads of the LB_WINDOWS x 32 nearest unread predecessors at once
// (window m, lane l holds bucket j - 32m - l), so a look-back that has to
// pass a few hundred buckets still costs one memory round trip; windows are
// then folded nearest first: wait until the window is published, fold its
// descriptors far-to-near with an ordered shuffle reduction up to the
// nearest inclusive descriptor.  Returns (on every lane) the slot at which
// bucket b's items start (c_in).  A window holding an unpublished descriptor
// is re-read at most spin_limit times, 32 ns apart; past that the warp sets
// DEV_ERR_TIMEOUT and returns 0, so the kernel ends and the host reports
// GQF_ERR_TIMEOUT.
// ---------------------------------------------------------------------
constexpr int LB_WINDOWS = 4;

__device__ inline uint32_t lookback_cin_warp(unsigned long long *status, uint32_t b, uint32_t *err,
                                             uint32_t spin_limit = SPIN_LIMIT)
{
    const int lane = threadIdx.x & 31;
    LayoutFn acc{0u, 0u};  // functions of the windows already folded (nearer buckets)
    int j = (int)b - 1;
    for (;;) {
        unsigned long long v[LB_WINDOWS];
#pragma unroll
        for (int m = 0; m < LB_WINDOWS; m++) {
            const int idx = j - 32 * m - lane;
            v[m] = idx >= 0 ? ld_relaxed_u64(status + idx) : lb_pack_inc(0u);  // before bucket 0: slot 0
        }
#pragma unroll
        for (int m = 0; m < LB_WINDOWS; m++) {
            const int idx = j - 32 * m - lane;
            unsigned long long vm = v[m];
            uint32_t spins = 0;
            for (;;) {
                unsigned pending = __ballot_sync(0xffffffffu, (vm >> 62) == 0);
                if (!pending) break;
                if (++spins > spin_limit) {
                    if (lane == 0) atomicOr(err, DEV_ERR_TIMEOUT);
                    return 0u;
                }
                __nanosleep(32);
                if (idx >= 0 && (vm >> 62) == 0) vm = ld_relaxed_u64(status + idx);
            }
            unsigned incm = __ballot_sync(0xffffffffu, (vm >> 62) == 2ull);
            const int L = incm ? __ffs(incm) - 1 : 32;  // nearest inclusive lane
            // lane function: aggregate map; the inclusive lane becomes the
            // constant max(c, c_L) (applied to c = 0); lanes past it identity
            LayoutFn f{0u, 0u};
            if (lane < L) f = LayoutFn{(uint32_t)((vm >> 31) & LB_VMAX), (uint32_t)(vm & LB_VMAX)};
            else if (lane == L) f = LayoutFn{0u, (uint32_t)(vm & LB_VMAX)};
            // ordered reduction: farther lanes (higher index) apply first
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                LayoutFn far;
                far.n = __shfl_down_sync(0xffffffffu, f.n, o);
                far.F = __shfl_down_sync(0xffffffffu, f.F, o);
                if (lane + o < 32 && (lane & (2 * o - 1)) == 0) f = compose(far, f);
            }
            f.n = __shfl_sync(0xffffffffu, f.n, 0);
            f.F = __shfl_sync(0xffffffffu, f.F, 0);
            if (incm) return acc.apply(f.apply(0u));
            acc = compose(f, acc);
        }
        j -= 32 * LB_WINDOWS;
    }
}

// Shared-memory word skew: a thread that owns a run of 16 consecutive words
// starts 17 words after its neighbour, so the lanes of a warp stepping
// through their runs hit distinct banks.
__device__ __forceinline__ uint32_t skew16(uint32_t w) { return w + (w >> 4); }

// Bitmap layout: one u32 remainder set per local quotient, one pad uint4
// after every 8 uint4s, so threads owning 32 consecutive quotients sit 9
// uint4s apart and a quarter-warp of uint4 loads covers all 32 banks.
__device__ __forceinline__ uint32_t mask_word(uint32_t x)
{
    uint32_t u = x >> 2;
    return 4 * (u + (u >> 3)) + (x & 3u);
}

// u16 counters packed two per (skewed) u32 word
__device__ __forceinline__ uint32_t cnt16_get(const uint32_t *a, uint32_t i)
{
    return (a[skew16(i >> 1)] >> ((i & 1) * 16)) & 0xFFFFu;
}
__device__ __forceinline__ uint32_t cnt16_fetch_inc(uint32_t *a, uint32_t i)
{
    uint32_t old = atomicAdd(a + skew16(i >> 1), 1u << ((i & 1) * 16));
    return (old >> ((i & 1) * 16)) & 0xFFFFu;
}

template <typename T>
__device__ void small_sort(T *v, uint32_t n)
{
    if (n < 2) return;
    if (n <= 24) {
        for (uint32_t i = 1; i < n; i++) {
            T x = v[i];
            int j = (int)i - 1;
            while (j >= 0 && v[j] > x) {
                v[j + 1] = v[j];
                j--;
            }
            v[j + 1] = x;
        }
        return;
    }
    // heap sort for the rare large group (skewed input)
    auto sift = [&](uint32_t root, uint32_t end) {
        while (2 * root + 1 < end) {
            uint32_t c = 2 * root + 1;
            if (c + 1 < end && v[c] < v[c + 1]) c++;
            if (!(v[root] < v[c])) return;
            T t = v[root];
            v[root] = v[c];
            v[c] = t;
            root = c;
        }
    };
    for (int s = (int)n / 2 - 1; s >= 0; s--) sift((uint32_t)s, n);
    for (uint32_t e = n - 1; e > 0; e--) {
        T t = v[0];
        v[0] = v[e];
        v[e] = t;
        sift(0, e);
    }
}

// Per remainder value, how many copies the rebuilt group keeps, given ca
// copies from source A (the table's current contents) and cb from source B
// (the batch).  The reference semantics each op reproduces:
//   OP_BUILD   bulkBuildSegmentedLayouts: all of B, unique when NoDuplicates
//              (quotientFilter.cu:1478-1482)
//   OP_INSERT  insert: a fingerprint already present is left alone, a new one
//              is stored once (insertItemGPU :499-504)
//   OP_DELETE  superclusterDeletes: each delete removes one stored copy
//              (deleteItemGPU :1076-1200)
//   OP_MERGE   insertViaMerge / mergeTwoFilters: merged multiset, unique when
//              NoDuplicates (:1659-1664, :1808-1813)
enum LayoutOp : int { OP_BUILD = 0, OP_INSERT = 1, OP_DELETE = 2, OP_MERGE = 3 };

__device__ __forceinline__ uint32_t keep_count(int op, int nodup, uint32_t ca, uint32_t cb)
{
    switch (op) {
    case OP_INSERT: return ca ? ca : (cb ? 1u : 0u);
    case OP_DELETE: return ca > cb ? ca - cb : 0u;
    default: return nodup ? ((ca + cb) ? 1u : 0u) : ca + cb;
    }
}

// One source of fingerprints per bucket: items[base(b) .. base(b)+cnt[b]).
struct BucketSrc {
    const uint32_t *items;
    const uint32_t *base;  // nullptr: b * stride
    uint32_t stride;
    const uint32_t *cnt;   // nullptr: source absent
    __device__ __forceinline__ size_t start(uint32_t b) const { return base ? (size_t)base[b] : (size_t)b * stride; }
    // With speculative strides a bucket that overflowed counts more items
    // than its region holds (the host reruns the op with exact bases); read
    // at most the region, which keeps the last bucket inside the buffer.
    __device__ __forceinline__ uint32_t count(uint32_t b) const
    {
        return cnt ? (base ? cnt[b] : min(cnt[b], stride)) : 0u;
    }
};

struct LayoutArgs {
    BucketSrc A, B;
    uint8_t *table;
    uint32_t q, r, tb, nb, nslots;
    uint32_t cap_items;  // tagged remainders one CTA can hold (general mode)
    int op, nodup;
    // Remainder-bitmap mode: r = 5 and the op has set semantics (NoDup
    // build/merge, insert/delete into a table without duplicate
    // fingerprints); `a_dups` (device flag, may be null) vetoes it at run
    // time when the table holds duplicates.
    int bitmap_ok;
    const uint32_t *a_dups;
    unsigned long long *status;
    uint32_t *ticket;
    uint32_t *fix_list;
    uint32_t *fix_cnt;
    uint32_t fix_cap;
    // Fix-ups past fix_cap: an error (0), or dropped (1) because the caller
    // repairs the filter's occupied bits from its items when *fix_cnt ends
    // above fix_cap (batched builds).
    int fix_soft = 0;
    uint32_t *err;
    // In-place update (insert / delete, one-byte slots, bitmap mode): A is
    // decoded bucket by bucket from this snapshot of the table taken before
    // the op, instead of from an extracted list.  A bucket it cannot decode
    // here (duplicate or out-of-order remainders, runs past its staged
    // slice) sets *fused_fail and the host reruns the op the general way.
    const uint8_t *src_table = nullptr;
    uint32_t *fused_fail = nullptr;
    // When set, the launch does nothing unless *gate is nonzero (the general
    // path queued behind an asynchronous in-place update, run only if that
    // update could not place some bucket).
    const uint32_t *gate = nullptr;
};

// Shared-memory plan of k_bucket_layout: region 0 holds either the
// remainder bitmaps (one u32 per quotient) or the packed u16 group counters
// plus the tagged remainders; the tile buffer follows.
__host__ __device__ inline size_t layout_region0_bytes(uint32_t tb, uint32_t cap_items, int bpe, bool bitmap)
{
    size_t S = (size_t)1 << tb;
    size_t gen = 4 * (S / 2 + S / 32 + 8) + (((size_t)cap_items * bpe + 15) & ~(size_t)15);
    size_t bit = 4 * (S + S / 8);
    return bitmap && bit > gen ? bit : gen;
}
// The tile buffer's byte offsets are skewed by 16 bytes per 128: threads
// emitting slots about 32 apart then write distinct shared-memory banks, and
// 16-byte-aligned offsets stay 16-byte aligned.
__host__ __device__ inline size_t tile_skew(size_t off) { return off + ((off >> 7) << 4); }
__host__ __device__ inline size_t tile_bytes(uint32_t tb, int bpe)
{
    return (tile_skew((((size_t)1 << tb) + SPILL_SLOTS) * bpe + 32) + 16 + 15) & ~(size_t)15;
}
__host__ __device__ inline size_t layout_smem_bytes(uint32_t tb, uint32_t cap_items, int bpe, bool bitmap)
{
    size_t S = (size_t)1 << tb;
    size_t r0 = (layout_region0_bytes(tb, cap_items, bpe, bitmap) + 15) & ~(size_t)15;
    return r0 + tile_bytes(tb, bpe) + S / 8;  // + occupied bit per quotient
}
// Extra shared memory of the in-place update decode: per 32-slot word of
// the staged slice its run-start mask and the run starts before it, per
// 32-quotient word of the bucket its occupied mask and the count before it.
__host__ __device__ inline size_t layout_fused_bytes(uint32_t tb)
{
    const size_t S = (size_t)1 << tb, LW = (S + SPILL_SLOTS) / 32, QW = S / 32;
    return ((LW * 4 + 15) & ~(size_t)15) + ((LW * 2 + 15) & ~(size_t)15) + ((QW * 4 + 15) & ~(size_t)15) +
           ((QW * 2 + 15) & ~(size_t)15);
}

// Group walk (general mode): quotients [qb, qb+QPT) in slot order, calling
// emit(xa, rem, k) for every item the rebuilt table holds (k = index of the
// item within its quotient's run).  Groups hold (rem << 1 | source) sorted.
template <typename Rem, typename Emit>
__device__ __forceinline__ void walk_groups(const uint32_t *s_cnt, const Rem *s_rem, uint32_t qb, uint32_t QPT,
                                            uint32_t x0, int op, int nodup, Emit &&emit)
{
    for (uint32_t j = 0; j < QPT; j++) {
        uint32_t x = qb + j;
        uint32_t g0 = x ? cnt16_get(s_cnt, x - 1) : 0u, g1 = cnt16_get(s_cnt, x);
        uint32_t kk = 0;
        for (uint32_t k = g0; k < g1;) {
            uint32_t v = (uint32_t)s_rem[k] >> 1, ca = 0, cb = 0;
            while (k < g1 && ((uint32_t)s_rem[k] >> 1) == v) {
                if (s_rem[k] & 1) cb++; else ca++;
                k++;
            }
            uint32_t keep = keep_count(op, nodup, ca, cb);
            for (uint32_t c = 0; c < keep; c++) emit(x0 + x, v, kk++);
        }
    }
}

// ---------------------------------------------------------------------
// K2: one CTA per bucket (taken in ticket order for the look-back).
// ---------------------------------------------------------------------
// THREADS threads own QPT consecutive quotients each (S = THREADS * QPT).
// FUSED instantiations carry the in-place update decode (LayoutArgs::
// src_table); the others compile without it.
template <int THREADS, int QPT_, int BPE, bool FUSED = false>
__device__ __forceinline__ void bucket_layout_body(const LayoutArgs &a, const uint32_t b)
{
    using Rem = typename std::conditional<BPE == 1, uint8_t, uint16_t>::type;
    extern __shared__ __align__(16) uint8_t smem_layout[];
    const uint32_t S = 1u << a.tb;
    const bool bitmap = BPE == 1 && a.bitmap_ok && (a.src_table || !(a.a_dups && *a.a_dups));
    uint32_t *s_cnt = reinterpret_cast<uint32_t *>(smem_layout);   // general: u16 counters
    uint32_t *s_mask = reinterpret_cast<uint32_t *>(smem_layout);  // bitmap: u32 per local quotient
    Rem *s_rem = reinterpret_cast<Rem *>(smem_layout + 4 * ((size_t)S / 2 + S / 32 + 8));
    uint8_t *s_tile = smem_layout + ((layout_region0_bytes(a.tb, a.cap_items, BPE, a.bitmap_ok != 0) + 15) &
                                     ~(size_t)15);
    const uint32_t BUF = S + SPILL_SLOTS;  // slots the tile buffer holds

    __shared__ uint32_t s_warp[33];
    __shared__ uint32_t s_cin, s_cout, s_nfix, s_fbase;
    __shared__ LayoutFn s_wfn[THREADS / 32];
    __shared__ LayoutFn s_wexcl[THREADS / 32];
    __shared__ uint32_t s_fix[256];

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) s_nfix = 0;
    __syncthreads();
    const uint32_t na = a.A.count(b), nbn = a.B.count(b);
    const uint32_t n = na + nbn;
    const size_t abase = na ? a.A.start(b) : 0, bbase = nbn ? a.B.start(b) : 0;
    const uint32_t x0 = b * S;  // first quotient of the bucket
    const uint32_t rmask = (1u << a.r) - 1u;
    constexpr uint32_t QPT = QPT_;  // S == THREADS * QPT
    const uint32_t qb = tid * QPT;

    if (!bitmap && n > a.cap_items) {
        // cannot sort here: flag it (the host falls back) and keep the chain alive
        if (tid == 0) {
            atomicOr(a.err, DEV_ERR_BUCKET_CAP);
            st_relaxed_u64(a.status + b, lb_pack_inc(x0));
        }
        return;
    }
    auto item = [&](uint32_t i) -> uint32_t {
        return i < na ? a.A.items[abase + i] : a.B.items[bbase + (i - na)];
    };
    // items are read in batches of LB per thread so LB loads are in flight
    constexpr int LB = 8;

    if (FUSED && BPE == 1 && bitmap && a.src_table) {
        // In-place update: decode this bucket's old contents from the
        // snapshot.  Runs are stored in quotient order, one per occupied
        // quotient; the runs starting at or past x0 are first the D0 still
        // pending from quotients below x0, then those of the bucket's
        // occupied quotients in order.
        const uint32_t L = BUF;
        uint8_t *s_sl = s_tile;  // the slice, in the tile buffer until the emit
        uint8_t *fx = smem_layout + ((layout_smem_bytes(a.tb, a.cap_items, BPE, true) + 15) & ~(size_t)15);
        const size_t o1 = ((size_t)(L / 32) * 4 + 15) & ~(size_t)15, o2 = ((size_t)(L / 32) * 2 + 15) & ~(size_t)15,
                     o3 = ((size_t)(S / 32) * 4 + 15) & ~(size_t)15;
        uint32_t *s_rs32 = reinterpret_cast<uint32_t *>(fx);
        uint16_t *s_rsp = reinterpret_cast<uint16_t *>(fx + o1);
        uint32_t *s_oc32 = reinterpret_cast<uint32_t *>(fx + o1 + o2);
        uint16_t *s_ocp = reinterpret_cast<uint16_t *>(fx + o1 + o2 + o3);
        __shared__ int s_D0;
        __shared__ uint32_t s_nrs;
        for (uint32_t i = tid; i < (S + S / 8) / 4; i += THREADS)
            reinterpret_cast<uint4 *>(s_mask)[i] = make_uint4(0, 0, 0, 0);
        const uint8_t *src = a.src_table;
        for (uint32_t i = tid * 16; i < L; i += THREADS * 16) {
            uint4 w4;
            if ((size_t)x0 + i + 16 <= a.nslots) {
                w4 = __ldg(reinterpret_cast<const uint4 *>(src + x0 + i));
            } else {
                uint8_t tmp[16];
#pragma unroll
                for (int k = 0; k < 16; k++) tmp[k] = (size_t)x0 + i + k < a.nslots ? src[x0 + i + k] : 0;
                w4 = *reinterpret_cast<uint4 *>(tmp);
            }
            *reinterpret_cast<uint4 *>(s_sl + i) = w4;
        }
        if (wid == 0) {
            // runs of quotients below x0 still pending at x0
            const int D = pending_runs_warp(src, x0);
            if (lane == 0) s_D0 = D;
        }
        __syncthreads();
        // 32-slot masks: run starts over the slice, occupied over the bucket
        for (uint32_t w = tid; w < L / 32; w += THREADS) {
            uint32_t rsm = 0, ocm = 0;
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const Flags8 f = flags8(*reinterpret_cast<const uint64_t *>(s_sl + 32 * w + 8 * h));
                rsm |= ((f.nonempty & ~f.cont) & 0xFFu) << (8 * h);
                ocm |= (f.occ & 0xFFu) << (8 * h);
            }
            s_rs32[w] = rsm;
            if (w < S / 32) s_oc32[w] = ocm;
        }
        __syncthreads();
        // exclusive prefix counts: thread-contiguous word ranges + block scan
        {
            const uint32_t per = (L / 32 + THREADS - 1) / THREADS;
            const uint32_t w0 = min(L / 32, tid * per), w1 = min(L / 32, w0 + per);
            uint32_t cr = 0, co = 0;
            for (uint32_t w = w0; w < w1; w++) {
                cr += __popc(s_rs32[w]);
                if (w < S / 32) co += __popc(s_oc32[w]);
            }
            uint32_t ir = cr, io = co;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t x = __shfl_up_sync(0xffffffffu, ir, o), y = __shfl_up_sync(0xffffffffu, io, o);
                if (lane >= o) {
                    ir += x;
                    io += y;
                }
            }
            if (lane == 31) {
                s_wfn[wid].n = ir;
                s_wfn[wid].F = io;
            }
            __syncthreads();
            uint32_t pr = ir - cr, po = io - co;
            for (int w = 0; w < wid; w++) {
                pr += s_wfn[w].n;
                po += s_wfn[w].F;
            }
            if (tid == THREADS - 1) s_nrs = pr + cr;  // run starts in the slice
            for (uint32_t w = w0; w < w1; w++) {
                s_rsp[w] = (uint16_t)pr;
                pr += __popc(s_rs32[w]);
                if (w < S / 32) {
                    s_ocp[w] = (uint16_t)po;
                    po += __popc(s_oc32[w]);
                }
            }
        }
        // the batch: its remainders, per quotient, into the bitmaps
        for (uint32_t i0 = 0; i0 < nbn; i0 += THREADS * LB) {
            uint32_t v[LB];
#pragma unroll
            for (int k = 0; k < LB; k++) {
                const uint32_t i = i0 + k * THREADS + tid;
                v[k] = i < nbn ? a.B.items[bbase + i] : 0u;
            }
#pragma unroll
            for (int k = 0; k < LB; k++)
                if (i0 + k * THREADS + tid < nbn)
                    atomicOr(s_mask + mask_word((v[k] >> a.r) & (S - 1)), 1u << (v[k] & rmask));
        }
        __syncthreads();
        {
            // each thread decodes the runs of its own QPT quotients: the run
            // of its first occupied quotient is run start number D0 + (the
            // bucket's occupied quotients before qb); later ones follow in
            // slot order.  Then per quotient: old set | batch (insert) or
            // old set & ~batch (delete).
            const int D0 = s_D0;
            const int nrs = (int)s_nrs;
            const uint32_t qw = qb >> 5, qs = qb & 31;
            const uint32_t ocm = (s_oc32[qw] >> qs) & (QPT >= 32 ? 0xFFFFFFFFu : ((1u << (QPT & 31)) - 1u));
            const int j0 = (int)s_ocp[qw] + __popc(s_oc32[qw] & ((1u << qs) - 1u));
            const bool del = a.op == OP_DELETE;
            bool bad = false;
            uint32_t pos = 0;  // current run start (slot of the slice)
            if (ocm) {
                const int k = D0 + j0;
                if (k < 0 || k >= nrs) {
                    bad = true;
                } else {
                    uint32_t lo = 0, hi = L / 32;  // last word with s_rsp[w] <= k
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if ((int)s_rsp[mid] <= k) lo = mid;
                        else hi = mid;
                    }
                    pos = (lo << 5) + (uint32_t)select_bit(s_rs32[lo], k - (int)s_rsp[lo]);
                }
            }
            bool first = true;
#pragma unroll 4
            for (uint32_t jq = 0; jq < QPT; jq++) {
                uint32_t am = 0;
                if (((ocm >> jq) & 1u) && !bad) {
                    if (!first) {  // the next run start, at or past the previous run's end
                        uint32_t w = pos >> 5;
                        uint32_t mm = pos < L ? (s_rs32[w] & ~((1u << (pos & 31)) - 1u)) : 0u;
                        while (!mm && ++w < L / 32) mm = s_rs32[w];
                        if (!mm) bad = true;
                        else pos = (w << 5) + (uint32_t)(__ffs(mm) - 1);
                    }
                    first = false;
                    if (!bad) {
                        int prev = -1;
                        for (;;) {
                            const uint32_t rem = (uint32_t)s_sl[pos] >> 3;
                            if ((int)rem <= prev) bad = true;  // duplicate or unsorted run
                            prev = (int)rem;
                            am |= 1u << rem;
                            if (++pos >= L) {
                                bad = true;  // the run may continue past the slice
                                break;
                            }
                            const uint32_t e2 = s_sl[pos];
                            if (!((e2 & 7u) && (e2 & 2u))) break;
                        }
                    }
                }
                uint32_t *mw = s_mask + mask_word(qb + jq);
                *mw = del ? (am & ~*mw) : (am | *mw);
            }
            if (bad) atomicOr(a.fused_fail, 1u);
        }
        __syncthreads();
    } else if (bitmap && na == 0 && a.op != OP_DELETE && ((bbase & 3) == 0)) {
        // build from one 16-byte aligned source (the speculative bucket
        // stride keeps bucket starts aligned): the first four items per
        // thread as one 16-byte load issued before the masks are cleared,
        // the rest four at a time
        const uint4 *src4 = reinterpret_cast<const uint4 *>(a.B.items + bbase);
        const uint32_t n4 = nbn >> 2;
        auto put = [&](uint32_t v) {
            atomicOr(s_mask + mask_word((v >> a.r) & (S - 1)), 1u << (v & rmask));
        };
        constexpr int LV = 4;  // 16-byte loads in flight per thread
        uint4 w[LV];
#pragma unroll
        for (int k = 0; k < LV; k++) {
            const uint32_t j = k * THREADS + tid;
            w[k] = j < n4 ? __ldg(src4 + j) : make_uint4(0, 0, 0, 0);
        }
        for (uint32_t i = tid; i < (S + S / 8) / 4; i += THREADS)
            reinterpret_cast<uint4 *>(s_mask)[i] = make_uint4(0, 0, 0, 0);
        __syncthreads();
        for (uint32_t j0 = 0;; j0 += LV * THREADS) {
#pragma unroll
            for (int k = 0; k < LV; k++) {
                if (j0 + k * THREADS + tid < n4) {
                    put(w[k].x);
                    put(w[k].y);
                    put(w[k].z);
                    put(w[k].w);
                }
            }
            if (j0 + LV * THREADS >= n4) break;
#pragma unroll
            for (int k = 0; k < LV; k++) {
                const uint32_t j = j0 + LV * THREADS + k * THREADS + tid;
                w[k] = j < n4 ? __ldg(src4 + j) : make_uint4(0, 0, 0, 0);
            }
        }
        for (uint32_t i = (n4 << 2) + tid; i < nbn; i += THREADS) put(a.B.items[bbase + i]);  // tail
        __syncthreads();
    } else if (bitmap) {
        // A: remainder sets by quotient (A first, then B); mask of local
        // quotient x lives at word mask_word(x) (one pad uint4 per 8)
        for (uint32_t i = tid; i < (S + S / 8) / 4; i += THREADS)
            reinterpret_cast<uint4 *>(s_mask)[i] = make_uint4(0, 0, 0, 0);
        __syncthreads();
        for (int src = 0; src < 2; src++) {
            const uint32_t lo_i = src ? na : 0u, hi_i = src ? n : na;
            const bool clear = src == 1 && a.op == OP_DELETE;
            for (uint32_t i0 = lo_i; i0 < hi_i; i0 += THREADS * LB) {
                uint32_t v[LB];
#pragma unroll
                for (int k = 0; k < LB; k++) {
                    uint32_t i = i0 + k * THREADS + tid;
                    v[k] = i < hi_i ? item(i) : 0u;
                }
#pragma unroll
                for (int k = 0; k < LB; k++) {
                    if (i0 + k * THREADS + tid < hi_i) {
                        uint32_t w = mask_word((v[k] >> a.r) & (S - 1)), bit = 1u << (v[k] & rmask);
                        if (clear) atomicAnd(s_mask + w, ~bit);
                        else atomicOr(s_mask + w, bit);
                    }
                }
            }
            __syncthreads();
        }
    } else {
        // A: counting sort of tagged remainders by local quotient
        for (uint32_t i = tid; i < S / 2 + S / 32 + 8; i += THREADS) s_cnt[i] = 0;
        __syncthreads();
        for (uint32_t i0 = 0; i0 < n; i0 += THREADS * LB) {
            uint32_t v[LB];
#pragma unroll
            for (int k = 0; k < LB; k++) {
                uint32_t i = i0 + k * THREADS + tid;
                v[k] = i < n ? item(i) : 0u;
            }
#pragma unroll
            for (int k = 0; k < LB; k++)
                if (i0 + k * THREADS + tid < n) cnt16_fetch_inc(s_cnt, (v[k] >> a.r) & (S - 1));
        }
        __syncthreads();
        // exclusive scan of the u16 counters: thread owns QPT consecutive quotients
        {
            uint32_t sum = 0;
            for (uint32_t j = 0; j < QPT; j++) sum += cnt16_get(s_cnt, qb + j);
            uint32_t incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane == 31) s_warp[wid] = incl;
            __syncthreads();
            if (wid == 0) {
                uint32_t v = lane < THREADS / 32 ? s_warp[lane] : 0;
                uint32_t iv = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t t = __shfl_up_sync(0xffffffffu, iv, o);
                    if (lane >= o) iv += t;
                }
                if (lane < THREADS / 32) s_warp[lane] = iv - v;
            }
            __syncthreads();
            uint32_t run = s_warp[wid] + incl - sum;
            for (uint32_t j = 0; j < QPT; j += 2) {  // QPT even: whole words
                uint32_t c0 = cnt16_get(s_cnt, qb + j), c1 = cnt16_get(s_cnt, qb + j + 1);
                s_cnt[skew16((qb + j) >> 1)] = run | ((run + c0) << 16);
                run += c0 + c1;
            }
        }
        __syncthreads();
        for (uint32_t i0 = 0; i0 < n; i0 += THREADS * LB) {
            uint32_t v[LB];
#pragma unroll
            for (int k = 0; k < LB; k++) {
                uint32_t i = i0 + k * THREADS + tid;
                v[k] = i < n ? item(i) : 0u;
            }
#pragma unroll
            for (int k = 0; k < LB; k++) {
                uint32_t i = i0 + k * THREADS + tid;
                if (i < n) {
                    uint32_t p = cnt16_fetch_inc(s_cnt, (v[k] >> a.r) & (S - 1));
                    s_rem[p] = (Rem)(((v[k] & rmask) << 1) | (i >= na ? 1u : 0u));
                }
            }
        }
        __syncthreads();
        // s_cnt[x] now holds the END of group x; group x = [end(x-1), end(x))
        for (uint32_t j = 0; j < QPT; j++) {
            uint32_t x = qb + j;
            uint32_t g0 = x ? cnt16_get(s_cnt, x - 1) : 0u, g1 = cnt16_get(s_cnt, x);
            if (g1 - g0 > 1) small_sort(s_rem + g0, g1 - g0);
        }
    }
    // Bitmap mode: this thread's QPT remainder sets, held in registers
    // (QPT/4 conflict-free uint4 loads: thread strides are 9 uint4 apart).
    uint32_t mreg[QPT];
    if (bitmap) {
#pragma unroll
        for (uint32_t j = 0; j < QPT / 4; j++) {
            uint4 m4 = reinterpret_cast<const uint4 *>(s_mask)[mask_word(qb + 4 * j) >> 2];
            mreg[4 * j] = m4.x;
            mreg[4 * j + 1] = m4.y;
            mreg[4 * j + 2] = m4.z;
            mreg[4 * j + 3] = m4.w;
        }
    }
    auto warp_incl = [&](LayoutFn f) -> LayoutFn {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            LayoutFn p;
            p.n = __shfl_up_sync(0xffffffffu, f.n, o);
            p.F = __shfl_up_sync(0xffffffffu, f.F, o);
            if (lane >= o) f = compose(p, f);
        }
        return f;
    };
    // every item the rebuilt bucket keeps, in slot order, for this thread
    // (general mode)
    auto walk = [&](auto &&emit) { walk_groups(s_cnt, s_rem, qb, QPT, x0, a.op, a.nodup, emit); };

    // B/C: this thread's layout map, then a warp scan of the maps
    LayoutFn fn{0u, 0u};
    if (bitmap) {
        uint32_t c = 0, cnt_items = 0;
#pragma unroll
        for (uint32_t j = 0; j < QPT; j++) {
            uint32_t k = __popc(mreg[j]);
            if (k) {
                uint32_t xa = x0 + qb + j;
                c = (xa > c ? xa : c) + k;
                cnt_items += k;
            }
        }
        fn.n = cnt_items;
        fn.F = cnt_items ? c : 0u;
    } else {
        uint32_t c = 0, cnt_items = 0;
        walk([&](uint32_t xa, uint32_t, uint32_t) {
            uint32_t pos = xa > c ? xa : c;
            c = pos + 1;
            cnt_items++;
        });
        fn.n = cnt_items;
        fn.F = cnt_items ? c : 0u;
    }
    LayoutFn wexcl{0u, 0u};
    {
        LayoutFn incl = warp_incl(fn);
        wexcl.n = __shfl_up_sync(0xffffffffu, incl.n, 1);
        wexcl.F = __shfl_up_sync(0xffffffffu, incl.F, 1);
        if (lane == 0) wexcl = LayoutFn{0u, 0u};
        if (lane == 31) s_wfn[wid] = incl;
    }
    __syncthreads();
    if (wid == 0) {
        LayoutFn acc{0u, 0u};
        for (int w = 0; w < THREADS / 32; w++) {
            if (lane == 0) s_wexcl[w] = acc;
            acc = compose(acc, s_wfn[w]);
        }
        // D: publish the aggregate, look back, publish the inclusive value
        if (lane == 0 && (acc.n > LB_VMAX / 2 || acc.F > LB_VMAX / 2)) atomicOr(a.err, DEV_ERR_FULL);
        uint32_t cin = 0;
        if (b != 0) {
            if (lane == 0) st_relaxed_u64(a.status + b, lb_pack_agg(acc.n, acc.F));
            cin = lookback_cin_warp(a.status, b, a.err);
        }
        uint32_t cout = acc.apply(cin);
        if (lane == 0) {
            st_relaxed_u64(a.status + b, lb_pack_inc(cout));
            s_cin = cin;
            s_cout = cout;
        }
    }
    __syncthreads();
    const uint32_t cin = s_cin, cout = s_cout;
    const uint32_t lo = cin > x0 ? cin : x0;
    uint32_t hi = cout > x0 + S ? cout : x0 + S;
    if (hi > a.nslots) {
        if (cout > a.nslots && tid == 0) atomicOr(a.err, DEV_ERR_FULL);
        hi = a.nslots;
    }
    const uint32_t span = hi > lo ? hi - lo : 0u;
    const uint32_t bufslots = span < BUF ? span : BUF;
    const size_t gs = (size_t)lo * BPE;             // first table byte written
    const size_t ge = gs + (size_t)bufslots * BPE;  // end of the buffered part
    const size_t gal = gs & ~(size_t)15;            // smem byte 0 <-> table byte gal
    // occupied bits of the bucket's own quotients, one bit per slot x0..x0+S
    uint32_t *s_occ = reinterpret_cast<uint32_t *>(s_tile + tile_bytes(a.tb, BPE));
    for (size_t i = tid * 16; i < tile_skew(ge - gal); i += THREADS * 16)
        *reinterpret_cast<uint4 *>(s_tile + i) = make_uint4(0, 0, 0, 0);
    for (uint32_t i = tid; i < S / 32; i += THREADS) s_occ[i] = 0;
    __syncthreads();

    auto put_elem = [&](uint32_t pos, uint32_t e) {
        uint8_t *d = (pos - lo < bufslots) ? s_tile + tile_skew((size_t)pos * BPE - gal) : a.table + (size_t)pos * BPE;
        if (BPE == 1) {
            d[0] = (uint8_t)e;
        } else {
            d[0] = (uint8_t)(e >> 8);
            d[1] = (uint8_t)e;
        }
    };
    auto add_fix = [&](uint32_t xa) {
        uint32_t p = atomicAdd(&s_nfix, 1u);
        if (p < 256) {
            s_fix[p] = xa;
        } else {
            uint32_t gp = atomicAdd(a.fix_cnt, 1u);
            if (gp < a.fix_cap) a.fix_list[gp] = xa;
            else if (!a.fix_soft) atomicOr(a.err, DEV_ERR_BUCKET_CAP);
        }
    };
    // E: emit elements; record occupied quotients (bit array) and the ones
    // whose slot an earlier bucket writes (fix-ups)
    if (bitmap) {
        const LayoutFn texcl = compose(s_wexcl[wid], wexcl);
        uint32_t c = texcl.apply(cin);
        // occupied quotients of this thread; those below lo (their slot was
        // written by an earlier bucket) become fix-ups
        uint32_t nz = 0;
#pragma unroll
        for (uint32_t j = 0; j < QPT; j++) nz |= (mreg[j] != 0u ? 1u : 0u) << j;
        const uint32_t xb = x0 + qb;
        const uint32_t nbelow = lo > xb ? min(lo - xb, 32u) : 0u;
        const uint32_t bmask = nbelow >= 32u ? 0xFFFFFFFFu : ((1u << nbelow) - 1u);
        for (uint32_t fx = nz & bmask; fx; fx &= fx - 1u) add_fix(xb + (uint32_t)__ffs(fx) - 1u);
        const uint32_t occ = nz & ~bmask;
        if (QPT >= 32) s_occ[qb >> 5] = occ;  // this thread owns the whole word
        else if (occ) atomicOr(s_occ + (qb >> 5), occ << (qb & 31));
        // the thread's items in slot order, one per iteration (a loop per
        // quotient would make the warp wait for its fullest quotient at
        // every step); the next quotient's set comes from shared memory
        uint32_t m = 0, pos = 0, e0 = 0, nzr = nz;
        for (uint32_t it = 0; it < fn.n; it++) {
            if (!m) {
                const uint32_t j = (uint32_t)__ffs(nzr) - 1u;
                nzr &= nzr - 1u;
                m = s_mask[mask_word(qb + j)];
                const uint32_t xa = xb + j;
                pos = xa > c ? xa : c;
                e0 = pos != xa ? 1u : 0u;  // shifted
            }
            const uint32_t v = (uint32_t)__ffs(m) - 1u;
            m &= m - 1u;
            if (pos < hi) put_elem(pos, (v << 3) | e0);
            e0 = 3u;  // later items of the run: continuation + shifted
            c = ++pos;
        }
    } else {
        const LayoutFn texcl = compose(s_wexcl[wid], wexcl);
        uint32_t c = texcl.apply(cin);
        walk([&](uint32_t xa, uint32_t rem, uint32_t kk) {
            uint32_t pos = xa > c ? xa : c;
            c = pos + 1;
            if (kk == 0) {
                if (xa >= lo) atomicOr(s_occ + ((xa - x0) >> 5), 1u << ((xa - x0) & 31));
                else add_fix(xa);
            }
            if (pos >= hi) return;  // past the table: reported as FULL
            put_elem(pos, (rem << 3) | (kk ? 2u : 0u) | (pos != xa ? 1u : 0u));
        });
    }
    __syncthreads();
    // occupied bit of slot at table byte g (g on an element's last byte)
    auto occ_at = [&](size_t g) -> uint32_t {
        size_t slot = g / BPE;
        if (slot < x0 || slot >= (size_t)x0 + S) return 0u;
        uint32_t o = (uint32_t)(slot - x0);
        return (s_occ[o >> 5] >> (o & 31)) & 1u;
    };
    {
        uint32_t nf = s_nfix < 256 ? s_nfix : 256;
        if (tid == 0 && nf) s_fbase = atomicAdd(a.fix_cnt, nf);
        __syncthreads();
        for (uint32_t i = tid; i < nf; i += THREADS) {
            uint32_t gp = s_fbase + i;
            if (gp < a.fix_cap) a.fix_list[gp] = s_fix[i];
            else if (!a.fix_soft) atomicOr(a.err, DEV_ERR_BUCKET_CAP);
        }
    }
    // G: store the tile (occupied bits merged in): head bytes, 16-byte body,
    // tail bytes
    {
        size_t h_end = (gs + 15) & ~(size_t)15;
        if (h_end > ge) h_end = ge;
        size_t b_end = ge & ~(size_t)15;
        if (b_end < h_end) b_end = h_end;
        auto byte_out = [&](size_t g) -> uint8_t {
            uint8_t v = s_tile[tile_skew(g - gal)];
            if ((g % BPE) == BPE - 1) v |= (uint8_t)(occ_at(g) << 2);
            return v;
        };
        for (size_t g = gs + tid; g < h_end; g += THREADS) a.table[g] = byte_out(g);
        for (size_t g = h_end + (size_t)tid * 16; g < b_end; g += (size_t)THREADS * 16) {
            uint4 v = *reinterpret_cast<const uint4 *>(s_tile + tile_skew(g - gal));
            if (BPE == 1) {
                // 16 slots: spread their 16 occupied bits onto bit 2 of each byte
                uint32_t bits = 0;
                if (g >= x0 && g < (size_t)x0 + S) {  // g - x0 is a multiple of 16
                    uint32_t o = (uint32_t)(g - x0);
                    bits = (s_occ[o >> 5] >> (o & 16u)) & 0xFFFFu;
                }
                auto spread4 = [](uint32_t x4) -> uint32_t { return ((x4 * 0x00204081u) & 0x01010101u) << 2; };
                v.x |= spread4(bits & 15u);
                v.y |= spread4((bits >> 4) & 15u);
                v.z |= spread4((bits >> 8) & 15u);
                v.w |= spread4((bits >> 12) & 15u);
            } else {
                uint8_t *pb = reinterpret_cast<uint8_t *>(&v);
                for (int k = 0; k < 16; k++)
                    if (((g + k) % BPE) == BPE - 1) pb[k] |= (uint8_t)(occ_at(g + k) << 2);
            }
            *reinterpret_cast<uint4 *>(a.table + g) = v;
        }
        for (size_t g = b_end + tid; g < ge; g += THREADS) a.table[g] = byte_out(g);
    }
}

// One CTA per bucket, taken in ticket order so every bucket's predecessors
// are running or done when it looks back.
template <int THREADS, int QPT_, int BPE, bool FUSED = false>
__global__ void __launch_bounds__(THREADS, (THREADS >= 1024 ? 1 : 2)) k_bucket_layout(LayoutArgs a)
{
    if (a.gate && !*a.gate) return;
    __shared__ uint32_t s_ticket;
    if (threadIdx.x == 0) s_ticket = atomicAdd(a.ticket, 1u);
    __syncthreads();
    bucket_layout_body<THREADS, QPT_, BPE, FUSED>(a, s_ticket);
}

template <int BPE>
__global__ void k_fixup_occ(uint8_t *table, const uint32_t *fix_list, const uint32_t *fix_cnt, uint32_t fix_cap,
                            const uint32_t *gate = nullptr)
{
    if (gate && !*gate) return;
    uint32_t nf = min(*fix_cnt, fix_cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x)
        table[(size_t)fix_list[i] * BPE + (BPE - 1)] |= 4u;
}

}  // namespace gqf

#include "sqf_merge.cuh"
