// C ABI of the rank-and-select quotient filter: host orchestration.
// Compiled twice: as is (RBITS 5, gqf_rsqf_* names) and from rsqf8_api.cu
// (RBITS 8, gqf_rsqf8_* names).
#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "host_common.cuh"
#include "rsqf.cuh"
#include "rsqf_build.cuh"
#include "sqf_build.cuh"

#ifndef GQF_RSQF_API
#define GQF_RSQF_API(name) gqf_rsqf_##name
#endif

namespace GQF_RSQF_NS {
using namespace ::gqf;

static bool rsqf_q_ok(unsigned q) { return q >= 7 && q + RSQF_R <= 31; }

static uint32_t ceil_log2u(uint64_t x)
{
    uint32_t l = 0;
    while ((1ull << l) < x) l++;
    return l;
}

// Bucket geometry for RSQF batches (fingerprint = quotient << 5 | remainder,
// the SQF r = 5 layout): ~12k items per bucket, at most 4096 buckets.
static BucketGeom rsqf_geom(uint32_t q, uint64_t n)
{
    BucketGeom g;
    uint32_t tb_lo = std::max<uint32_t>(7, q > 12 ? q - 12 : 0);
    uint32_t tb_hi = std::min<uint32_t>(q, 15);
    uint32_t tb = ceil_log2u((12000ull << q) / (n ? n : 1));
    tb = std::min(std::max(tb, tb_lo), tb_hi);
    g.q = q;
    g.r = RSQF_R;
    g.tb = tb;
    g.nb = 1u << (q - tb);
    g.shift = RSQF_R + tb;
    g.fp_mask = (1u << (q + RSQF_R)) - 1u;
    return g;
}

template <typename K>
static cudaError_t set_smem(K kernel, size_t bytes)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

__global__ void __launch_bounds__(1024) k_rsqf_scan_bases(const uint32_t *cnt, uint32_t nb, uint32_t *base)
{
    __shared__ uint32_t s[4097];
    __shared__ uint32_t sw[33];
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) s[i] = cnt[i];
    __syncthreads();
    uint32_t tot = block_exclusive_scan_u32<1024>(s, nb, sw);
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) base[i] = s[i];
    if (threadIdx.x == 0) base[nb] = tot;
}

// Sorts each bucket of fingerprints in place (exact bucket bases, so the
// whole array ends up sorted): counting sort by local quotient in shared
// memory, then the (small) groups of equal quotient by value.
constexpr int SORT_THREADS = 512;
__host__ __device__ inline size_t sort_smem_bytes(uint32_t tb, uint32_t cap)
{
    size_t S = (size_t)1 << tb;
    return 4 * (S / 2 + S / 32 + 8) + 4 * (size_t)cap;
}
// With bmax non-null it also stores, per bucket, max(quotient_j - j) over
// the bucket's items (j = index in the whole sorted array), the input of the
// canonical-position scan.
__global__ void __launch_bounds__(SORT_THREADS) k_bucket_sort(uint32_t *items, const uint32_t *base,
                                                             const uint32_t *cnt, uint32_t tb, uint32_t cap,
                                                             uint32_t *err, int32_t *bmax)
{
    extern __shared__ __align__(16) uint32_t smem_sort[];
    const uint32_t S = 1u << tb;
    uint32_t *s_cnt = smem_sort;
    uint32_t *s_it = smem_sort + (S / 2 + S / 32 + 8);
    __shared__ uint32_t s_warp[33];
    const uint32_t b = blockIdx.x, n = cnt[b];
    const size_t b0 = base[b];
    if (n <= 1 || n > cap) {
        if (threadIdx.x == 0) {
            if (n > cap) atomicOr(err, DEV_ERR_BUCKET_CAP);
            if (bmax) bmax[b] = n == 1 ? (int32_t)(items[b0] >> RSQF_R) - (int32_t)b0 : INT_MIN;
        }
        return;
    }
    for (uint32_t i = threadIdx.x; i < S / 2 + S / 32 + 8; i += SORT_THREADS) s_cnt[i] = 0;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += SORT_THREADS) cnt16_fetch_inc(s_cnt, (items[b0 + i] >> RSQF_R) & (S - 1));
    __syncthreads();
    // exclusive scan of the packed u16 counters, S/2 words in skewed order
    {
        // quotients per thread, even so the two u16 counters of a word
        // belong to one thread
        const uint32_t per = max(2u, ((S + SORT_THREADS - 1) / SORT_THREADS + 1) & ~1u);
        const uint32_t q0 = min(S, threadIdx.x * per), q1 = min(S, q0 + per);
        uint32_t sum = 0;
        for (uint32_t x = q0; x < q1; x++) sum += cnt16_get(s_cnt, x);
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        uint32_t incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) s_warp[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint32_t v = lane < SORT_THREADS / 32 ? s_warp[lane] : 0, iv = v;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, iv, o);
                if (lane >= o) iv += t;
            }
            if (lane < SORT_THREADS / 32) s_warp[lane] = iv - v;
        }
        __syncthreads();
        uint32_t run = s_warp[wid] + incl - sum;
        __syncthreads();
        for (uint32_t x = q0; x < q1; x++) {
            uint32_t c = cnt16_get(s_cnt, x);
            uint32_t w = skew16(x >> 1), sh = (x & 1) * 16;
            s_cnt[w] = (s_cnt[w] & ~(0xFFFFu << sh)) | (run << sh);
            run += c;
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += SORT_THREADS) {
        uint32_t v = items[b0 + i];
        s_it[cnt16_fetch_inc(s_cnt, (v >> RSQF_R) & (S - 1))] = v;
    }
    __syncthreads();
    for (uint32_t x = threadIdx.x; x < S; x += SORT_THREADS) {
        uint32_t g0 = x ? cnt16_get(s_cnt, x - 1) : 0u, g1 = cnt16_get(s_cnt, x);
        if (g1 - g0 > 1) small_sort(s_it + g0, g1 - g0);
    }
    __syncthreads();
    int32_t m = INT_MIN;
    for (uint32_t i = threadIdx.x; i < n; i += SORT_THREADS) {
        const uint32_t v = s_it[i];
        items[b0 + i] = v;
        m = max(m, (int32_t)(v >> RSQF_R) - (int32_t)(b0 + i));
    }
    if (bmax) {
        int32_t tot;
        block_excl_max<SORT_THREADS>(m, reinterpret_cast<int32_t *>(s_warp), tot);
        if (threadIdx.x == 0) bmax[b] = tot;
    }
}

// Lists this round's groups: every active group start with batch items.
// Groups of at most RSQF_SMALL_GROUP blocks (nearly all of an incremental
// batch) go to list 0, replayed by warps with small staging areas, many per
// SM; groups of at most RSQF_WARP_GROUP_MAX blocks to list 1; larger ones to
// list 2, replayed by one thread each in global memory.
constexpr uint32_t RSQF_SMALL_GROUP = 16;      // 1 KB of staging per warp
constexpr uint32_t RSQF_WARP_GROUP_MAX = 224;  // 14 KB of staging per warp
__global__ void k_rsqf_groups(uint32_t nblocks, const uint8_t *__restrict__ start, uint8_t *__restrict__ active,
                              const uint32_t *__restrict__ fhome, uint32_t *__restrict__ list0,
                              uint32_t *__restrict__ list1, uint32_t *__restrict__ list2, uint32_t *__restrict__ counts)
{
    const uint32_t total = nblocks + 1;  // logical blocks + guard block
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < total; b += gridDim.x * blockDim.x) {
        if (!start[b] || !active[b]) continue;
        active[b] = 0;
        uint32_t e = b + 1;
        while (e < total && !start[e]) e++;
        if (fhome[min(b, nblocks)] == fhome[min(e, nblocks)]) continue;  // no items: table unchanged
        const int which = e - b <= RSQF_SMALL_GROUP ? 0 : (e - b <= RSQF_WARP_GROUP_MAX ? 1 : 2);
        uint32_t *list = which == 0 ? list0 : (which == 1 ? list1 : list2);
        const uint32_t k = atomicAdd(counts + which, 1u);
        list[2 * k] = b;
        list[2 * k + 1] = e;
    }
}

// One replay round, a warp per listed group (WARPS warps per CTA, each with
// its own MAXB-block staging area): stage the group's blocks from t0,
// insert its items (fhome: first sorted index homed at or past each block)
// in ascending order, write the blocks back unless a write left the group
// (then the group is marked crossed and t is left as it was).
// Where a build's replay of group [b, e) (items [i0, i1)) may start.  An
// ascending insert departs from the canonical positions only once its walk
// meets a block whose offset exceeds 62, and in a cluster that first happens
// for the first item positioned in the cluster's first such block S1
// (items before it sit below S1, items homed before the group stay out of
// it): items [i0, fpos[S1]) are canonical (the rule is pinned on the oracle
// by tests/test_oracle.py), so the replay writes their canonical state and
// runs the reference insert from fpos[S1] on.  `sus` marks blocks whose
// canonical offset exceeds 62; a group without one replays all its items.
__device__ __forceinline__ uint32_t rsqf_replay_start(const uint8_t *sus, const uint32_t *fpos, uint32_t b,
                                                      uint32_t e, uint32_t i0, uint32_t i1)
{
    for (uint32_t blk = b; blk < e; blk++)
        if (sus[blk]) return min(max(fpos[blk], i0), i1);
    return i0;
}

template <uint32_t MAXB, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_rsqf_round_warp(
    uint8_t *__restrict__ t, const uint8_t *__restrict__ t0, uint32_t nblocks, uint32_t q,
    const uint32_t *__restrict__ fps, const uint32_t *__restrict__ fhome, const uint32_t *__restrict__ list,
    const uint32_t *__restrict__ count, uint8_t *__restrict__ crossed, uint32_t *n_crossed,
    int32_t *__restrict__ ret, int t0_zero, const uint8_t *__restrict__ sus, const uint32_t *__restrict__ fpos)
{
    __shared__ __align__(16) uint8_t sm_all[WARPS][MAXB * RSQF_SB];
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint8_t *sm = sm_all[wid];
    const uint32_t ng = *count;
    for (uint32_t gi = blockIdx.x * WARPS + wid; gi < ng; gi += gridDim.x * WARPS) {
        const uint32_t b = list[2 * gi], e = list[2 * gi + 1];
        for (uint32_t i = lane; i < (e - b) * RSQF_SW; i += 32) {  // staged words: offset, occ, runEnds, remainders
            const uint32_t blk = b + i / RSQF_SW, w = i % RSQF_SW;
            const uint8_t *src = t0 + (size_t)blk * RSQF_BB;
            uint64_t v;
            if (w == 0) v = src[0];
            else if (w == 1) v = ld_u64_unaligned(src + 1);
            else if (w == 2) v = ld_u64_unaligned(src + 9);
            else v = ld_u64_unaligned(src + 17 + 8 * (w - 3));
            *reinterpret_cast<uint64_t *>(sm + (size_t)(blk - b) * RSQF_SB + 8 * w) = v;
        }
        __syncwarp();
        RsqfWarpTable f{sm, t0, nblocks, b, e, false, lane, t0_zero != 0};
        const uint32_t i0 = fhome[min(b, nblocks)], i1 = fhome[min(e, nblocks)];
        uint32_t istart = i0;
        if (sus) {
            // a build: the canonical state of the items before the first
            // block of offset > 62, then the exact replay from there
            istart = rsqf_replay_start(sus, fpos, b, min(e, nblocks), i0, i1);
            for (uint32_t i = i0 + lane; i < istart; i += 32) {
                const uint32_t fp = fps[i], s = (uint32_t)ret[i];
                const uint32_t blk = s / RSQF_SPB, sl = s % RSQF_SPB, hb = (fp >> RSQF_R) / RSQF_SPB;
                unsigned long long *bs = reinterpret_cast<unsigned long long *>(sm + (size_t)(blk - b) * RSQF_SB);
                unsigned long long *bh = reinterpret_cast<unsigned long long *>(sm + (size_t)(hb - b) * RSQF_SB);
                atomicOr(bh + 1, 1ull << ((fp >> RSQF_R) % RSQF_SPB));  // occupieds of the home block
                if (i + 1 == istart || (fps[i + 1] >> RSQF_R) != (fp >> RSQF_R)) atomicOr(bs + 2, 1ull << sl);
                const uint32_t bit = sl * RSQF_R, wi = bit >> 6, sh = bit & 63;
                const unsigned long long r = fp & RSQF_RMASK;
                atomicOr(bs + 3 + wi, r << sh);
                if (sh + RSQF_R > 64) atomicOr(bs + 4 + wi, r >> (64 - sh));
            }
            // offsets: items homed below the block and stored in it
            for (uint32_t blk = b + lane; blk < e && blk < nblocks; blk += 32) {
                const uint32_t hi = min(fhome[blk], istart), lo = max(fpos[blk], i0);
                sm[(size_t)(blk - b) * RSQF_SB] = (uint8_t)(hi > lo ? hi - lo : 0u);
            }
            __syncwarp();
        }
        for (uint32_t i = istart; i < i1; i++) {
            const int32_t slot = rsqf_insert(f, q, fps[i]);
            if (f.crossed) break;
            if (lane == 0) ret[i] = slot;
        }
        __syncwarp();
        if (f.crossed) {
            if (lane == 0) {
                crossed[b] = 1;
                atomicAdd(n_crossed, 1u);
            }
        } else {
            for (uint32_t k = lane; k < (e - b) * RSQF_BB; k += 32) {
                const size_t a = (size_t)b * RSQF_BB + k;
                t[a] = *f.staged_byte(a);
            }
            if (lane == 0) crossed[b] = 0;
        }
        __syncwarp();
    }
}

// The same round for groups too large to stage: one thread per group,
// blocks restored from t0 in place.
__global__ void k_rsqf_round_big(uint8_t *t, const uint8_t *t0, uint32_t nblocks, uint32_t q, const uint32_t *fps,
                                 const uint32_t *fhome, const uint32_t *blist, const uint32_t *counts,
                                 uint8_t *crossed, uint32_t *n_crossed, int32_t *ret, int t0_zero,
                                 const uint8_t *sus, const uint32_t *fpos)
{
    const uint32_t ng = counts[2];
    for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ng; gi += gridDim.x * blockDim.x) {
        const uint32_t b = blist[2 * gi], e = blist[2 * gi + 1];
        for (size_t i = (size_t)b * RSQF_BB; i < (size_t)e * RSQF_BB; i++) t[i] = t0[i];
        RsqfGroupTable f{t, t0, nblocks, b, e, false, t0_zero != 0};
        const uint32_t i0 = fhome[min(b, nblocks)], i1 = fhome[min(e, nblocks)];
        uint32_t istart = i0;
        if (sus) {  // a build: as in k_rsqf_round_warp, on the packed blocks
            istart = rsqf_replay_start(sus, fpos, b, min(e, nblocks), i0, i1);
            for (uint32_t i = i0; i < istart; i++) {
                const uint32_t fp = fps[i], s = (uint32_t)ret[i];
                const uint32_t blk = s / RSQF_SPB, sl = s % RSQF_SPB, hq = (fp >> RSQF_R);
                f.set_occ(hq / RSQF_SPB, f.occ(hq / RSQF_SPB) | (1ull << (hq % RSQF_SPB)));
                if (i + 1 == istart || (fps[i + 1] >> RSQF_R) != hq) f.set_re(blk, f.re(blk) | (1ull << sl));
                f.set_rem(blk, sl, fp & RSQF_RMASK);
            }
            for (uint32_t blk = b; blk < e && blk < nblocks; blk++) {
                const uint32_t hi = min(fhome[blk], istart), lo = max(fpos[blk], i0);
                f.set_off(blk, hi > lo ? hi - lo : 0u);
            }
        }
        bool cross = false;
        for (uint32_t i = istart; i < i1; i++) {
            const int32_t slot = rsqf_insert(f, q, fps[i]);
            if (f.crossed) {
                cross = true;
                break;
            }
            ret[i] = slot;
        }
        crossed[b] = cross ? 1 : 0;
        if (cross) atomicAdd(n_crossed, 1u);
    }
}

// Merge every crossed group with its successor (chains collapse in one
// pass) and mark the merged groups active for the next round.
__global__ void k_rsqf_merge(uint32_t nblocks, uint8_t *start, uint8_t *active, uint8_t *crossed)
{
    const uint32_t total = nblocks + 1;
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < total; b += gridDim.x * blockDim.x) {
        if (!start[b] || !crossed[b]) continue;
        uint32_t e = b + 1;
        while (e < total && !start[e]) e++;
        if (e < total) start[e] = 0;  // successor joins this group
        active[b] = 1;
        crossed[b] = 0;
    }
}

}  // namespace GQF_RSQF_NS

using namespace GQF_RSQF_NS;

extern "C" {

size_t GQF_RSQF_API(num_blocks)(unsigned int q) { return (((size_t)1u << q) + 63) / 64 + 1; }

int GQF_RSQF_API(init)(gqf_rsqf *cqf, unsigned int q)
{
    if (!cqf || !rsqf_q_ok(q)) return GQF_ERR_ARG;
    cqf->qbits = q;
    cqf->numBlocks = (unsigned)GQF_RSQF_API(num_blocks)(q);
    size_t bytes = rsqf_table_bytes(cqf->numBlocks);
    void *p = nullptr;
    GQF_CK(cudaMalloc(&p, bytes));
    GQF_CK(cudaMemset(p, 0, bytes));
    cqf->blocks = p;
    return GQF_OK;
}

int GQF_RSQF_API(free)(gqf_rsqf *cqf)
{
    if (!cqf) return GQF_ERR_ARG;
    if (cqf->blocks) GQF_CK(cudaFree(cqf->blocks));
    cqf->blocks = nullptr;
    return GQF_OK;
}

static bool rsqf_ok(const gqf_rsqf *c)
{
    return c && c->blocks && rsqf_q_ok(c->qbits) && c->numBlocks == GQF_RSQF_API(num_blocks)(c->qbits);
}

int GQF_RSQF_API(lookup_unsorted)(const gqf_rsqf *cqf, int n, const uint32_t *d_keys, int32_t *d_out, void *stream,
                             float *ms)
{
    if (!rsqf_ok(cqf) || n < 0 || (n > 0 && (!d_keys || !d_out))) return GQF_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Arena &ar = arena(current_device(), s);
    std::lock_guard<std::mutex> lk(ar.mu);
    int st = call_begin(ar, s, ms != nullptr);
    if (st) return st;
    if (n > 0) {
        RsqfView v{static_cast<const uint8_t *>(cqf->blocks), cqf->numBlocks};
        const DeviceInfo &di = device_info(current_device());
        uint32_t grid = std::min<uint32_t>((n + RSQF_LOOKUP_THREADS - 1) / RSQF_LOOKUP_THREADS, di.sms * 32);
        k_rsqf_lookup_unsorted<<<grid, RSQF_LOOKUP_THREADS, 0, s>>>(d_keys, (uint32_t)n, v, cqf->qbits, d_out);
        count_launches(1);
    }
    return call_end(ar, s, ms);
}

// Hash + exact bucketing of a batch into (items, optional idx, base, cnt).
static int rsqf_bucket(const uint32_t *keys, uint32_t n, const BucketGeom &g, uint32_t *items, uint32_t *idx,
                       uint32_t *cnt, uint32_t *base, uint32_t *err, cudaStream_t s)
{
    GQF_CK(cudaMemsetAsync(cnt, 0, g.nb * 4, s));
    const uint32_t hchunk = SCATTER_THREADS * SCATTER_IPT;
    GQF_CK(set_smem(k_bucket_hist<SCATTER_THREADS, SCATTER_IPT>, g.nb * 4));
    k_bucket_hist<SCATTER_THREADS, SCATTER_IPT><<<(n + hchunk - 1) / hchunk, SCATTER_THREADS, g.nb * 4, s>>>(
        keys, n, g, cnt);
    k_rsqf_scan_bases<<<1, 1024, 0, s>>>(cnt, g.nb, base);
    GQF_CK(cudaMemsetAsync(cnt, 0, g.nb * 4, s));
    if (idx) {
        auto kfn = k_hash_bucket<PAIR_THREADS, PAIR_IPT, true>;
        size_t sm = (size_t)2 * PAIR_THREADS * PAIR_IPT * 4 + (size_t)g.nb * 8;
        GQF_CK(set_smem(kfn, sm));
        const uint32_t chunk = PAIR_THREADS * PAIR_IPT;
        kfn<<<(n + chunk - 1) / chunk, PAIR_THREADS, sm, s>>>(keys, n, g, base, 0xFFFFFFFFu, cnt, items, idx, err);
    } else {
        auto kfn = k_hash_bucket<SCATTER_THREADS, SCATTER_IPT, false>;
        size_t sm = (size_t)SCATTER_THREADS * SCATTER_IPT * 4 + (size_t)g.nb * 8;
        GQF_CK(set_smem(kfn, sm));
        kfn<<<(n + hchunk - 1) / hchunk, SCATTER_THREADS, sm, s>>>(keys, n, g, base, 0xFFFFFFFFu, cnt, items,
                                                                   nullptr, err);
    }
    count_launches(3);
    GQF_CK(cudaGetLastError());
    return GQF_OK;
}

int GQF_RSQF_API(lookup_sorted)(const gqf_rsqf *cqf, int n, const uint32_t *d_keys, int32_t *d_out, void *stream,
                           float *ms)
{
    if (!rsqf_ok(cqf) || n < 0 || (n > 0 && (!d_keys || !d_out))) return GQF_ERR_ARG;
    // Results go to the queries' input positions either way.  A batch of at
    // least one query per 16 slots is answered faster by direct probes (a
    // lookup is a rank and a select inside one or two blocks) than by grouping
    // the queries by block first.
    if ((uint64_t)n * 16 >= (uint64_t)cqf->numBlocks * 64)
        return GQF_RSQF_API(lookup_unsorted)(cqf, n, d_keys, d_out, stream, ms);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const BucketGeom g = rsqf_geom(cqf->qbits, (uint64_t)n);
    Arena &ar = arena(current_device(), s);
    std::lock_guard<std::mutex> lk(ar.mu);
    Sizer z;
    z.take<uint32_t>(g.nb);
    z.take<uint32_t>(g.nb + 1);
    z.take<uint32_t>(std::max(n, 1));
    z.take<uint32_t>(std::max(n, 1));
    void *basep = arena_reserve(ar, z.off);
    if (!basep) return GQF_ERR_NOMEM;
    Carver c(basep);
    uint32_t *cnt = c.take<uint32_t>(g.nb), *base = c.take<uint32_t>(g.nb + 1);
    uint32_t *items = c.take<uint32_t>(std::max(n, 1)), *idx = c.take<uint32_t>(std::max(n, 1));
    int st = call_begin(ar, s, ms != nullptr);
    if (st) return st;
    if (n > 0) {
        st = rsqf_bucket(d_keys, (uint32_t)n, g, items, idx, cnt, base, ar.err, s);
        if (st) return st;
        RsqfView v{static_cast<const uint8_t *>(cqf->blocks), cqf->numBlocks};
        k_rsqf_lookup_bucketed<<<g.nb, RSQF_LOOKUP_THREADS, 0, s>>>(items, idx, base, cnt, v, cqf->qbits, d_out);
        count_launches(1);
    }
    return call_end(ar, s, ms);
}

// insertGPU (RSQF.cu:882-988): the batch is hashed and sorted, then applied
// in ascending order with the reference's sequential insert semantics.
//  * Empty filter: blocks written from the canonical positions
//    (k_rsqf_positions, k_rsqf_assemble); clusters holding a block whose
//    offset exceeds 62 are then replayed exactly (see rsqf_build.cuh).
//  * Non-empty filter (or a batch past capacity): groups of blocks split at
//    estimated pending-shift boundaries are replayed in parallel
//    (k_rsqf_round); a group whose writes leave it is merged with its
//    successor and replayed from the pre-batch table until none does.
// Return slots are indexed by sorted position, as the reference's are.
// sus / fpos: a build into an empty filter (replays start after the
// canonical prefix of each group); null for incremental batches.
static int rsqf_replay_rounds(uint8_t *t, const uint8_t *t0, uint32_t nbl, uint32_t q, const uint32_t *items,
                              const uint32_t *fhome, uint8_t *start, uint8_t *active, uint8_t *crossed,
                              uint32_t *wlist, uint32_t *blist, uint32_t *ctr, int32_t *d_ret, bool t0_zero,
                              cudaStream_t s, const uint8_t *sus = nullptr, const uint32_t *fpos = nullptr)
{
    const DeviceInfo &di = device_info(current_device());
    const uint32_t grid = std::min<uint32_t>((nbl + 1 + 255) / 256, di.sms * 8);
    for (int round = 0;; round++) {
        GQF_CK(cudaMemsetAsync(ctr, 0, 4 * sizeof(uint32_t), s));  // three list sizes, crossed
        k_rsqf_groups<<<grid, 256, 0, s>>>(nbl, start, active, fhome, wlist, wlist + 2 * (size_t)(nbl + 1), blist,
                                           ctr);
        k_rsqf_round_warp<RSQF_SMALL_GROUP, 8><<<di.sms * 8, 256, 0, s>>>(t, t0, nbl, q, items, fhome, wlist, ctr,
                                                                        crossed, ctr + 3, d_ret, t0_zero ? 1 : 0, sus, fpos);
        k_rsqf_round_warp<RSQF_WARP_GROUP_MAX, 1><<<di.sms * 16, 32, 0, s>>>(
            t, t0, nbl, q, items, fhome, wlist + 2 * (size_t)(nbl + 1), ctr + 1, crossed, ctr + 3, d_ret,
            t0_zero ? 1 : 0, sus, fpos);
        k_rsqf_round_big<<<std::max(1, di.sms), 64, 0, s>>>(t, t0, nbl, q, items, fhome, blist, ctr, crossed,
                                                             ctr + 3, d_ret, t0_zero ? 1 : 0, sus, fpos);
        count_launches(4);
        uint32_t h_n = 0;
        GQF_CK(cudaMemcpyAsync(&h_n, ctr + 3, 4, cudaMemcpyDeviceToHost, s));
        GQF_CK(cudaStreamSynchronize(s));
        if (h_n == 0) return GQF_OK;
        if (round > 100000) return GQF_ERR_TIMEOUT;
        k_rsqf_merge<<<grid, 256, 0, s>>>(nbl, start, active, crossed);
        count_launches(1);
    }
}

int GQF_RSQF_API(insert)(const gqf_rsqf *cqf, int n, const uint32_t *d_keys, int32_t *d_ret, void *stream, float *ms)
{
    if (!rsqf_ok(cqf) || n < 0 || (n > 0 && (!d_keys || !d_ret))) return GQF_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t q = cqf->qbits, nbl = cqf->numBlocks;
    const BucketGeom g = rsqf_geom(q, (uint64_t)n);
    const size_t tbytes = rsqf_table_bytes(nbl);
    const uint32_t ntiles = (nbl + 1 + PEND_TILE - 1) / PEND_TILE;
    uint8_t *table = static_cast<uint8_t *>(cqf->blocks);
    Arena &ar = arena(current_device(), s);
    std::lock_guard<std::mutex> lk(ar.mu);
    Sizer z;
    z.take<uint32_t>(g.nb);
    z.take<uint32_t>(g.nb + 1);
    z.take<uint32_t>(std::max(n, 1));
    z.take<int32_t>(g.nb);
    z.take<int32_t>(g.nb);
    z.take<uint32_t>(nbl + 1);
    z.take<uint32_t>(nbl + 1);
    z.take<uint8_t>(tbytes);
    for (int k = 0; k < 4; k++) z.take<uint8_t>(nbl + 1);
    z.take<PendFn>(nbl + 1);
    z.take<PendFn>(ntiles);
    z.take<uint32_t>(RCTL_WORDS);
    z.take<uint32_t>(4);
    z.take<uint32_t>(4 * (size_t)(nbl + 1));
    z.take<uint32_t>(2 * (size_t)(nbl + 1));
    void *basep = arena_reserve(ar, z.off);
    if (!basep) return GQF_ERR_NOMEM;
    Carver c(basep);
    uint32_t *cnt = c.take<uint32_t>(g.nb), *base = c.take<uint32_t>(g.nb + 1);
    uint32_t *items = c.take<uint32_t>(std::max(n, 1));
    int32_t *bmax = c.take<int32_t>(g.nb), *bpre = c.take<int32_t>(g.nb);
    uint32_t *fpos = c.take<uint32_t>(nbl + 1), *fhome = c.take<uint32_t>(nbl + 1);
    uint8_t *t0 = c.take<uint8_t>(tbytes);
    uint8_t *start = c.take<uint8_t>(nbl + 1), *active = c.take<uint8_t>(nbl + 1), *crossed = c.take<uint8_t>(nbl + 1),
            *sus = c.take<uint8_t>(nbl + 1);
    PendFn *fn = c.take<PendFn>(nbl + 1), *tile_fn = c.take<PendFn>(ntiles);
    uint32_t *ctl = c.take<uint32_t>(RCTL_WORDS), *ctr = c.take<uint32_t>(4);
    uint32_t *wlist = c.take<uint32_t>(4 * (size_t)(nbl + 1)), *blist = c.take<uint32_t>(2 * (size_t)(nbl + 1));
    int st = call_begin(ar, s, true);
    if (st) return st;
    if (n > 0) {
        const DeviceInfo &di = device_info(current_device());
        GQF_CK(cudaMemsetAsync(ctl, 0, RCTL_WORDS * 4, s));
        k_rsqf_nonzero<<<di.sms * 4, 512, 0, s>>>(table, (size_t)(nbl + 1) * RSQF_BB, ctl);
        count_launches(1);
        st = rsqf_bucket(d_keys, (uint32_t)n, g, items, nullptr, cnt, base, ar.err, s);
        if (st) return st;
        // per-bucket sort: capacity from the largest bucket the smem allows
        size_t maxsm = (size_t)(di.smem_optin > 0 ? di.smem_optin : 99 * 1024) - 2048;
        size_t fixed = sort_smem_bytes(g.tb, 0);
        uint32_t cap = maxsm > fixed ? (uint32_t)std::min<size_t>((maxsm - fixed) / 4, 65535) : 0;
        size_t sm = sort_smem_bytes(g.tb, cap);
        GQF_CK(set_smem(k_bucket_sort, sm));
        k_bucket_sort<<<g.nb, SORT_THREADS, sm, s>>>(items, base, cnt, g.tb, cap, ar.err, bmax);
        k_rsqf_scan_max<<<1, 1024, 0, s>>>(bmax, g.nb, bpre);
        k_rsqf_positions<<<g.nb, RPOS_THREADS, 0, s>>>(items, (uint32_t)n, base, cnt, bpre, nbl, nbl * RSQF_SPB,
                                                       d_ret, fpos, fhome, ctl, ar.err);
        const uint32_t agrid = std::min<uint32_t>((nbl + 1 + 7) / 8, di.sms * 64);
        k_rsqf_assemble<<<agrid, 256, 0, s>>>(table, items, d_ret, (uint32_t)n, nbl, fpos, fhome, start, sus, ctl, ar.err);
        count_launches(4);
        GQF_CK(cudaGetLastError());
        uint32_t h_ctl[RCTL_WORDS], h_err = 0;
        GQF_CK(cudaMemcpyAsync(h_ctl, ctl, sizeof h_ctl, cudaMemcpyDeviceToHost, s));
        GQF_CK(cudaMemcpyAsync(&h_err, ar.err, sizeof h_err, cudaMemcpyDeviceToHost, s));
        GQF_CK(cudaStreamSynchronize(s));
        if (h_err) return dev_err_to_status(h_err);
        const uint32_t grid = std::min<uint32_t>((nbl + 1 + 255) / 256, di.sms * 16);
        if (!h_ctl[RCTL_NONEMPTY] && !h_ctl[RCTL_OVER]) {
            if (h_ctl[RCTL_NSUS]) {
                // replay the clusters the canonical positions do not describe,
                // each from its empty blocks
                GQF_CK(cudaMemsetAsync(t0, 0, tbytes, s));
                GQF_CK(cudaMemsetAsync(active, 0, nbl + 1, s));
                GQF_CK(cudaMemsetAsync(crossed, 0, nbl + 1, s));
                k_rsqf_mark_sus<<<grid, 256, 0, s>>>(nbl, start, sus, active);
                count_launches(1);
                st = rsqf_replay_rounds(table, t0, nbl, q, items, fhome, start, active, crossed, wlist, blist, ctr,
                                        d_ret, true, s, sus, fpos);
                if (st) return st;
            }
        } else {
            GQF_CK(cudaMemcpyAsync(t0, table, tbytes, cudaMemcpyDeviceToDevice, s));
            RsqfView v0{t0, nbl};
            k_pend_reduce<<<ntiles, PEND_THREADS, 0, s>>>(v0, nbl, items, fhome, fn, tile_fn);
            k_pend_scan_tiles<<<1, 32, 0, s>>>(tile_fn, ntiles);
            k_pend_apply<<<ntiles, PEND_THREADS, 0, s>>>(nbl, fn, tile_fn, start, active, crossed);
            count_launches(3);
            st = rsqf_replay_rounds(table, t0, nbl, q, items, fhome, start, active, crossed, wlist, blist, ctr, d_ret,
                                    false, s);
            if (st) return st;
        }
    }
    return call_end(ar, s, ms ? ms : nullptr);
}

}  // extern "C"
