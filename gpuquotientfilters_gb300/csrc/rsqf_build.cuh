// RSQF batch insert: the parallel parts around the exact replay.
//
// insertGPU (RSQF.cu:882-988) applies a batch in ascending fingerprint order
// with the sequential insert of insertIntoRegions (RSQF.cu:645-875).  Two
// facts make most of that work parallel without changing a byte of the
// result:
//
//  * Into an empty filter, ascending-order inserts never move an earlier
//    item: item i of the sorted batch lands at pos_i = max(quotient_i,
//    pos_{i-1} + 1), and the blocks are a pure function of those positions
//    (occupieds from the quotients, runEnds at the last item of each
//    quotient, offset[B] = items homed below block B stored at or past it).
//    This holds wherever every block's offset stays below 63; where an
//    offset reaches 63 the reference's findFirstUnusedSlot (RSQF.cpp:
//    341-365) starts skipping free slots and the layout departs from the
//    positions.  Those clusters (bounded by blocks of offset 0, which no
//    insert crosses) are replayed exactly; everything else is written
//    directly by k_rsqf_assemble.
//
//  * Into a non-empty filter, an insert shifts items right up to the first
//    free slot, so a block boundary that the batch's pending shifts do not
//    reach splits the batch into independent groups.  k_pend_* estimate
//    those boundaries from the free slots of the pre-batch table (a
//    max-plus scan of "pending shifts" over blocks, two per insert); the
//    replay verifies
//    every group and merges any group whose writes leave it, so the
//    estimate only affects speed, never the result.
#pragma once

#include <climits>

#include "rsqf.cuh"

namespace GQF_RSQF_NS {

// control words of one insert call (device)
enum : uint32_t { RCTL_NONEMPTY = 0, RCTL_OVER = 1, RCTL_NSUS = 2, RCTL_WORDS = 4 };

// ctl[RCTL_NONEMPTY] != 0 when any byte of [t, t + bytes) is non-zero.
// t is a cudaMalloc'd table (16-byte aligned).
__global__ void k_rsqf_nonzero(const uint8_t *__restrict__ t, size_t bytes, uint32_t *ctl)
{
    const size_t n16 = bytes / 16;
    const uint4 *t4 = reinterpret_cast<const uint4 *>(t);
    uint32_t any = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x) {
        const uint4 v = t4[i];
        any |= v.x | v.y | v.z | v.w;
    }
    if (blockIdx.x == 0)
        for (size_t i = n16 * 16 + threadIdx.x; i < bytes; i += blockDim.x) any |= t[i];
    if (__syncthreads_or(any != 0) && threadIdx.x == 0) atomicOr(ctl + RCTL_NONEMPTY, 1u);
}

// Exclusive max-scan of one int32 per thread across the block; `total`
// receives the block's maximum.  s_w holds THREADS/32 + 1 ints.
template <int THREADS>
__device__ __forceinline__ int32_t block_excl_max(int32_t v, int32_t *s_w, int32_t &total)
{
    constexpr int NW = THREADS / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl = max(incl, t);
    }
    int32_t ex = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) ex = INT_MIN;
    if (lane == 31) s_w[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int32_t x = lane < NW ? s_w[lane] : INT_MIN;
        int32_t xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi = max(xi, t);
        }
        int32_t xe = __shfl_up_sync(0xffffffffu, xi, 1);
        if (lane == 0) xe = INT_MIN;
        if (lane < NW) s_w[lane] = xe;
        if (lane == NW - 1) s_w[NW] = xi;
    }
    __syncthreads();
    const int32_t r = max(ex, s_w[wid]);
    total = s_w[NW];
    __syncthreads();
    return r;
}

// Exclusive prefix max over the per-bucket maxima (one CTA, nb <= 4096).
__global__ void __launch_bounds__(1024) k_rsqf_scan_max(const int32_t *__restrict__ bmax, uint32_t nb,
                                                        int32_t *__restrict__ bpre)
{
    __shared__ int32_t s_w[33];
    const uint32_t per = (nb + 1023) / 1024;
    const uint32_t b0 = min(nb, threadIdx.x * per), b1 = min(nb, b0 + per);
    int32_t m = INT_MIN;
    for (uint32_t b = b0; b < b1; b++) m = max(m, bmax[b]);
    int32_t tot;
    int32_t run = block_excl_max<1024>(m, s_w, tot);
    for (uint32_t b = b0; b < b1; b++) {
        bpre[b] = run;
        run = max(run, bmax[b]);
    }
}

// Canonical positions of the sorted batch and the two block indexes.
// One CTA per bucket (buckets hold consecutive ranges of the sorted array):
//   pos[i]   = i + max_{j <= i} (quotient_j - j)   (= max(quotient_i, pos[i-1] + 1))
//   fpos[B]  = first i with pos[i]  >= 64 B      (B in [0, nbl])
//   fhome[B] = first i with quotient_i >= 64 B   (B in [0, nbl])
// ctl[RCTL_OVER] is set when a position reaches cap_slots.
constexpr int RPOS_THREADS = 512;
constexpr int RPOS_IPT = 8;
constexpr uint32_t RPOS_CH = RPOS_THREADS * RPOS_IPT;
__global__ void __launch_bounds__(RPOS_THREADS) k_rsqf_positions(
    const uint32_t *__restrict__ fps, uint32_t n, const uint32_t *__restrict__ base,
    const uint32_t *__restrict__ cnt, const int32_t *__restrict__ bpre, uint32_t nbl, uint32_t cap_slots,
    int32_t *__restrict__ pos, uint32_t *__restrict__ fpos, uint32_t *__restrict__ fhome, uint32_t *ctl,
    const uint32_t *err)
{
    if (*err & DEV_ERR_BUCKET_CAP) return;  // buckets unsorted: the host reports the error
    __shared__ uint32_t s_v[RPOS_CH + RPOS_CH / 32];
    __shared__ int32_t s_w[RPOS_THREADS / 32 + 1];
    __shared__ int64_t s_lastpos;
    auto pad = [](uint32_t i) { return i + (i >> 5); };
    const uint32_t b = blockIdx.x, nbi = cnt[b], b0 = base[b];
    const int tid = threadIdx.x;
    int32_t carry = bpre[b];
    // position of the item before this chunk (-1: none)
    if (tid == 0) s_lastpos = b0 == 0 ? -1 : (int64_t)(b0 - 1) + bpre[b];
    __syncthreads();
    for (uint32_t c0 = 0; c0 < nbi; c0 += RPOS_CH) {
#pragma unroll
        for (int k = 0; k < RPOS_IPT; k++) {
            const uint32_t li = k * RPOS_THREADS + tid;
            s_v[pad(li)] = c0 + li < nbi ? fps[b0 + c0 + li] : 0u;
        }
        __syncthreads();
        int32_t loc[RPOS_IPT];
        uint32_t hb[RPOS_IPT];
        int32_t m = INT_MIN;
#pragma unroll
        for (int k = 0; k < RPOS_IPT; k++) {
            const uint32_t li = tid * RPOS_IPT + k;
            const uint32_t v = s_v[pad(li)];
            hb[k] = (v >> RSQF_R) / RSQF_SPB;
            if (c0 + li < nbi) m = max(m, (int32_t)(v >> RSQF_R) - (int32_t)(b0 + c0 + li));
            loc[k] = m;
        }
        int32_t tot;
        const int32_t ex = max(carry, block_excl_max<RPOS_THREADS>(m, s_w, tot));
        const int64_t prevpos = s_lastpos;  // read before the chunk's positions land
        // previous item's home block for the first item of this thread
        uint32_t li0 = tid * RPOS_IPT;
        int64_t hprev = -1;
        if (b0 + c0 + li0 > 0 && c0 + li0 < nbi) hprev = (int64_t)((fps[b0 + c0 + li0 - 1] >> RSQF_R) / RSQF_SPB);
        __syncthreads();  // everyone has read s_v / s_lastpos
#pragma unroll
        for (int k = 0; k < RPOS_IPT; k++) {
            const uint32_t li = tid * RPOS_IPT + k;
            if (c0 + li < nbi) {
                int64_t p = (int64_t)(b0 + c0 + li) + max(ex, loc[k]);
                if (p >= (int64_t)cap_slots) {
                    atomicOr(ctl + RCTL_OVER, 1u);
                    p = cap_slots;  // clamped; the positions are not used then
                }
                s_v[pad(li)] = (uint32_t)p;
            }
        }
        __syncthreads();
        // block indexes: item i opens blocks (blk(i-1), blk(i)]
#pragma unroll
        for (int k = 0; k < RPOS_IPT; k++) {
            const uint32_t li = tid * RPOS_IPT + k;
            if (c0 + li >= nbi) break;
            const uint32_t i = b0 + c0 + li;
            const int64_t p = s_v[pad(li)];
            const int64_t pp = li ? (int64_t)s_v[pad(li - 1)] : prevpos;
            const int64_t pb = pp < 0 ? -1 : pp / RSQF_SPB;
            for (int64_t B = pb + 1; B <= p / RSQF_SPB && B <= (int64_t)nbl; B++) fpos[B] = i;
            const int64_t hpb = k ? (int64_t)hb[k - 1] : hprev;
            for (int64_t B = hpb + 1; B <= (int64_t)hb[k]; B++) fhome[B] = i;
            if (i + 1 == n) {
                for (int64_t B = p / RSQF_SPB + 1; B <= (int64_t)nbl; B++) fpos[B] = n;
                for (int64_t B = (int64_t)hb[k] + 1; B <= (int64_t)nbl; B++) fhome[B] = n;
            }
        }
        for (int k = 0; k < RPOS_IPT; k++) {
            const uint32_t li = k * RPOS_THREADS + tid;
            if (c0 + li < nbi) pos[b0 + c0 + li] = (int32_t)s_v[pad(li)];
        }
        __syncthreads();
        if (tid == 0) {
            const uint32_t last = min(RPOS_CH, nbi - c0) - 1;
            s_lastpos = s_v[pad(last)];
        }
        carry = max(carry, tot);
        __syncthreads();
    }
}

// Writes every logical block from the canonical positions (warp per block)
// unless the filter was not empty or the batch overflowed.  start[B] marks
// blocks of offset 0 (no insert crosses into them); sus[B] marks blocks
// whose offset exceeds 62, whose clusters are replayed afterwards.
constexpr uint32_t RSQF_MAX_CANON_OFFSET = 62;
__global__ void __launch_bounds__(256) k_rsqf_assemble(uint8_t *__restrict__ t, const uint32_t *__restrict__ fps,
                                                       const int32_t *__restrict__ pos, uint32_t n, uint32_t nbl,
                                                       const uint32_t *__restrict__ fpos,
                                                       const uint32_t *__restrict__ fhome, uint8_t *__restrict__ start,
                                                       uint8_t *__restrict__ sus, uint32_t *ctl, const uint32_t *err)
{
    if ((ctl[RCTL_NONEMPTY] | ctl[RCTL_OVER]) || (*err & DEV_ERR_BUCKET_CAP)) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t B = w0; B <= nbl; B += nw) {
        if (B == nbl) {  // guard block: its own group, never written here
            if (lane == 0) {
                start[B] = 1;
                sus[B] = 0;
            }
            continue;
        }
        const uint32_t s0 = B * RSQF_SPB;
        const uint32_t a = min(fpos[B], n), e = min(fpos[B + 1], n), c = min(fhome[B], n), d = min(fhome[B + 1], n);
        const uint32_t off = c - a;  // items homed below B stored at or past slot s0
        uint64_t occ = 0, re = 0, w[RSQF_R];
#pragma unroll
        for (int k = 0; k < (int)RSQF_R; k++) w[k] = 0;
        for (uint32_t i = c + lane; i < d; i += 32) occ |= 1ull << ((fps[i] >> RSQF_R) % RSQF_SPB);
        for (uint32_t i = a + lane; i < e; i += 32) {
            const uint32_t fp = fps[i];
            const uint32_t s = (uint32_t)pos[i] - s0;
            const bool last = i + 1 == n || (fps[i + 1] >> RSQF_R) != (fp >> RSQF_R);
            if (last) re |= 1ull << s;
            const uint32_t bit = s * RSQF_R, wi = bit >> 6, sh = bit & 63;
            const uint64_t r = fp & RSQF_RMASK;
#pragma unroll
            for (int k = 0; k < (int)RSQF_R; k++) {
                if ((uint32_t)k == wi) w[k] |= r << sh;
                if ((uint32_t)k == wi + 1 && sh + RSQF_R > 64) w[k] |= r >> (64 - sh);
            }
        }
        auto or64 = [](uint64_t x) -> uint64_t {
            const uint32_t lo = __reduce_or_sync(0xffffffffu, (uint32_t)x);
            const uint32_t hi = __reduce_or_sync(0xffffffffu, (uint32_t)(x >> 32));
            return ((uint64_t)hi << 32) | lo;
        };
        occ = or64(occ);
        re = or64(re);
#pragma unroll
        for (int k = 0; k < (int)RSQF_R; k++) w[k] = or64(w[k]);
        uint8_t *blk = t + (size_t)B * RSQF_BB;
        for (uint32_t j = lane; j < RSQF_BB; j += 32) {
            uint8_t v;
            if (j == 0) {
                v = (uint8_t)off;
            } else if (j < 9) {
                v = (uint8_t)(occ >> (8 * (j - 1)));
            } else if (j < 17) {
                v = (uint8_t)(re >> (8 * (j - 9)));
            } else {
                const uint32_t k = j - 17;
                uint64_t x = w[0];
#pragma unroll
                for (int q = 1; q < (int)RSQF_R; q++)
                    if ((k >> 3) == (uint32_t)q) x = w[q];
                v = (uint8_t)(x >> (8 * (k & 7)));
            }
            blk[j] = v;
        }
        if (lane == 0) {
            start[B] = off == 0 ? 1 : 0;
            const bool bad = off > RSQF_MAX_CANON_OFFSET;
            sus[B] = bad ? 1 : 0;
            if (bad) atomicAdd(ctl + RCTL_NSUS, 1u);
        }
    }
}

// Marks for replay the group (run of blocks from a start block) holding
// each flagged block.
__global__ void k_rsqf_mark_sus(uint32_t nbl, const uint8_t *__restrict__ start, const uint8_t *__restrict__ sus,
                                uint8_t *__restrict__ active)
{
    for (uint32_t B = blockIdx.x * blockDim.x + threadIdx.x; B <= nbl; B += gridDim.x * blockDim.x) {
        if (!sus[B]) continue;
        uint32_t g = B;
        while (g > 0 && !start[g]) g--;
        active[g] = 1;
    }
}

// ---------------------------------------------------------------------
// Pending-shift groups for a non-empty filter.
// (d, c) stands for P -> max(c, P + d) with c >= max(0, d): the number of
// shifts still looking for a free slot after a range of slots, given P
// before it.  An insert homed in the range adds one; a free slot absorbs
// one.  Composition (a then b) = (a.d + b.d, max(b.c, a.c + b.d)).
// ---------------------------------------------------------------------
struct PendFn {
    int32_t d, c;
};
__device__ __forceinline__ PendFn pend_compose(PendFn a, PendFn b)
{
    return PendFn{a.d + b.d, max(b.c, a.c + b.d)};
}
__device__ __forceinline__ PendFn pend_shfl_up(PendFn f, int o)
{
    return PendFn{__shfl_up_sync(0xffffffffu, f.d, o), __shfl_up_sync(0xffffffffu, f.c, o)};
}

// Free slots of block B: slots covered neither by spill from earlier blocks
// (the offset byte) nor by a run of the block's own quotients.  An estimate
// for tables the reference's order-sensitive insert left irregular.
__device__ __forceinline__ uint64_t rsqf_free_mask(const RsqfView &v, uint32_t B)
{
    const uint32_t off = v.off(B);
    uint64_t occ = v.occ(B);
    uint64_t ends = v.re(B) & ~lowmask64(off);
    uint64_t used = lowmask64(off);
    int32_t prev_end = (int32_t)off - 1;
    while (occ) {
        const int32_t x = __ffsll((long long)occ) - 1;
        occ &= occ - 1;
        const int32_t st = max(x, prev_end + 1);
        if (st > 63) break;
        if (!ends) {
            used |= ~lowmask64((uint32_t)st);
            break;
        }
        int32_t e = __ffsll((long long)ends) - 1;
        ends &= ends - 1;
        if (e < st) e = st;
        used |= lowmask64((uint32_t)e + 1) & ~lowmask64((uint32_t)st);
        prev_end = e;
    }
    return ~used;
}

__device__ __forceinline__ PendFn rsqf_block_pend(const RsqfView &v, uint32_t B, uint32_t nbl,
                                                  const uint32_t *__restrict__ fps,
                                                  const uint32_t *__restrict__ fhome)
{
    PendFn f{0, 0};
    const uint64_t fr = rsqf_free_mask(v, B);
    uint32_t cur = 0;
    if (B < nbl) {
        const uint32_t i1 = fhome[B + 1];
        for (uint32_t i = fhome[B]; i < i1; i++) {
            const uint32_t hs = (fps[i] >> RSQF_R) % RSQF_SPB;
            if (hs > cur) {
                const int32_t L = __popcll(fr & lowmask64(hs) & ~lowmask64(cur));
                f.d -= L;
                f.c = max(f.c - L, 0);
                cur = hs;
            }
            // each insert is charged two free slots: findFirstUnusedSlot can
            // pass over a free slot (its rank == 0 case), so the estimate
            // leans towards larger groups over extra replay rounds
            f.d += 2;
            f.c += 2;
        }
    }
    const int32_t L = __popcll(fr & ~lowmask64(cur));
    f.d -= L;
    f.c = max(f.c - L, 0);
    return f;
}

constexpr int PEND_THREADS = 256;
constexpr int PEND_BPT = 8;
constexpr uint32_t PEND_TILE = PEND_THREADS * PEND_BPT;

// Ordered (non-commutative) exclusive block scan of PendFn; `total` gets the
// block's composition.  s_w holds THREADS/32 + 1 entries.
template <int THREADS>
__device__ __forceinline__ PendFn block_excl_pend(PendFn v, PendFn *s_w, PendFn &total)
{
    constexpr int NW = THREADS / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    PendFn incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const PendFn p = pend_shfl_up(incl, o);
        if (lane >= o) incl = pend_compose(p, incl);
    }
    PendFn ex = pend_shfl_up(incl, 1);
    if (lane == 0) ex = PendFn{0, 0};
    if (lane == 31) s_w[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        PendFn x = lane < NW ? s_w[lane] : PendFn{0, 0};
        PendFn xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const PendFn p = pend_shfl_up(xi, o);
            if (lane >= o) xi = pend_compose(p, xi);
        }
        PendFn xe = pend_shfl_up(xi, 1);
        if (lane == 0) xe = PendFn{0, 0};
        if (lane < NW) s_w[lane] = xe;
        if (lane == NW - 1) s_w[NW] = xi;
    }
    __syncthreads();
    const PendFn r = pend_compose(s_w[wid], ex);
    total = s_w[NW];
    __syncthreads();
    return r;
}

// Per-block functions (kept in fn) and per-tile compositions.
__global__ void __launch_bounds__(PEND_THREADS) k_pend_reduce(RsqfView v, uint32_t nbl,
                                                              const uint32_t *__restrict__ fps,
                                                              const uint32_t *__restrict__ fhome,
                                                              PendFn *__restrict__ fn, PendFn *__restrict__ tile_fn)
{
    __shared__ PendFn s_w[PEND_THREADS / 32 + 1];
    const uint32_t B0 = blockIdx.x * PEND_TILE + threadIdx.x * PEND_BPT;
    PendFn acc{0, 0};
    for (uint32_t k = 0; k < PEND_BPT; k++) {
        const uint32_t B = B0 + k;
        if (B > nbl) break;
        const PendFn f = rsqf_block_pend(v, B, nbl, fps, fhome);
        fn[B] = f;
        acc = pend_compose(acc, f);
    }
    PendFn tot;
    block_excl_pend<PEND_THREADS>(acc, s_w, tot);
    if (threadIdx.x == 0) tile_fn[blockIdx.x] = tot;
}

// Exclusive composition over the tiles (a few hundred; one thread).
__global__ void k_pend_scan_tiles(PendFn *tile_fn, uint32_t ntiles)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    PendFn acc{0, 0};
    for (uint32_t t = 0; t < ntiles; t++) {
        const PendFn f = tile_fn[t];
        tile_fn[t] = acc;
        acc = pend_compose(acc, f);
    }
}

// start[B] = no shift pending at the start of block B; every group with
// batch items is active for the first replay round.
__global__ void __launch_bounds__(PEND_THREADS) k_pend_apply(uint32_t nbl, const PendFn *__restrict__ fn,
                                                             const PendFn *__restrict__ tile_excl,
                                                             uint8_t *__restrict__ start, uint8_t *__restrict__ active,
                                                             uint8_t *__restrict__ crossed)
{
    __shared__ PendFn s_w[PEND_THREADS / 32 + 1];
    const uint32_t B0 = blockIdx.x * PEND_TILE + threadIdx.x * PEND_BPT;
    PendFn f[PEND_BPT];
    PendFn acc{0, 0};
#pragma unroll
    for (int k = 0; k < PEND_BPT; k++) {
        const uint32_t B = B0 + k;
        f[k] = B <= nbl ? fn[B] : PendFn{0, 0};
        acc = pend_compose(acc, f[k]);
    }
    PendFn tot;
    PendFn pre = pend_compose(tile_excl[blockIdx.x], block_excl_pend<PEND_THREADS>(acc, s_w, tot));
#pragma unroll
    for (int k = 0; k < PEND_BPT; k++) {
        const uint32_t B = B0 + k;
        if (B > nbl) break;
        const uint8_t st = (B == 0 || pre.c == 0) ? 1 : 0;  // shifts pending on entry = pre.c
        start[B] = st;
        active[B] = st;
        crossed[B] = 0;
        pre = pend_compose(pre, f[k]);
    }
}

}  // namespace GQF_RSQF_NS
