// SQF lookups.
//
// The reference (hashAndLookUp, quotientFilter.cu:320-357, with
// findRunStartGPU :172-196) walks bytes one dependent load at a time: back
// to the cluster start while `shifted`, then forward counting runs, then
// through the run.  Here one thread answers one query from 8-slot words:
// each 8-byte load yields the occupied / continuation / shifted / non-empty
// masks of 8 slots (SWAR pack), the walk back to the cluster start
// accumulates D = #occupied - #run-starts in [cluster start, fq), and the
// query's run is the (D+1)-th run start at or after fq (runs are stored in
// quotient order, one per occupied quotient).  The run is then scanned in
// registers.  Result: the slot of the first element of the run whose
// remainder equals fr, or NOT_FOUND -- the reference's return value.
#pragma once

#include "qf_device.cuh"

namespace gqf {

struct TableView {
    const uint8_t *t;
    uint32_t q, r;
    uint32_t nslots;      // (1<<q)*1.1
    uint32_t nbytes;      // table bytes
    uint32_t nwords_full; // 8-byte words fully inside the table
};

QF_HD uint64_t ld_word(const TableView &v, uint32_t w)
{
#ifdef __CUDA_ARCH__
    if (w < v.nwords_full) return __ldg(reinterpret_cast<const unsigned long long *>(v.t) + w);
#else
    if (w < v.nwords_full) return reinterpret_cast<const unsigned long long *>(v.t)[w];
#endif
    uint64_t x = 0;
    for (uint32_t k = 0; k < 8; k++) {
        uint32_t i = w * 8 + k;
        if (i < v.nbytes) x |= (uint64_t)v.t[i] << (8 * k);
    }
    return x;
}

// One query against a table of 1-byte slots (r <= 5), walking 8-slot words
// with every test done on all 8 bytes of a word at once (byte-lane SWAR:
// bit 0 of byte k flags slot k, popcounts count slots, the lowest or highest
// flagged byte finds one).  The walk is the reference's (findRunStartGPU,
// quotientFilter.cu:172-196, and the run scan of hashAndLookUp, :320-357):
//   1. home word of fq: not occupied -> miss;
//   2. back to the last unshifted slot at or below fq (the cluster start or
//      any later slot where no run is pending), counting
//      D = #occupied - #run starts in [that slot, fq);
//   3. forward: fq's run is the (D+1)-th run start at or after fq;
//   4. the run's elements in slot order up to the first remainder >= fr:
//      equal -> its slot, greater or end of run -> miss.
// x = the home word, loaded by the caller so several queries' first loads
// can be in flight together.
QF_HD uint32_t sqf_query_b1(const TableView &v, uint32_t fq, uint32_t fr, uint64_t x)
{
    constexpr uint64_t OCC = 0x0404040404040404ull;  // occupied bit of every byte
    const uint32_t w = fq >> 3, k = fq & 7u;
    const uint32_t half = k < 4 ? (uint32_t)x : (uint32_t)(x >> 32);
    if (!((half >> (8 * (k & 3u) + 2)) & 1u)) return GQF_NOT_FOUND;
    const uint64_t below = bytes_below(k);
    const uint64_t rs = bl_run_starts(x);
    const uint64_t st = bl_unshifted(x) & bytes_below(k + 1);
    int D;
    if (st) {
        const uint64_t R = below & ~bytes_below(highest_byte(st));
        D = popc64(x & OCC & R) - popc64(rs & R);
    } else {
        D = popc64(x & OCC & below) - popc64(rs & below);
        for (int ww = (int)w - 1; ww >= 0; ww--) {
            const uint64_t y = ld_word(v, (uint32_t)ww);
            const uint64_t s2 = bl_unshifted(y);
            const uint64_t o2 = y & OCC, r2 = bl_run_starts(y);
            if (s2) {
                const uint64_t R = ~bytes_below(highest_byte(s2));
                D += popc64(o2 & R) - popc64(r2 & R);
                break;
            }
            D += popc64(o2) - popc64(r2);
        }
    }
    const uint32_t nwords = (v.nslots + 7) >> 3;
    uint64_t rsm = rs & ~below;
    uint32_t ws = w;
    for (;;) {
        const int c = popc64(rsm);
        if (c > D) break;
        D -= c;
        if (++ws >= nwords) return GQF_NOT_FOUND;
        x = ld_word(v, ws);
        rsm = bl_run_starts(x);
    }
    // byte b of rsm * BL_LO = number of run starts in bytes [0, b]; the
    // first byte where it exceeds D holds the (D+1)-th
    uint32_t j = lowest_byte((((rsm * BL_LO) | BL_HI) - (uint64_t)(D + 1) * BL_LO) & BL_HI);
    uint32_t ef = j + 1;  // first byte that may end the run
    const uint64_t frl = (uint64_t)fr * BL_LO;
    for (;;) {
        // bit 7 of byte b: remainder of slot b >= fr
        const uint64_t ge = ((((x >> 3) & 0x1F1F1F1F1F1F1F1Full) | BL_HI) - frl) & BL_HI;
        const uint64_t ends = (~x >> 1) & BL_LO & ~bytes_below(ef);  // not a continuation
        const uint32_t e = ends ? lowest_byte(ends) : 8u;
        const uint64_t m = ge & bytes_below(e) & ~bytes_below(j);
        if (m) {
            const uint32_t b = lowest_byte(m);
            return (((uint32_t)(x >> (8 * b + 3)) & 0x1Fu) == fr) ? ws * 8 + b : GQF_NOT_FOUND;
        }
        if (e < 8 || ++ws >= nwords) return GQF_NOT_FOUND;
        x = ld_word(v, ws);
        j = 0;
        ef = 0;
    }
}

// Generic slot walk for multi-byte slots (r = 13: 2-byte big-endian).
template <int BPE>
__device__ __forceinline__ uint32_t sqf_get(const TableView &v, uint32_t i)
{
    if (i >= v.nslots) return 0;
    const uint8_t *p = v.t + (size_t)i * BPE;
    uint32_t e = p[0];
    for (int k = 1; k < BPE; k++) e = (e << 8) | p[k];
    return e;
}

template <int BPE>
__device__ __forceinline__ uint32_t sqf_query_generic(const TableView &v, uint32_t fq, uint32_t fr)
{
    if (!e_occ(sqf_get<BPE>(v, fq))) return GQF_NOT_FOUND;
    uint32_t b = fq;
    while (e_shift(sqf_get<BPE>(v, b)) && b > 0) b--;
    uint32_t s = b;
    while (b != fq) {
        do { s++; } while (e_cont(sqf_get<BPE>(v, s)) && s < v.nslots);
        do { b++; } while (!e_occ(sqf_get<BPE>(v, b)) && b < v.nslots);
    }
    do {
        uint32_t rem = sqf_get<BPE>(v, s) >> 3;
        if (rem == fr) return s;
        if (rem > fr) return GQF_NOT_FOUND;
        s++;
    } while (e_cont(sqf_get<BPE>(v, s)));
    return GQF_NOT_FOUND;
}

template <int BPE>
__device__ __forceinline__ uint32_t sqf_query(const TableView &v, uint32_t fp)
{
    uint32_t fq = (fp >> v.r) & ((1u << v.q) - 1u);
    uint32_t fr = fp & ((1u << v.r) - 1u);
    if (BPE == 1) return sqf_query_b1(v, fq, fr, ld_word(v, fq >> 3));
    return sqf_query_generic<BPE>(v, fq, fr);
}

// Queries per thread in flight in the lookup kernels.
constexpr int LOOKUP_QPT = 4;
constexpr int LOOKUP_THREADS = 256;

// QPT queries of one thread: keys loaded together, first table words
// loaded together, then each walk finishes (rarely needing more words).
template <int BPE>
__device__ __forceinline__ void sqf_query_batch(const TableView &v, const uint32_t (&fp)[LOOKUP_QPT],
                                                const bool (&valid)[LOOKUP_QPT], uint32_t (&res)[LOOKUP_QPT])
{
    if (BPE == 1) {
        uint64_t x[LOOKUP_QPT];
#pragma unroll
        for (int k = 0; k < LOOKUP_QPT; k++) {
            uint32_t fq = (fp[k] >> v.r) & ((1u << v.q) - 1u);
            x[k] = valid[k] ? ld_word(v, fq >> 3) : 0ull;
        }
#pragma unroll
        for (int k = 0; k < LOOKUP_QPT; k++) {
            uint32_t fq = (fp[k] >> v.r) & ((1u << v.q) - 1u);
            uint32_t fr = fp[k] & ((1u << v.r) - 1u);
            res[k] = valid[k] ? sqf_query_b1(v, fq, fr, x[k]) : GQF_NOT_FOUND;
        }
    } else {
#pragma unroll
        for (int k = 0; k < LOOKUP_QPT; k++) res[k] = valid[k] ? sqf_query<BPE>(v, fp[k]) : GQF_NOT_FOUND;
    }
}

// launchUnsortedLookups: QPT queries per thread, coalesced keys.
template <int BPE, int QPT>
__global__ void __launch_bounds__(LOOKUP_THREADS) k_lookup_unsorted(const uint32_t *__restrict__ keys, uint32_t n,
                                                                   TableView v, uint32_t *__restrict__ out)
{
    const uint32_t fpmask = (v.q + v.r >= 32) ? 0xFFFFFFFFu : ((1u << (v.q + v.r)) - 1u);
    const uint32_t qmask = (1u << v.q) - 1u, rmask = (1u << v.r) - 1u;
    const uint32_t per_block = LOOKUP_THREADS * QPT;
    for (uint64_t b0 = (uint64_t)blockIdx.x * per_block; b0 < n; b0 += (uint64_t)gridDim.x * per_block) {
        uint32_t fp[QPT];
        bool valid[QPT];
#pragma unroll
        for (int k = 0; k < QPT; k++) {
            const uint64_t i = b0 + (uint64_t)k * LOOKUP_THREADS + threadIdx.x;
            valid[k] = i < n;
            fp[k] = valid[k] ? __ldg(keys + i) : 0u;
        }
        uint64_t x[QPT];
#pragma unroll
        for (int k = 0; k < QPT; k++) {
            fp[k] = aphash32(fp[k]) & fpmask;
            x[k] = (BPE == 1 && valid[k]) ? ld_word(v, ((fp[k] >> v.r) & qmask) >> 3) : 0ull;
        }
#pragma unroll
        for (int k = 0; k < QPT; k++) {
            if (!valid[k]) continue;
            const uint32_t res = BPE == 1 ? sqf_query_b1(v, (fp[k] >> v.r) & qmask, fp[k] & rmask, x[k])
                                          : sqf_query<BPE>(v, fp[k]);
            out[b0 + (uint64_t)k * LOOKUP_THREADS + threadIdx.x] = res;
        }
    }
}

}  // namespace gqf

#include "sqf_build.cuh"

namespace gqf {

// launchSortedLookups: queries arrive grouped by table region (bucket b
// holds the queries whose quotient lies in [b*2^tb, (b+1)*2^tb)), so one
// CTA's probes stay inside one ~2^tb-byte stretch of the table; results go
// straight to their input positions (the reference sorts them back by
// index instead, quotientFilter.cu:304-305).
template <int BPE>
__global__ void __launch_bounds__(LOOKUP_THREADS) k_lookup_bucketed(BucketSrc src, const uint32_t *__restrict__ idx,
                                                                   TableView v, uint32_t *__restrict__ out)
{
    const uint32_t b = blockIdx.x;
    const uint32_t n = src.count(b);
    const size_t base = src.start(b);
    for (uint32_t i0 = 0; i0 < n; i0 += LOOKUP_THREADS * LOOKUP_QPT) {
        uint32_t fp[LOOKUP_QPT], id[LOOKUP_QPT], res[LOOKUP_QPT];
        bool valid[LOOKUP_QPT];
#pragma unroll
        for (int k = 0; k < LOOKUP_QPT; k++) {
            uint32_t i = i0 + k * LOOKUP_THREADS + threadIdx.x;
            valid[k] = i < n;
            fp[k] = valid[k] ? src.items[base + i] : 0u;
            id[k] = valid[k] ? idx[base + i] : 0u;
        }
        sqf_query_batch<BPE>(v, fp, valid, res);
#pragma unroll
        for (int k = 0; k < LOOKUP_QPT; k++)
            if (valid[k]) out[id[k]] = res[k];
    }
}

// ---------------------------------------------------------------------------
// Sorted lookups, one-byte slots, from a shared-memory image of the bucket.
// A bucket's queries all have quotients in [x0, x0 + 2^tb).  The CTA stages
// the table slice [x0, x0 + 2^tb + LKS_MARGIN) once, and indexes it once:
// per 8-slot word the occupied mask and the occupied count before it, and
// the list of run starts in slot order.  Runs are stored in quotient order,
// one per occupied quotient, so the run of the j-th occupied quotient at or
// past x0 is run start number D0 + j, where D0 counts the runs of quotients
// below x0 still pending at x0 (the walk-back of sqf_query_b1 for slot x0,
// done once per bucket).  A query then costs a few shared-memory reads and a
// short scan of its run; a run starting or ending outside the staged slice
// falls back to sqf_query_b1 on the table.  Results equal sqf_query_b1's on
// every valid table.
// ---------------------------------------------------------------------------
constexpr int LKS_THREADS = 256;
constexpr uint32_t LKS_MARGIN = 2048;

__host__ __device__ inline size_t lks_smem_bytes(uint32_t tb)
{
    const size_t L = ((size_t)1 << tb) + LKS_MARGIN;  // slots staged
    const size_t W = L / 8;                            // 8-slot words
    return L + 2 * W + W + 2 * L + 64;                 // bytes, occupied prefix, masks, run starts
}

static __global__ void __launch_bounds__(LKS_THREADS) k_lookup_bucketed_s(BucketSrc src, const uint32_t *__restrict__ idx,
                                                                  TableView v, uint32_t tb,
                                                                  uint32_t *__restrict__ out)
{
    extern __shared__ __align__(16) uint8_t smem_lks[];
    const uint32_t S = 1u << tb, L = S + LKS_MARGIN, W = L / 8;
    uint8_t *s_tab = smem_lks;
    uint16_t *s_occp = reinterpret_cast<uint16_t *>(s_tab + L);
    uint8_t *s_occ8 = reinterpret_cast<uint8_t *>(s_occp + W);
    uint16_t *s_rs = reinterpret_cast<uint16_t *>(s_occ8 + ((W + 1) & ~1u));
    __shared__ uint32_t s_wsum[2][LKS_THREADS / 32];
    __shared__ int s_D0;
    __shared__ uint32_t s_nrs;
    const uint32_t b = blockIdx.x, n = src.count(b);
    if (n == 0) return;
    const size_t base = src.start(b);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t x0 = b << tb;
    // stage slots [x0, x0 + L), zero past the table
    for (uint32_t i = tid * 16; i < L; i += LKS_THREADS * 16) {
        uint4 w4;
        if ((size_t)x0 + i + 16 <= v.nbytes) {
            w4 = __ldg(reinterpret_cast<const uint4 *>(v.t + x0 + i));
        } else {
            uint8_t tmp[16];
#pragma unroll
            for (int k = 0; k < 16; k++) tmp[k] = (size_t)x0 + i + k < v.nbytes ? v.t[x0 + i + k] : 0;
            w4 = *reinterpret_cast<uint4 *>(tmp);
        }
        *reinterpret_cast<uint4 *>(s_tab + i) = w4;
    }
    if (wid == 0) {
        // runs of quotients below x0 still pending at x0
        const int D = pending_runs_warp(v.t, x0);
        if (lane == 0) s_D0 = D;
    }
    __syncthreads();
    // index: this thread's words [w0, w1)
    const uint32_t per = (W + LKS_THREADS - 1) / LKS_THREADS;
    const uint32_t w0 = min(W, tid * per), w1 = min(W, w0 + per);
    uint32_t nocc = 0, nrs = 0;
    for (uint32_t w = w0; w < w1; w++) {
        const Flags8 f = flags8(*reinterpret_cast<const uint64_t *>(s_tab + 8 * w));
        nocc += popc32(f.occ);
        nrs += popc32(f.nonempty & ~f.cont);
    }
    uint32_t io = nocc, ir = nrs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t a = __shfl_up_sync(0xffffffffu, io, o), c = __shfl_up_sync(0xffffffffu, ir, o);
        if (lane >= o) {
            io += a;
            ir += c;
        }
    }
    if (lane == 31) {
        s_wsum[0][wid] = io;
        s_wsum[1][wid] = ir;
    }
    __syncthreads();
    uint32_t po = io - nocc, pr = ir - nrs;
    for (int w = 0; w < wid; w++) {
        po += s_wsum[0][w];
        pr += s_wsum[1][w];
    }
    if (tid == LKS_THREADS - 1) s_nrs = pr + nrs;
    for (uint32_t w = w0; w < w1; w++) {
        const Flags8 f = flags8(*reinterpret_cast<const uint64_t *>(s_tab + 8 * w));
        s_occp[w] = (uint16_t)po;
        s_occ8[w] = (uint8_t)f.occ;
        po += popc32(f.occ);
        for (uint32_t m = f.nonempty & ~f.cont & 0xFFu; m; m &= m - 1u) s_rs[pr++] = (uint16_t)(8 * w + lowest_bit(m));
    }
    __syncthreads();
    const int D0 = s_D0;
    const uint32_t nrs_all = s_nrs;
    const uint32_t qmask = (1u << v.q) - 1u, rmask = (1u << v.r) - 1u;
    for (uint32_t i = tid; i < n; i += LKS_THREADS) {
        const uint32_t fp = src.items[base + i], qi = idx[base + i];
        const uint32_t fq = (fp >> v.r) & qmask, fr = fp & rmask;
        const uint32_t lq = fq - x0, w = lq >> 3, k = lq & 7u;
        const uint32_t m8 = s_occ8[w];
        uint32_t res = GQF_NOT_FOUND;
        if ((m8 >> k) & 1u) {
            const int rk = D0 + (int)s_occp[w] + popc32(m8 & ((1u << k) - 1u));
            bool fallback = rk < 0 || (uint32_t)rk >= nrs_all;
            if (!fallback) {
                uint32_t p = s_rs[rk];
                for (;;) {
                    const uint32_t e = s_tab[p];
                    const uint32_t rem = e >> 3;
                    if (rem == fr) {
                        res = x0 + p;
                        break;
                    }
                    if (rem > fr) break;
                    if (++p >= L) {
                        fallback = true;
                        break;
                    }
                    if (!((s_tab[p] >> 1) & 1u)) break;
                }
            }
            if (fallback) res = sqf_query_b1(v, fq, fr, ld_word(v, fq >> 3));
        }
        out[qi] = res;
    }
}

}  // namespace gqf
