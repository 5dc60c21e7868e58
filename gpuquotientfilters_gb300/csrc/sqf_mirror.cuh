// Unsorted lookups on one-byte slots through a bit-plane mirror of the table.
//
// The reference answers each query by walking slot bytes (hashAndLookUp,
// quotientFilter.cu:320-357, with findRunStartGPU :172-196).  A large batch
// here first transposes the table, once per call, into 32-byte group records
// (k_sqf_mirror), then answers every query from two records with 32-bit mask
// arithmetic (k_lookup_mirror).  The table itself is not changed.
//
// Record of group G (slots [31G, 31G + 31)), eight 32-bit words; bit i of
// words 0..7 describes slot 31G + i:
//   v[0] occupied, v[1] run start (non-empty and not a continuation),
//   v[2] continuation, v[3 + b] bit b of the remainder (b < 5);
//   bit 31 of v[t] = bit t of P(G), the number of runs of quotients below
//   31G that start at or after 31G (255: 255 or more).
// P is the lookup's walk-back count D at the group's first slot.  Along the
// table D(x + 1) = D(x) + occupied(x) - runstart(x): each occupied quotient
// opens one pending run and each run start closes one, runs being stored in
// quotient order.  A record is one 32-byte sector, read with one 256-bit load.
//
// Query fq = 31G + k, remainder fr, from records G and G + 1 (62 slots):
//   not occupied at k -> miss;
//   D = P + #occupied - #run starts in [31G, fq);
//   the window of slots [fq, fq + 32) (a funnel shift of the two records);
//   fq's run is the (D+1)-th run start in the window; it ends before the
//   first later slot that is not a continuation;
//   remainders are compared bit-sliced on all 32 window slots at once:
//   the first slot of the run with remainder >= fr decides (equal: its slot;
//   greater or none before the run ends: miss).
// When the window cannot decide (P saturated, run start or the deciding slot
// past fq + 31) the query falls back to sqf_query_b1 on the table.  Results
// equal sqf_query_b1's, i.e. the reference's, on every table.
#pragma once

#include "sqf_lookup.cuh"
#include "tma.cuh"

namespace gqf {

constexpr uint32_t MIR_SLOTS = 31;                      // slots per group
constexpr uint32_t MIR_WORDS = 31;                      // table words per build thread (8 groups)
constexpr int MIR_BUILD_THREADS = 128;
constexpr uint32_t MIR_TILE = MIR_BUILD_THREADS * MIR_WORDS * 8;  // table bytes per build tile
constexpr uint32_t MIRROR_UNDECIDED = 0xFFFFFFFEu;
constexpr int MIR_LOOKUP_THREADS = 256;

// groups covering nslots; the mirror holds one more, all-zero, record
QF_HD uint32_t mir_groups(uint32_t nslots) { return (nslots + MIR_SLOTS - 1) / MIR_SLOTS; }
QF_HD size_t mir_bytes(uint32_t nslots) { return (size_t)(mir_groups(nslots) + 1) * 32; }

QF_HD uint32_t fshr32(uint32_t lo, uint32_t hi, uint32_t s)  // (hi:lo >> s), s < 32
{
#ifdef __CUDA_ARCH__
    return __funnelshift_r(lo, hi, s);
#else
    return s ? (lo >> s) | (hi << (32 - s)) : lo;
#endif
}

// position of the (j+1)-th set bit of m (m has more than j set bits)
QF_HD uint32_t nth_bit(uint32_t m, int j)
{
#ifdef __CUDA_ARCH__
    return __fns(m, 0, j + 1);
#else
    return (uint32_t)select_bit(m, j);
#endif
}

// Record of group G from the slot bytes (bytes past nbytes read as empty);
// the build kernel's transposition must give exactly this.
QF_HD void mirror_record(const uint8_t *t, uint32_t nbytes, uint32_t G, int P, uint32_t (&v)[8])
{
    for (int w = 0; w < 8; w++) v[w] = 0;
    for (uint32_t i = 0; i < MIR_SLOTS; i++) {
        const size_t s = (size_t)G * MIR_SLOTS + i;
        const uint32_t e = s < nbytes ? t[s] : 0u;
        const uint32_t occ = (e >> 2) & 1u, cont = (e >> 1) & 1u, sh = e & 1u;
        v[0] |= occ << i;
        v[1] |= ((occ | sh) & ~cont & 1u) << i;
        v[2] |= cont << i;
        for (int b = 0; b < 5; b++) v[3 + b] |= ((e >> (3 + b)) & 1u) << i;
    }
    const uint32_t p = (P < 0 || P > 254) ? 255u : (uint32_t)P;
    for (int w = 0; w < 8; w++) v[w] |= ((p >> w) & 1u) << 31;
}

QF_HD uint32_t mirror_P(const uint32_t (&r0)[8])
{
    uint32_t P = 0;
#pragma unroll
    for (int t = 7; t >= 0; t--) P = (P << 1) | (r0[t] >> 31);
    return P;
}

// One query from records G (r0) and G + 1 (r1); k = fq - 31G.
QF_HD uint32_t mirror_query(uint32_t fq, uint32_t fr, uint32_t k, const uint32_t (&r0)[8], const uint32_t (&r1)[8])
{
    if (!((r0[0] >> k) & 1u)) return GQF_NOT_FOUND;
    const uint32_t P = mirror_P(r0);
    if (P >= 255) return MIRROR_UNDECIDED;
    const uint32_t lowk = (1u << k) - 1u;
    const int D = (int)P + popc32(r0[0] & lowk) - popc32(r0[1] & lowk);
    // window slots fq .. fq + 31: record bits k.. of G then bits 0.. of G + 1
    // (bit 31 of each word is P, shifted out by the << 1)
    const uint32_t Sw = fshr32(r0[1] << 1, r1[1], k + 1);
    if (D < 0 || popc32(Sw) <= D) return MIRROR_UNDECIDED;
    const uint32_t s = nth_bit(Sw, D);
    const uint32_t Cw = fshr32(r0[2] << 1, r1[2], k + 1);
    const uint32_t ends = ~Cw & (0xFFFFFFFEu << s);  // slots after s that are not continuations
    const uint32_t e = ends ? (uint32_t)lowest_bit(ends) : 32u;
    const uint32_t run = (e >= 32 ? ~0u : ((1u << e) - 1u)) & ~((1u << s) - 1u);
    // bit-sliced compare of the window's remainders with fr, high bit first
    uint32_t eq = ~0u, gt = 0u;
#pragma unroll
    for (int b = 4; b >= 0; b--) {
        const uint32_t Rw = fshr32(r0[3 + b] << 1, r1[3 + b], k + 1);
        const uint32_t fb = 0u - ((fr >> b) & 1u);
        gt |= eq & Rw & ~fb;
        eq &= ~(Rw ^ fb);
    }
    const uint32_t m = (gt | eq) & run;
    if (!m) return e >= 32 ? MIRROR_UNDECIDED : GQF_NOT_FOUND;
    const uint32_t f = (uint32_t)lowest_bit(m);
    return ((eq >> f) & 1u) ? fq + f : GQF_NOT_FOUND;
}

// 8x8 bit transpose of one table word: byte b of the result holds bit b of
// the 8 slot bytes, slot i at bit i.
QF_HD uint64_t bit_transpose8(uint64_t x)
{
    uint64_t t;
    t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull;
    x = x ^ t ^ (t << 7);
    t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull;
    x = x ^ t ^ (t << 14);
    t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull;
    x = x ^ t ^ (t << 28);
    return x;
}

// byte i of the result = byte (sel >> 4i) & 7 of the 8 bytes b:a (a low)
QF_HD uint32_t byte_perm(uint32_t a, uint32_t b, uint32_t sel)
{
#ifdef __CUDA_ARCH__
    return __byte_perm(a, b, sel);
#else
    const uint64_t ab = (uint64_t)a | ((uint64_t)b << 32);
    uint32_t r = 0;
    for (int i = 0; i < 4; i++) r |= (uint32_t)((ab >> (8 * ((sel >> (4 * i)) & 7u))) & 0xFFu) << (8 * i);
    return r;
#endif
}

// One build thread's 31 table words (248 slots) -> the record words (P bits
// clear) of its 8 groups of 31 slots, and per group #occupied - #run starts.
// Planes come per 32-slot chunk: four 8x8 bit transposes, then a 4x4 byte
// transpose (byte b of plane word t = plane t of word b); group g (bits
// [31g, 31g + 31) of the thread's slots) is cut from the chunk holding its
// first slot and the next.  Gives exactly mirror_record's words.
QF_HD void mirror_groups(const uint64_t *sw, uint32_t (&gp)[8][8], int (&cnt)[8])
{
    uint32_t prev[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int c = 0; c < 8; c++) {
        uint32_t lo[4], hi[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int wi = 4 * c + j;
            const uint64_t y = wi < (int)MIR_WORDS ? bit_transpose8(sw[wi]) : 0ull;
            lo[j] = (uint32_t)y;
            hi[j] = (uint32_t)(y >> 32);
        }
        uint32_t raw[8];  // bit b of the slot bytes: 0 shifted, 1 continuation, 2 occupied, 3.. remainder
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const uint32_t *x = h ? hi : lo;
            const uint32_t ab01 = byte_perm(x[0], x[1], 0x5140), ab23 = byte_perm(x[0], x[1], 0x7362);
            const uint32_t cd01 = byte_perm(x[2], x[3], 0x5140), cd23 = byte_perm(x[2], x[3], 0x7362);
            raw[4 * h + 0] = byte_perm(ab01, cd01, 0x5410);
            raw[4 * h + 1] = byte_perm(ab01, cd01, 0x7632);
            raw[4 * h + 2] = byte_perm(ab23, cd23, 0x5410);
            raw[4 * h + 3] = byte_perm(ab23, cd23, 0x7632);
        }
        uint32_t cur[8];
        cur[0] = raw[2];
        cur[1] = (raw[2] | raw[0]) & ~raw[1];
        cur[2] = raw[1];
#pragma unroll
        for (int b = 0; b < 5; b++) cur[3 + b] = raw[3 + b];
        // group g is complete once the chunk after the one holding its first slot is in
        if (c >= 1) {
#pragma unroll
            for (int g = 0; g < 8; g++) {
                if (((31 * g) >> 5) == c - 1) {
                    const int off = (31 * g) & 31;
#pragma unroll
                    for (int w = 0; w < 8; w++) gp[g][w] = fshr32(prev[w], cur[w], (uint32_t)off) & 0x7FFFFFFFu;
                    cnt[g] = popc32(gp[g][0]) - popc32(gp[g][1]);
                }
            }
        }
#pragma unroll
        for (int w = 0; w < 8; w++) prev[w] = cur[w];
    }
}

#ifdef __CUDACC__
// ---- build ---------------------------------------------------------------

__device__ __forceinline__ uint64_t l2_policy_evict_last()
{
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_first()
{
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
// 32-byte record loads / stores (one sector, 256-bit accesses; 32-byte aligned)
__device__ __forceinline__ void ld_record(const uint4 *rec, uint32_t G, uint64_t pol, uint32_t (&r)[8])
{
    asm volatile("ld.global.nc.L2::cache_hint.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "l"(rec + 2 * (size_t)G), "l"(pol));
}
__device__ __forceinline__ void st_record(uint4 *rec, uint32_t G, uint64_t pol, const uint32_t (&p)[8])
{
    asm volatile("st.global.L2::cache_hint.v8.u32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8}, %9;" ::"l"(rec + 2 * (size_t)G),
                 "r"(p[0]), "r"(p[1]), "r"(p[2]), "r"(p[3]), "r"(p[4]), "r"(p[5]), "r"(p[6]), "r"(p[7]), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ uint32_t ld_stream_u32(const uint32_t *p, uint64_t pol)
{
    uint32_t v;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void st_stream_u32(uint32_t *p, uint32_t v, uint64_t pol)
{
    asm volatile("st.global.L1::no_allocate.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}

// One staged tile (MIR_TILE bytes at st, its first group G0tile, D at its
// first slot Dtile): every thread turns its 31 words (248 slots) into 8
// records.  Returns D after the tile.  Contains one __syncthreads.
__device__ __forceinline__ int mirror_tile(const uint8_t *st, int Dtile, uint32_t G0tile, uint4 *__restrict__ rec,
                                           uint32_t ngroups, int *s_wsum)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint64_t *sw = reinterpret_cast<const uint64_t *>(st) + MIR_WORDS * tid;
    uint32_t gp[8][8];  // [group][record word]
    int cnt[8];
    mirror_groups(sw, gp, cnt);
    int tot = 0;
#pragma unroll
    for (int g = 0; g < 8; g++) tot += cnt[g];
    int incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o) incl += y;
    }
    if (lane == 31) s_wsum[wid] = incl;
    __syncthreads();
    int D = Dtile + incl - tot;
    int all = 0;
#pragma unroll
    for (uint32_t w = 0; w < MIR_BUILD_THREADS / 32; w++) {
        const int x = s_wsum[w];
        if (w < wid) D += x;
        all += x;
    }
    const uint32_t G0 = G0tile + 8 * tid;
    const uint64_t pol = l2_policy_evict_last();  // the lookups read the records next
#pragma unroll
    for (int g = 0; g < 8; g++) {
        const uint32_t P = (D < 0 || D > 254) ? 255u : (uint32_t)D;
        D += cnt[g];
        uint32_t pl[8];
#pragma unroll
        for (int w = 0; w < 8; w++) pl[w] = gp[g][w] | (((P >> w) & 1u) << 31);
        if (G0 + g <= ngroups) st_record(rec, G0 + g, pol, pl);
    }
    return Dtile + all;
}

// Persistent build: CTA b takes a contiguous run of tiles, double-buffered in
// shared memory by 1-D bulk copies (TMA) on two mbarriers; D enters its first
// tile from the walk-back before it and then carries from tile to tile.  The
// table must be 16-byte aligned.  A wait that gives up sets DEV_ERR_TIMEOUT.
static __global__ void __launch_bounds__(MIR_BUILD_THREADS) k_sqf_mirror(TableView v, uint4 *__restrict__ rec,
                                                                        uint32_t ngroups, uint32_t ntiles,
                                                                        uint32_t *__restrict__ err)
{
    extern __shared__ __align__(128) uint8_t mir_smem[];  // 2 * MIR_TILE
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int s_entry;
    __shared__ int s_wsum[MIR_BUILD_THREADS / 32];
    __shared__ uint32_t s_fail;
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t per = ntiles / gridDim.x, extra = ntiles % gridDim.x;
    const uint32_t t0 = blockIdx.x * per + min(blockIdx.x, extra);
    const uint32_t t1 = t0 + per + (blockIdx.x < extra ? 1u : 0u);
    if (t0 >= t1) return;
    // bytes of tile t that one bulk copy brings in (16-byte multiple, inside the table)
    auto copy_bytes = [&](uint32_t t) -> uint32_t {
        const uint64_t a = (uint64_t)t * MIR_TILE;
        if (a >= v.nbytes) return 0u;
        const uint64_t rem = (v.nbytes - a) & ~15ull;
        return rem < MIR_TILE ? (uint32_t)rem : MIR_TILE;
    };
    uint32_t pend = 0;  // thread 0: stages with a copy in flight
    // the table streams through L2 (evict first); the records stay (evict last)
    const uint64_t pass = l2_policy_evict_first();
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
        s_fail = 0;
        for (uint32_t j = 0; j < 2; j++) {
            const uint32_t b = t0 + j < t1 ? copy_bytes(t0 + j) : 0u;
            if (b) {
                mbar_arrive_expect_tx(&bar[j], b);
                bulk_g2s_hint(mir_smem + j * MIR_TILE, v.t + (size_t)(t0 + j) * MIR_TILE, b, &bar[j], pass);
                pend |= 1u << j;
            }
        }
    }
    if (wid == 0) {
        const uint32_t x0 = t0 * MIR_TILE;
        const int D = x0 < v.nslots ? pending_runs_warp(v.t, x0) : 0;
        if (lane == 0) s_entry = D;
    }
    __syncthreads();
    int Dtile = s_entry;
    for (uint32_t t = t0; t < t1; t++) {
        const uint32_t j = (t - t0) & 1u, par = ((t - t0) >> 1) & 1u;
        uint8_t *st = mir_smem + j * MIR_TILE;
        const uint32_t b = copy_bytes(t);
        if (b) {
            if (mbar_wait_bounded(&bar[j], par, SPIN_LIMIT)) {
                if (tid == 0) pend &= ~(1u << j);
            } else {
                s_fail = 1;
            }
        }
        if (b < MIR_TILE) {  // the table's ragged end, then empty slots
            const size_t a = (size_t)t * MIR_TILE;
            for (uint32_t i = b + tid; i < MIR_TILE; i += MIR_BUILD_THREADS) st[i] = a + i < v.nbytes ? v.t[a + i] : 0;
        }
        __syncthreads();
        if (s_fail) break;
        Dtile = mirror_tile(st, Dtile, t * (MIR_TILE / MIR_SLOTS), rec, ngroups, s_wsum);
        __syncthreads();  // the stage is free again
        if (tid == 0 && t + 2 < t1) {
            const uint32_t b2 = copy_bytes(t + 2);
            if (b2) {
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&bar[j], b2);
                bulk_g2s_hint(st, v.t + (size_t)(t + 2) * MIR_TILE, b2, &bar[j], pass);
                pend |= 1u << j;
            }
        }
    }
    if (tid == 0 && s_fail) {
        atomicOr(err, DEV_ERR_TIMEOUT);
        // no copy may still be writing this CTA's shared memory when it exits
        for (uint32_t j = 0; j < 2; j++)
            if (pend & (1u << j))
                for (uint32_t par = 0; par < 2; par++) mbar_wait_bounded(&bar[j], par, SPIN_LIMIT);
    }
}

// ---- lookups ---------------------------------------------------------------
// One query per thread per grid-stride step; the next step's key is loaded
// while this one's records are in flight.  Keys and results stream past L2
// (evict first); the records stay (evict last).
static __global__ void __launch_bounds__(MIR_LOOKUP_THREADS) k_lookup_mirror(const uint32_t *__restrict__ keys,
                                                                            uint32_t n, TableView v,
                                                                            const uint4 *__restrict__ rec,
                                                                            uint32_t *__restrict__ out)
{
    const uint32_t fpmask = (v.q + v.r >= 32) ? 0xFFFFFFFFu : ((1u << (v.q + v.r)) - 1u);
    const uint32_t qmask = (1u << v.q) - 1u, rmask = (1u << v.r) - 1u;
    const uint64_t keep = l2_policy_evict_last(), pass = l2_policy_evict_first();
    const uint64_t stride = (uint64_t)gridDim.x * MIR_LOOKUP_THREADS;
    uint64_t i = (uint64_t)blockIdx.x * MIR_LOOKUP_THREADS + threadIdx.x;
    uint32_t key = i < n ? ld_stream_u32(keys + i, pass) : 0u;
    for (; i < n; i += stride) {
        const uint32_t knext = i + stride < n ? ld_stream_u32(keys + i + stride, pass) : 0u;
        const uint32_t fp = aphash32(key) & fpmask;
        const uint32_t fq = (fp >> v.r) & qmask, fr = fp & rmask;
        const uint32_t G = fq / MIR_SLOTS, k = fq - G * MIR_SLOTS;
        uint32_t r0[8], r1[8];
        ld_record(rec, G, keep, r0);
        ld_record(rec, G + 1, keep, r1);
        uint32_t res = mirror_query(fq, fr, k, r0, r1);
        if (res == MIRROR_UNDECIDED) res = sqf_query_b1(v, fq, fr, ld_word(v, fq >> 3));
        st_stream_u32(out + i, res, pass);
        key = knext;
    }
}
#endif

}  // namespace gqf
