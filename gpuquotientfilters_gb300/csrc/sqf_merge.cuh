// In-place insert for one-byte slots (k_bucket_insert_merge), split from
// sqf_build.cuh whose bucket machinery it uses: the look-back over bucket
// descriptors, the layout maps, the tile and descriptor helpers.
#pragma once

#include "sqf_build.cuh"

namespace gqf {

// ---------------------------------------------------------------------
// In-place insert by merging (one-byte slots).
//
// Inserting only moves elements right, so a stored element at old slot s
// lands at max(s, c) where c is the first free slot after everything placed
// before it: its home quotient is never needed.  An inserted fingerprint of
// quotient q lands at max(q, c).  Each is the layout step c -> max(c, K) + 1
// of the canonical recurrence, so a bucket is: the staged old slice in slot
// order with the new fingerprints merged in at their insertion points, the
// per-thread maps composed by the usual block scan and look-back, and the
// result written once.  Only elements that move are touched: the old slice
// is copied as it is, then every insertion (and a shift carried into a
// thread's stretch) moves the elements after it one slot at a time until an
// empty slot absorbs the shift.  A moved element keeps its remainder and
// continuation bit (the old head of a run gains one when a new fingerprint
// goes in front of it) and becomes shifted; occupied bits only gain the new
// quotients.  A fingerprint already stored, or repeated in the batch, is
// inserted at most once (OP_INSERT).  Anything this path cannot place (more
// than MERGE_ITEMS new fingerprints in the bucket, runs past the staged
// slice) sets *fused_fail and the host reruns the op the general way.
// ---------------------------------------------------------------------
constexpr uint32_t MERGE_ITEMS = 1024;  // new fingerprints one bucket merges
constexpr uint32_t MERGE_WS = 64;       // slots per stretch (a thread owns whole stretches)

// Shared-memory plan of the merge (byte offsets; all 16-byte aligned).
struct MergePlan {
    size_t sl, out, rs32, rsp, oc32, ocp, ne32, occ, wcnt, wbase, it, ip, ord, rk, fl, total;
};
__host__ __device__ inline MergePlan merge_plan(uint32_t tb)
{
    const size_t S = (size_t)1 << tb, L = S + SPILL_SLOTS, NW = L / 32, NWIN = L / MERGE_WS, NI = MERGE_ITEMS;
    auto a16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
    MergePlan m;
    size_t o = 0;
    m.sl = o;    o += a16(L + 16);       // the old slice
    m.out = o;   o += a16(L + 48);       // the rebuilt stretch
    m.rs32 = o;  o += a16(NW * 4);
    m.rsp = o;   o += a16(NW * 2);
    m.oc32 = o;  o += a16(S / 32 * 4);
    m.ocp = o;   o += a16(S / 32 * 2);
    m.ne32 = o;  o += a16(NW * 4);
    m.occ = o;   o += a16(S / 8);
    m.wcnt = o;  o += a16(NWIN * 4);
    m.wbase = o; o += a16(NWIN * 4);
    m.it = o;    o += a16(NI * 4);
    m.ip = o;    o += a16(NI * 4);
    m.ord = o;   o += a16(NI * 2);
    m.rk = o;    o += a16(NI * 2);
    m.fl = o;    o += a16(NI);
    m.total = o;
    return m;
}

template <int THREADS>
__device__ __forceinline__ void bucket_insert_merge(const LayoutArgs &a, const uint32_t b)
{
    extern __shared__ __align__(16) uint8_t smem_layout[];
    const uint32_t S = 1u << a.tb, L = S + SPILL_SLOTS, NW = L / 32, NWIN = L / MERGE_WS;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t x0 = b * S, r = a.r, rmask = (1u << r) - 1u;
    const MergePlan mp = merge_plan(a.tb);
    uint8_t *s_sl = smem_layout + mp.sl;    // the old slice, slots [x0, x0 + L)
    uint8_t *s_out = smem_layout + mp.out;  // the rebuilt stretch [gal, ge)
    uint32_t *s_rs32 = reinterpret_cast<uint32_t *>(smem_layout + mp.rs32);
    uint16_t *s_rsp = reinterpret_cast<uint16_t *>(smem_layout + mp.rsp);
    uint32_t *s_oc32 = reinterpret_cast<uint32_t *>(smem_layout + mp.oc32);
    uint16_t *s_ocp = reinterpret_cast<uint16_t *>(smem_layout + mp.ocp);
    uint32_t *s_ne32 = reinterpret_cast<uint32_t *>(smem_layout + mp.ne32);  // non-empty slots per 32-slot word
    uint32_t *s_occ = reinterpret_cast<uint32_t *>(smem_layout + mp.occ);
    uint32_t *s_wcnt = reinterpret_cast<uint32_t *>(smem_layout + mp.wcnt);    // new fingerprints per stretch
    uint32_t *s_wbase = reinterpret_cast<uint32_t *>(smem_layout + mp.wbase);  // their first index in s_ord
    uint32_t *s_it = reinterpret_cast<uint32_t *>(smem_layout + mp.it);
    uint32_t *s_ip = reinterpret_cast<uint32_t *>(smem_layout + mp.ip);        // insertion point (old slot)
    uint16_t *s_ord = reinterpret_cast<uint16_t *>(smem_layout + mp.ord);      // items grouped by stretch
    uint16_t *s_rk = reinterpret_cast<uint16_t *>(smem_layout + mp.rk);        // rank within the stretch
    uint8_t *s_fl = smem_layout + mp.fl;  // 1 skip, 2 head, 4 new quotient

    __shared__ int s_D0;
    __shared__ uint32_t s_nrs, s_nocc, s_lastne, s_pfirst, s_pend, s_bad;
    __shared__ uint32_t s_wsum[2][THREADS / 32];
    __shared__ LayoutFn s_wfn[THREADS / 32], s_wexcl[THREADS / 32];
    __shared__ uint32_t s_cin, s_cout, s_nfix, s_fbase;
    __shared__ uint32_t s_fix[256];

    const uint32_t nbn = a.B.count(b);
    const size_t bbase = nbn ? a.B.start(b) : 0;
    if (nbn > MERGE_ITEMS) {  // keep the look-back chain alive; the host reruns the op
        if (tid == 0) {
            atomicOr(a.fused_fail, 1u);
            st_relaxed_u64(a.status + b, lb_pack_inc(x0));
        }
        return;
    }
    if (tid == 0) {
        s_nfix = 0;
        s_bad = 0;
        s_lastne = 0;
    }
    // stage the old slice and the batch
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
    const uint32_t lmask = (S << r) - 1u;  // local fingerprint: local quotient << r | remainder
    for (uint32_t i = tid; i < nbn; i += THREADS) s_it[i] = a.B.items[bbase + i] & lmask;
    for (uint32_t w = tid; w < NWIN; w += THREADS) s_wcnt[w] = 0;
    if (wid == 0) {
        // runs of quotients below x0 still pending at x0
        const int D = pending_runs_warp(src, x0);
        if (lane == 0) s_D0 = D;
    }
    __syncthreads();
    // index: run starts and non-empty slots over the slice, occupied
    // quotients of the bucket, per 32-slot word, with exclusive prefix
    // counts; one past the last non-empty slot
    {
        const uint32_t per = (NW + THREADS - 1) / THREADS;
        const uint32_t w0 = min(NW, tid * per), w1 = min(NW, w0 + per);
        uint32_t cr = 0, co = 0, last = 0;
        for (uint32_t w = w0; w < w1; w++) {
            uint32_t rsm = 0, ocm = 0, nem = 0;
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const Flags8 f = flags8(*reinterpret_cast<const uint64_t *>(s_sl + 32 * w + 8 * h));
                rsm |= ((f.nonempty & ~f.cont) & 0xFFu) << (8 * h);
                ocm |= (f.occ & 0xFFu) << (8 * h);
                nem |= (f.nonempty & 0xFFu) << (8 * h);
            }
            s_rs32[w] = rsm;
            s_ne32[w] = nem;
            if (w < S / 32) s_oc32[w] = ocm;
            if (nem) last = 32 * w + (uint32_t)highest_bit(nem) + 1;
            cr += __popc(rsm);
            if (w < S / 32) co += __popc(ocm);
        }
        if (last) atomicMax(&s_lastne, last);
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
            s_wsum[0][wid] = ir;
            s_wsum[1][wid] = io;
        }
        __syncthreads();
        uint32_t pr = ir - cr, po = io - co;
        for (int w = 0; w < wid; w++) {
            pr += s_wsum[0][w];
            po += s_wsum[1][w];
        }
        if (tid == THREADS - 1) {
            s_nrs = pr + cr;
            s_nocc = po + co;
        }
        for (uint32_t w = w0; w < w1; w++) {
            s_rsp[w] = (uint16_t)pr;
            pr += __popc(s_rs32[w]);
            if (w < S / 32) {
                s_ocp[w] = (uint16_t)po;
                po += __popc(s_oc32[w]);
            }
        }
    }
    __syncthreads();
    const int D0 = s_D0, nrs = (int)s_nrs, nocc = (int)s_nocc;
    const uint32_t lastne = s_lastne;
    // slot of run start number R (R < nrs)
    auto run_start = [&](int R) -> uint32_t {
        uint32_t lo = 0, hi = NW;  // last word with s_rsp[w] <= R
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if ((int)s_rsp[mid] <= R) lo = mid;
            else hi = mid;
        }
        return (lo << 5) + (uint32_t)select_bit(s_rs32[lo], R - (int)s_rsp[lo]);
    };
    // the same from a word at or before the run start's (a run of quotient q
    // starts at or after slot q): a step or two instead of the binary search
    auto run_start_from = [&](int R, uint32_t w) -> uint32_t {
        while (w > 0 && (int)s_rsp[w] > R) w--;
        while (w + 1 < NW && (int)s_rsp[w + 1] <= R) w++;
        return (w << 5) + (uint32_t)select_bit(s_rs32[w], R - (int)s_rsp[w]);
    };
    if (tid == 0) {
        // the bucket's old runs occupy slots [pf, pe); runs past the slice,
        // or a last run that may continue past it, cannot be merged here
        const bool bad = D0 + nocc > nrs || (D0 + nocc == nrs && lastne >= L);
        const uint32_t pf = D0 < nrs ? run_start(D0) : lastne;
        const uint32_t pe = nocc == 0 ? pf : (D0 + nocc < nrs ? run_start(D0 + nocc) : lastne);
        s_pfirst = pf;
        s_pend = pe;
        if (bad) s_bad = 1;
    }
    // insertion point of each new fingerprint (the old slot it goes in
    // front of), and its rank among the fingerprints of its stretch
    for (uint32_t i = tid; i < nbn; i += THREADS) {
        const uint32_t v = s_it[i], ql = v >> r, rr = v & rmask;
        uint32_t fl = 0, ip = 0;
        const uint32_t ow = s_oc32[ql >> 5], bit = 1u << (ql & 31);
        const int R = D0 + (int)s_ocp[ql >> 5] + __popc(ow & (bit - 1u));
        if (ow & bit) {
            if (R >= nrs) {
                s_bad = 1;
            } else {
                const uint32_t p = run_start_from(R, ql >> 5);
                uint32_t t = p;
                for (;;) {
                    const uint32_t rem = (uint32_t)s_sl[t] >> 3;
                    if (rem >= rr) {
                        if (rem == rr) fl = 1;  // already stored
                        break;
                    }
                    if (++t >= L) {
                        s_bad = 1;
                        break;
                    }
                    const uint32_t e2 = s_sl[t];
                    if (!((e2 & 7u) && (e2 & 2u))) break;  // end of the run
                }
                ip = t;
                if (t == p) fl |= 2;  // in front of the old head
            }
        } else {
            ip = R < nrs ? run_start_from(R, ql >> 5) : lastne;
            fl |= 2 | 4;
        }
        if (ip >= L) {
            s_bad = 1;
            ip = L - 1;
        }
        s_ip[i] = ip;
        s_fl[i] = (uint8_t)fl;
        s_rk[i] = (uint16_t)atomicAdd(&s_wcnt[ip / MERGE_WS], 1u);
    }
    __syncthreads();
    // group the fingerprints by stretch: exclusive scan of the counts
    {
        const uint32_t per = (NWIN + THREADS - 1) / THREADS;
        const uint32_t w0 = min(NWIN, tid * per), w1 = min(NWIN, w0 + per);
        uint32_t cnt = 0;
        for (uint32_t w = w0; w < w1; w++) cnt += s_wcnt[w];
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += x;
        }
        if (lane == 31) s_wsum[0][wid] = incl;
        __syncthreads();
        uint32_t base = incl - cnt;
        for (int w = 0; w < wid; w++) base += s_wsum[0][w];
        for (uint32_t w = w0; w < w1; w++) {
            s_wbase[w] = base;
            base += s_wcnt[w];
        }
    }
    __syncthreads();
    for (uint32_t i = tid; i < nbn; i += THREADS) s_ord[s_wbase[s_ip[i] / MERGE_WS] + s_rk[i]] = (uint16_t)i;
    __syncthreads();
    if (s_bad) {
        if (tid == 0) {
            atomicOr(a.fused_fail, 1u);
            st_relaxed_u64(a.status + b, lb_pack_inc(x0));
        }
        return;
    }
    const uint32_t pfirst = s_pfirst, pend = s_pend;
    // this thread's stretches, windows [win0, win1), and their fingerprints
    const uint32_t wpt = (NWIN + THREADS - 1) / THREADS;
    const uint32_t win0 = min(NWIN, tid * wpt), win1 = min(NWIN, win0 + wpt);
    const uint32_t k0 = win0 < NWIN ? s_wbase[win0] : nbn;
    const uint32_t k1 = win1 < NWIN ? s_wbase[win1] : nbn;
    // order them by (insertion point, fingerprint) -- a handful per stretch --
    // then mark repeats, heads, displaced old heads and new quotients
    for (uint32_t k = k0 + 1; k < k1; k++) {
        const uint16_t x = s_ord[k];
        const uint64_t kx = ((uint64_t)s_ip[x] << 32) | s_it[x];
        uint32_t m = k;
        while (m > k0) {
            const uint16_t y = s_ord[m - 1];
            if ((((uint64_t)s_ip[y] << 32) | s_it[y]) <= kx) break;
            s_ord[m] = y;
            m--;
        }
        s_ord[m] = x;
    }
    for (uint32_t k = k0; k < k1; k++) {
        const uint32_t i = s_ord[k];
        uint32_t fl = s_fl[i];
        if (k > k0 && s_it[s_ord[k - 1]] == s_it[i]) fl |= 1u;  // repeated in the batch
        if (!(fl & 1u) && (fl & 2u)) {
            // the first kept fingerprint of its quotient at this point heads the run
            const uint32_t ql = s_it[i] >> r;
            for (uint32_t kk = k; kk > k0; kk--) {
                const uint32_t j = s_ord[kk - 1];
                if ((s_it[j] >> r) != ql || s_ip[j] != s_ip[i]) break;
                if (!(s_fl[j] & 1u)) {
                    fl &= ~2u;
                    break;
                }
            }
            if ((fl & 2u) && !(fl & 4u)) s_sl[s_ip[i]] |= 2u;  // the displaced old head continues the run
        }
        if (!(fl & 1u) && (fl & 4u)) atomicOr(s_oc32 + ((s_it[i] >> r) >> 5), 1u << ((s_it[i] >> r) & 31));
        s_fl[i] = (uint8_t)fl;
    }
    __syncthreads();
    // the bucket's old elements in [s0, s1)
    auto ours64 = [&](uint32_t w) -> uint64_t {  // stretch w (64 slots)
        uint64_t m = (uint64_t)s_ne32[2 * w] | ((uint64_t)s_ne32[2 * w + 1] << 32);
        const uint32_t a0 = w * MERGE_WS;
        if (pfirst > a0) m &= pfirst - a0 >= 64 ? 0ull : ~((1ull << (pfirst - a0)) - 1ull);
        if (pend < a0 + 64) m &= pend <= a0 ? 0ull : ((1ull << (pend - a0)) - 1ull);
        return m;
    };
    // walk [s0, s1) from c (the first free slot): elements keep their slots
    // until a fingerprint goes in or c runs past them; then each block of
    // consecutive elements moves by the same amount (c - its first slot),
    // and the empty slot after the block absorbs one slot of the shift.
    // emit(pos, byte) is called for every element that lands off its old
    // slot and every new fingerprint; returns (elements, final c)
    auto walk = [&](uint32_t c, auto &&emit) -> uint2 {
        uint32_t n = 0;
        uint32_t k = k0;
        for (uint32_t w = win0; w < win1; w++) {
            uint64_t m = ours64(w);
            const uint32_t a0 = w * MERGE_WS;
            n += __popcll(m);
            // every pass consumes a fingerprint or ends the stretch, and every
            // inner pass clears at least one bit of mm; the guards only back that up
            for (uint32_t guard = 0;; guard++) {
                if (guard > MERGE_ITEMS + 1) {
                    atomicOr(a.fused_fail, 1u);
                    break;
                }
                // next fingerprint in this stretch, or the stretch end
                const uint32_t stop = (k < k1 && s_ip[s_ord[k]] < a0 + MERGE_WS) ? s_ip[s_ord[k]] : a0 + MERGE_WS;
                const uint64_t below = stop - a0 >= 64 ? ~0ull : ((1ull << (stop - a0)) - 1ull);
                uint64_t mm = m & below;
                m &= ~below;
                for (uint32_t g2 = 0; mm && g2 <= 64; g2++) {
                    const uint32_t s = (uint32_t)(__ffsll((long long)mm) - 1);
                    const uint32_t sa = x0 + a0 + s;
                    if (c <= sa) {  // no shift from here to the stop
                        c = x0 + a0 + (uint32_t)(63 - __clzll((long long)mm)) + 1;
                        break;
                    }
                    // the block of consecutive elements from s moves to c
                    const uint64_t rest = ~(mm >> s);  // lowest set bit: first non-element
                    const uint32_t len = rest ? (uint32_t)(__ffsll((long long)rest) - 1) : 64u - s;
                    for (uint32_t t = 0; t < len; t++) emit(c + t, ((uint32_t)s_sl[a0 + s + t] & ~4u) | 1u);
                    c += len;
                    mm &= (s + len >= 64) ? 0ull : (~0ull << (s + len));
                }
                if (stop >= a0 + MERGE_WS) break;
                // the fingerprints inserted in front of old slot `stop`
                while (k < k1 && s_ip[s_ord[k]] == stop) {
                    const uint32_t i = s_ord[k++];
                    const uint32_t fl = s_fl[i];
                    if (fl & 1u) continue;
                    const uint32_t v = s_it[i], qa = x0 + (v >> r);
                    const uint32_t pos = qa > c ? qa : c;
                    emit(pos, ((v & rmask) << 3) | ((fl & 2u) ? 0u : 2u) | (pos != qa ? 1u : 0u));
                    c = pos + 1;
                    n++;
                }
            }
        }
        return make_uint2(n, c);
    };
    // this thread's layout map c -> max(c + n, F)
    LayoutFn fn{0u, 0u};
    {
        const uint2 nc = walk(0u, [&](uint32_t, uint32_t) {});
        fn.n = nc.x;
        fn.F = nc.x ? nc.y : 0u;
    }
    LayoutFn wexcl{0u, 0u};
    {
        LayoutFn f = fn;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            LayoutFn pv;
            pv.n = __shfl_up_sync(0xffffffffu, f.n, o);
            pv.F = __shfl_up_sync(0xffffffffu, f.F, o);
            if (lane >= o) f = compose(pv, f);
        }
        wexcl.n = __shfl_up_sync(0xffffffffu, f.n, 1);
        wexcl.F = __shfl_up_sync(0xffffffffu, f.F, 1);
        if (lane == 0) wexcl = LayoutFn{0u, 0u};
        if (lane == 31) s_wfn[wid] = f;
    }
    __syncthreads();
    if (wid == 0) {
        LayoutFn acc{0u, 0u};
        for (int w = 0; w < THREADS / 32; w++) {
            if (lane == 0) s_wexcl[w] = acc;
            acc = compose(acc, s_wfn[w]);
        }
        if (lane == 0 && (acc.n > LB_VMAX / 2 || acc.F > LB_VMAX / 2)) atomicOr(a.err, DEV_ERR_FULL);
        uint32_t cin = 0;
        if (b != 0) {
            if (lane == 0) st_relaxed_u64(a.status + b, lb_pack_agg(acc.n, acc.F));
            cin = lookback_cin_warp(a.status, b, a.err);
        }
        const uint32_t cout = acc.apply(cin);
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
    const uint32_t bufslots = span < L ? span : L;
    const size_t gs = lo, ge = gs + bufslots, gal = gs & ~(size_t)15;
    // the old contents of [gal, ge) as they are (slot x0 + i is s_sl[i];
    // slots past the slice are empty); elements that stay keep their bytes
    for (size_t g = gal + (size_t)tid * 16; g < ge; g += (size_t)THREADS * 16) {
        const size_t i = g - x0;
        const uint4 v = i + 16 <= L ? *reinterpret_cast<const uint4 *>(s_sl + i) : make_uint4(0, 0, 0, 0);
        *reinterpret_cast<uint4 *>(s_out + (g - gal)) = v;
    }
    // occupied quotients (old and new); those below lo become fix-ups
    for (uint32_t wq = tid; wq < S / 32; wq += THREADS) {
        const uint32_t nz = s_oc32[wq], xb = x0 + 32 * wq;
        const uint32_t nbelow = lo > xb ? min(lo - xb, 32u) : 0u;
        const uint32_t bmask = nbelow >= 32u ? 0xFFFFFFFFu : ((1u << nbelow) - 1u);
        for (uint32_t fxm = nz & bmask; fxm; fxm &= fxm - 1u) {
            const uint32_t xa = xb + (uint32_t)__ffs(fxm) - 1u;
            const uint32_t pp = atomicAdd(&s_nfix, 1u);
            if (pp < 256) {
                s_fix[pp] = xa;
            } else {
                const uint32_t gp = atomicAdd(a.fix_cnt, 1u);
                if (gp < a.fix_cap) a.fix_list[gp] = xa;
                else atomicOr(a.err, DEV_ERR_BUCKET_CAP);
            }
        }
        s_occ[wq] = nz & ~bmask;
    }
    __syncthreads();
    {
        const LayoutFn texcl = compose(s_wexcl[wid], wexcl);
        walk(texcl.apply(cin), [&](uint32_t pos, uint32_t e) {
            if (pos >= hi) return;  // past the table: reported as FULL
            if (pos - lo < bufslots) s_out[(size_t)pos - gal] = (uint8_t)e;
            else a.table[pos] = (uint8_t)e;
        });
    }
    __syncthreads();
    {
        const uint32_t nf = s_nfix < 256 ? s_nfix : 256;
        if (tid == 0 && nf) s_fbase = atomicAdd(a.fix_cnt, nf);
        __syncthreads();
        for (uint32_t i = tid; i < nf; i += THREADS) {
            const uint32_t gp = s_fbase + i;
            if (gp < a.fix_cap) a.fix_list[gp] = s_fix[i];
            else atomicOr(a.err, DEV_ERR_BUCKET_CAP);
        }
    }
    // store [gs, ge) with the new occupied bits merged in
    {
        auto occ_at = [&](size_t g) -> uint32_t {
            if (g < x0 || g >= (size_t)x0 + S) return 0u;
            const uint32_t o = (uint32_t)(g - x0);
            return (s_occ[o >> 5] >> (o & 31)) & 1u;
        };
        size_t h_end = (gs + 15) & ~(size_t)15;
        if (h_end > ge) h_end = ge;
        size_t b_end = ge & ~(size_t)15;
        if (b_end < h_end) b_end = h_end;
        for (size_t g = gs + tid; g < h_end; g += THREADS)
            a.table[g] = (uint8_t)(s_out[g - gal] | (occ_at(g) << 2));
        for (size_t g = h_end + (size_t)tid * 16; g < b_end; g += (size_t)THREADS * 16) {
            uint4 v = *reinterpret_cast<const uint4 *>(s_out + (g - gal));
            uint32_t bits = 0;
            if (g >= x0 && g < (size_t)x0 + S) {
                const uint32_t o = (uint32_t)(g - x0);
                bits = (s_occ[o >> 5] >> (o & 16u)) & 0xFFFFu;
            }
            auto spread4 = [](uint32_t x4) -> uint32_t { return ((x4 * 0x00204081u) & 0x01010101u) << 2; };
            v.x |= spread4(bits & 15u);
            v.y |= spread4((bits >> 4) & 15u);
            v.z |= spread4((bits >> 8) & 15u);
            v.w |= spread4((bits >> 12) & 15u);
            *reinterpret_cast<uint4 *>(a.table + g) = v;
        }
        for (size_t g = b_end + tid; g < ge; g += THREADS)
            a.table[g] = (uint8_t)(s_out[g - gal] | (occ_at(g) << 2));
    }
}

// In-place insert (one-byte slots): one CTA per bucket in ticket order,
// three CTAs per SM.
template <int THREADS>
__global__ void __launch_bounds__(THREADS, (THREADS >= 1024 ? 1 : 3)) k_bucket_insert_merge(LayoutArgs a)
{
    __shared__ uint32_t s_ticket;
    if (threadIdx.x == 0) s_ticket = atomicAdd(a.ticket, 1u);
    __syncthreads();
    bucket_insert_merge<THREADS>(a, s_ticket);
}

}  // namespace gqf
