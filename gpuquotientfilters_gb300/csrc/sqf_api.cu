// C ABI of the standard quotient filter: host orchestration of the kernels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>

#include "host_common.cuh"
#include "sqf_build.cuh"
#include "sqf_extract.cuh"
#include "sqf_lookup.cuh"
#include "sqf_mirror.cuh"

namespace gqf {

// ------------------------------------------------------------------ geometry
static bool qr_ok(unsigned q, unsigned r)
{
    // quotientFilter.cu:46-47 asserts q + r <= 32 and (r + 3) % 8 == 0; a
    // 32-bit fingerprint would need `1 << 32` in the hash modulus (:268), so
    // q + r <= 31 here.  q >= 7 keeps a bucket at least 128 quotients.
    return (r + 3) % 8 == 0 && (r + 3) / 8 <= 2 && q >= 7 && q + r <= 31 && r >= 1;
}

struct SqfGeom {
    uint32_t q, r, bpe, nslots;
    size_t T;
};
static SqfGeom geom_of(const gqf_sqf *qf)
{
    SqfGeom g;
    g.q = qf->qbits;
    g.r = qf->rbits;
    g.bpe = (g.r + 3) / 8;
    g.nslots = gqf_sqf_num_slots(g.q);
    g.T = gqf_sqf_table_bytes(g.q, g.r);
    return g;
}

static uint32_t ceil_log2(uint64_t x)
{
    uint32_t l = 0;
    while ((1ull << l) < x) l++;
    return l;
}

struct LayoutPlan {
    BucketGeom g;
    uint32_t stride;     // speculative bucket stride (items)
    uint32_t cap_items;  // per-CTA item capacity of k_bucket_layout
    size_t smem;
    int threads;
};

// Bucket geometry for `n_expect` items over 2^q quotients: about 12k items
// per bucket (one CTA sorts a bucket in shared memory), at most 4096 buckets
// (the scatter keeps two u32 per bucket in shared memory).
static LayoutPlan plan_layout(uint32_t q, uint32_t r, uint64_t n_expect, uint64_t n_b_expect, bool bitmap)
{
    const DeviceInfo &di = device_info(current_device());
    LayoutPlan p;
    uint32_t tb_lo = std::max<uint32_t>(7, q > 12 ? q - 12 : 0);
    uint32_t tb_hi = std::min<uint32_t>(q, 15);
    uint64_t denom = n_expect ? n_expect : 1;
    uint32_t tb = ceil_log2((12000ull << q) / denom);
    tb = std::min(std::max(tb, tb_lo), tb_hi);
    p.g.q = q;
    p.g.r = r;
    p.g.tb = tb;
    p.g.nb = 1u << (q - tb);
    p.g.shift = r + tb;
    p.g.fp_mask = (q + r >= 32) ? 0xFFFFFFFFu : ((1u << (q + r)) - 1u);
    double avg_b = (double)n_b_expect / p.g.nb;
    p.stride = (uint32_t)align_up((size_t)(avg_b + 10.0 * std::sqrt(avg_b) + 64.0), 32);
    int bpe = (r + 3) / 8;
    double avg = (double)n_expect / p.g.nb;
    uint32_t need = (uint32_t)(avg * 1.05 + 10.0 * std::sqrt(avg) + 256.0);
    p.threads = tb >= 10 ? (1 << (tb - 5)) : 32;
    size_t S = (size_t)1 << tb;
    size_t tile = tile_bytes(tb, bpe) + S / 8;
    size_t counters = 4 * (S / 2 + S / 32 + 8);
    size_t bitmaps = 4 * (S + S / 8);
    size_t budget = 100 * 1024;
    size_t maxsm = (size_t)(di.smem_optin > 0 ? di.smem_optin : 99 * 1024) - 4096;
    size_t need_bytes = std::max(counters + (size_t)need * bpe, bitmap ? bitmaps : 0) + tile + 16;
    if (need_bytes > budget) budget = maxsm;
    size_t r0 = budget > tile + 16 ? budget - tile - 16 : 0;
    size_t cap = r0 > counters ? (r0 - counters) / bpe : 0;
    cap = std::min<size_t>(cap & ~(size_t)15, 65520);
    p.cap_items = (uint32_t)cap;
    p.smem = layout_smem_bytes(tb, p.cap_items, bpe, bitmap);
    return p;
}

static size_t scatter_smem(uint32_t nb, bool pairs)
{
    size_t chunk = pairs ? (size_t)PAIR_THREADS * PAIR_IPT : (size_t)SCATTER_THREADS * SCATTER_IPT;
    return (pairs ? 2 : 1) * chunk * 4 + (size_t)nb * 8;
}

template <typename K>
static cudaError_t set_smem(K kernel, size_t bytes)
{
    // the attribute is per function and device; set it only when it grows
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> done;
    const std::pair<const void *, int> key(reinterpret_cast<const void *>(kernel), current_device());
    std::lock_guard<std::mutex> lk(mu);
    size_t &cur = done[key];
    if (bytes <= cur) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

// Device-side exclusive scan of bucket counts into bases (nb <= 4096).
__global__ void __launch_bounds__(1024) k_scan_bases(const uint32_t *cnt, uint32_t nb, uint32_t *base)
{
    __shared__ uint32_t s[4097];
    __shared__ uint32_t sw[33];
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) s[i] = cnt[i];
    __syncthreads();
    block_exclusive_scan_u32<1024>(s, nb, sw);
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) base[i] = s[i];
}

// ------------------------------------------------------------ the pipeline
// Scratch for one rebuild: control words, look-back descriptors, fix-ups,
// the bucketed batch (B) and optionally the table's extracted contents (A).
struct Scratch {
    uint32_t *bcnt;              // nb  : batch items per bucket
    unsigned long long *status;  // nb  : look-back descriptors
    uint32_t *ticket;
    uint32_t *fix_cnt;
    uint32_t *a_dups;  // table holds duplicate fingerprints (set by extraction)
    uint32_t *fused_fail;  // the in-place update could not decode some bucket
    uint8_t *snap;         // table snapshot of the in-place update
    uint32_t *bbase;  // nb+1: exact batch bases
    uint32_t *fix_list;
    uint32_t fix_cap;
    uint32_t *bitems;  // batch fingerprints
    uint32_t *bidx;    // batch indices (sorted lookups)
    // extracted table contents
    Counts3 *tiles;
    uint32_t *Q, *E, *abase, *acnt;
    uint32_t *E2, *a2base, *a2cnt;
    size_t ctrl_bytes;
};

struct ScratchReq {
    uint32_t nb;
    size_t batch_items;  // capacity of the bucketed batch
    bool pairs;
    bool extract;   // table contents needed
    bool extract2;  // second table (merge)
    uint32_t nslots;
    size_t snap_bytes = 0;  // in-place update: snapshot of the table
};

static Scratch carve(void *base, const ScratchReq &r, bool sizing_only, size_t *bytes_out)
{
    Scratch s{};
    auto lay = [&](auto &c) {
        size_t nb = r.nb;
        s.bcnt = c.template take<uint32_t>(nb, 8);
        s.status = c.template take<unsigned long long>(nb, 8);
        s.ticket = c.template take<uint32_t>(1, 4);
        s.fix_cnt = c.template take<uint32_t>(1, 4);
        s.a_dups = c.template take<uint32_t>(1, 4);
        s.fused_fail = c.template take<uint32_t>(1, 4);
        s.ctrl_bytes = c.off;
        s.bbase = c.template take<uint32_t>(nb + 1);
        s.fix_cap = std::max<uint32_t>(65536u, r.nslots / 8);
        s.fix_list = c.template take<uint32_t>(s.fix_cap);
        s.bitems = c.template take<uint32_t>(std::max<size_t>(r.batch_items, 1));
        s.bidx = r.pairs ? c.template take<uint32_t>(std::max<size_t>(r.batch_items, 1)) : nullptr;
        if (r.extract) {
            size_t ntiles = (r.nslots + EXTRACT_TILE - 1) / EXTRACT_TILE;
            s.tiles = c.template take<Counts3>(ntiles + 1);
            s.Q = c.template take<uint32_t>(r.nslots);
            s.E = c.template take<uint32_t>(r.nslots);
            s.abase = c.template take<uint32_t>(nb + 1);
            s.acnt = c.template take<uint32_t>(nb);
            if (r.extract2) {
                s.E2 = c.template take<uint32_t>(r.nslots);
                s.a2base = c.template take<uint32_t>(nb + 1);
                s.a2cnt = c.template take<uint32_t>(nb);
            }
        }
        s.snap = r.snap_bytes ? c.template take<uint8_t>(r.snap_bytes) : nullptr;
    };
    if (sizing_only) {
        Sizer z;
        lay(z);
        *bytes_out = z.off;
    } else {
        Carver c(base);
        lay(c);
        *bytes_out = c.off;
    }
    return s;
}

// Extract a table's fingerprints (sorted for canonical tables) into E and
// bucket them by quotient range.  Count of elements stays on the device.
template <int BPE>
static int extract_into(const uint8_t *table, uint32_t nslots, size_t nbytes, uint32_t r, const BucketGeom &g,
                        Counts3 *tiles, uint32_t *Q, uint32_t *E, uint32_t *base, uint32_t *cnt, uint32_t *dups,
                        cudaStream_t s, const uint32_t *gate = nullptr)
{
    uint32_t ntiles = (nslots + EXTRACT_TILE - 1) / EXTRACT_TILE;
    count_launches(6);
    k_tile_counts<BPE><<<ntiles, EXTRACT_THREADS, 0, s>>>(table, nslots, (uint32_t)nbytes, tiles, dups, gate);
    k_scan_counts3<<<1, 1024, 0, s>>>(tiles, ntiles, gate);
    k_occ_list<BPE><<<ntiles, EXTRACT_THREADS, 0, s>>>(table, nslots, (uint32_t)nbytes, tiles, Q, gate);
    k_extract<BPE><<<ntiles, EXTRACT_THREADS, 0, s>>>(table, nslots, (uint32_t)nbytes, r, tiles, Q, E, gate);
    uint32_t grid = (g.nb + 1 + 255) / 256;
    k_sorted_bounds<<<grid, 256, 0, s>>>(E, &tiles[ntiles].ne, g.nb, g.shift, base, cnt, gate);
    k_bounds_to_counts<<<grid, 256, 0, s>>>(base, g.nb, cnt, gate);
    GQF_CK(cudaGetLastError());
    return GQF_OK;
}

// Hash + bucket the batch keys.  exact: histogram + device scan first.
// Bucketing a batch: histogram + scan (exact bases) or speculative strides,
// then the scatter.  Batches of up to SMALL_BATCH keys (inserts, deletes,
// small builds) use 4096-key chunks so that enough CTAs share the work; the
// large ones 32K-key chunks.
constexpr uint32_t SMALL_BATCH = 1u << 22;
constexpr int SMALL_THREADS = 256, SMALL_IPT = 16;

template <int T, int IPT>
static int bucket_batch_keys(const uint32_t *keys, uint32_t n, const LayoutPlan &p, Scratch &sc, bool exact,
                             uint32_t *err, cudaStream_t s)
{
    const uint32_t grid = (n + T * IPT - 1) / (T * IPT);
    if (exact) {
        count_launches(2);
        GQF_CK(set_smem(k_bucket_hist<T, IPT>, p.g.nb * 4));
        k_bucket_hist<T, IPT><<<grid, T, p.g.nb * 4, s>>>(keys, n, p.g, sc.bcnt);
        k_scan_bases<<<1, 1024, 0, s>>>(sc.bcnt, p.g.nb, sc.bbase);
        GQF_CK(cudaMemsetAsync(sc.bcnt, 0, p.g.nb * 4, s));
    }
    count_launches(1);
    auto kfn = k_hash_bucket<T, IPT, false>;
    const size_t sm = (size_t)T * IPT * 4 + (size_t)p.g.nb * 8;
    GQF_CK(set_smem(kfn, sm));
    kfn<<<grid, T, sm, s>>>(keys, n, p.g, exact ? sc.bbase : nullptr, exact ? 0xFFFFFFFFu : p.stride, sc.bcnt,
                            sc.bitems, nullptr, err);
    GQF_CK(cudaGetLastError());
    return GQF_OK;
}

static int bucket_batch(const uint32_t *keys, uint32_t n, const LayoutPlan &p, Scratch &sc, bool exact, bool pairs,
                        uint32_t *err, cudaStream_t s)
{
    if (n == 0) return GQF_OK;
    if (!pairs) {
        return n <= SMALL_BATCH ? bucket_batch_keys<SMALL_THREADS, SMALL_IPT>(keys, n, p, sc, exact, err, s)
                                : bucket_batch_keys<SCATTER_THREADS, SCATTER_IPT>(keys, n, p, sc, exact, err, s);
    }
    const uint32_t chunk = PAIR_THREADS * PAIR_IPT;
    const uint32_t grid = (n + chunk - 1) / chunk;
    const size_t sm = scatter_smem(p.g.nb, pairs);
    if (exact) {
        count_launches(2);
        GQF_CK(set_smem(k_bucket_hist<SCATTER_THREADS, SCATTER_IPT>, p.g.nb * 4));
        const uint32_t hgrid = (n + SCATTER_THREADS * SCATTER_IPT - 1) / (SCATTER_THREADS * SCATTER_IPT);
        k_bucket_hist<SCATTER_THREADS, SCATTER_IPT><<<hgrid, SCATTER_THREADS, p.g.nb * 4, s>>>(keys, n, p.g, sc.bcnt);
        k_scan_bases<<<1, 1024, 0, s>>>(sc.bcnt, p.g.nb, sc.bbase);
        GQF_CK(cudaMemsetAsync(sc.bcnt, 0, p.g.nb * 4, s));
    }
    count_launches(1);
    auto kfn = k_hash_bucket<PAIR_THREADS, PAIR_IPT, true>;
    GQF_CK(set_smem(kfn, sm));
    kfn<<<grid, PAIR_THREADS, sm, s>>>(keys, n, p.g, exact ? sc.bbase : nullptr, exact ? 0xFFFFFFFFu : p.stride,
                                       sc.bcnt, sc.bitems, sc.bidx, err);
    GQF_CK(cudaGetLastError());
    return GQF_OK;
}

template <int BPE>
static int launch_layout(const LayoutPlan &p, const SqfGeom &tg, uint8_t *table, const BucketSrc &A,
                         const BucketSrc &B, int op, int nodup, bool bitmap_ok, const uint32_t *a_dups, Scratch &sc,
                         uint32_t *err, cudaStream_t s, const uint8_t *src_table = nullptr,
                         const uint32_t *gate = nullptr)
{
    // slots past the last bucket's quotients only receive spill: clear them
    // (a gated launch leaves that to k_fallback_prepare)
    size_t tail = (size_t)(1u << tg.q) * BPE;
    if (!gate && tg.T > tail) GQF_CK(cudaMemsetAsync(table + tail, 0, tg.T - tail, s));
    LayoutArgs a;
    a.A = A;
    a.B = B;
    a.table = table;
    a.q = tg.q;
    a.r = tg.r;
    a.tb = p.g.tb;
    a.nb = p.g.nb;
    a.nslots = tg.nslots;
    a.cap_items = p.cap_items;
    a.op = op;
    a.nodup = nodup;
    a.bitmap_ok = bitmap_ok ? 1 : 0;
    a.a_dups = a_dups;
    a.status = sc.status;
    a.ticket = sc.ticket;
    a.fix_list = sc.fix_list;
    a.fix_cnt = sc.fix_cnt;
    a.fix_cap = sc.fix_cap;
    a.err = err;
    a.src_table = src_table;
    a.fused_fail = src_table ? sc.fused_fail : nullptr;
    a.gate = gate;
    const size_t smem = p.smem + (src_table ? layout_fused_bytes(p.g.tb) + 16 : 0);
    // one thread per 32 consecutive quotients (fewer per thread below 1024
    // quotients per bucket)
    cudaError_t e = cudaSuccess;
    auto go = [&](auto kernel, int threads) {
        e = set_smem(kernel, smem);
        if (e == cudaSuccess) kernel<<<p.g.nb, threads, smem, s>>>(a);
    };
    if (src_table && BPE == 1 && op == OP_INSERT) {
        // in-place insert: merge into the staged old slices
        const size_t msm = merge_plan(p.g.tb).total;
        auto gm = [&](auto kernel, int threads) {
            e = set_smem(kernel, msm);
            if (e == cudaSuccess) kernel<<<p.g.nb, threads, msm, s>>>(a);
        };
        switch (p.g.tb) {
        case 15: gm(k_bucket_insert_merge<1024>, 1024); break;
        case 14: gm(k_bucket_insert_merge<512>, 512); break;
        case 13: gm(k_bucket_insert_merge<256>, 256); break;
        case 12: gm(k_bucket_insert_merge<128>, 128); break;
        case 11: gm(k_bucket_insert_merge<64>, 64); break;
        default: gm(k_bucket_insert_merge<32>, 32); break;
        }
    } else if (src_table && BPE == 1) {
        switch (p.g.tb) {
        case 15: go(k_bucket_layout<1024, 32, BPE, true>, 1024); break;
        case 14: go(k_bucket_layout<512, 32, BPE, true>, 512); break;
        case 13: go(k_bucket_layout<256, 32, BPE, true>, 256); break;
        case 12: go(k_bucket_layout<128, 32, BPE, true>, 128); break;
        case 11: go(k_bucket_layout<64, 32, BPE, true>, 64); break;
        case 10: go(k_bucket_layout<32, 32, BPE, true>, 32); break;
        case 9: go(k_bucket_layout<32, 16, BPE, true>, 32); break;
        case 8: go(k_bucket_layout<32, 8, BPE, true>, 32); break;
        default: go(k_bucket_layout<32, 4, BPE, true>, 32); break;
        }
    } else {
        switch (p.g.tb) {
        case 15: go(k_bucket_layout<1024, 32, BPE>, 1024); break;
        case 14: go(k_bucket_layout<512, 32, BPE>, 512); break;
        case 13: go(k_bucket_layout<256, 32, BPE>, 256); break;
        case 12: go(k_bucket_layout<128, 32, BPE>, 128); break;
        case 11: go(k_bucket_layout<64, 32, BPE>, 64); break;
        case 10: go(k_bucket_layout<32, 32, BPE>, 32); break;
        case 9: go(k_bucket_layout<32, 16, BPE>, 32); break;
        case 8: go(k_bucket_layout<32, 8, BPE>, 32); break;
        default: go(k_bucket_layout<32, 4, BPE>, 32); break;
        }
    }
    GQF_CK(e);
    const DeviceInfo &di = device_info(current_device());
    count_launches(2);
    k_fixup_occ<BPE><<<di.sms * 2, 256, 0, s>>>(table, sc.fix_list, sc.fix_cnt, sc.fix_cap, gate);
    GQF_CK(cudaGetLastError());
    return GQF_OK;
}

// Asynchronous in-place update that could not place some bucket (*gate
// set): reset what the general path's layout expects at zero -- look-back
// descriptors, bucket ticket, fix-up count, duplicate flag, the call's error
// word -- and clear the table's spill slots past the last bucket.  The
// general path then rebuilds every slot from the snapshot's contents.
__global__ void k_fallback_prepare(const uint32_t *__restrict__ gate, unsigned long long *status, uint32_t nb,
                                   uint32_t *ticket, uint32_t *fix_cnt, uint32_t *dups, uint32_t *err,
                                   uint8_t *tail, size_t tail_bytes)
{
    if (!*gate) return;
    const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x, step = (size_t)gridDim.x * blockDim.x;
    for (size_t i = i0; i < nb; i += step) status[i] = 0ull;
    for (size_t i = i0; i < tail_bytes; i += step) tail[i] = 0;
    if (i0 == 0) {
        *ticket = 0;
        *fix_cnt = 0;
        *dups = 0;
        *err = 0;
    }
}

enum class Src { NONE, TABLE, KEYS, TABLE2 };

// Scratch bytes of rebuild() for an insert or delete of n keys (the same
// sizing as below).
static size_t update_scratch_bytes(uint32_t q, uint32_t r, uint32_t n)
{
    const uint32_t nslots = gqf_sqf_num_slots(q);
    const uint64_t expect = std::min<uint64_t>((uint64_t)(nslots * 0.9) + n, (uint64_t)nslots * 2);
    LayoutPlan p = plan_layout(q, r, expect, n, r == 5);
    ScratchReq req{p.g.nb, (size_t)p.g.nb * p.stride, false, true, false, nslots};
    size_t bytes = 0, bytes_exact = 0;
    carve(nullptr, req, true, &bytes);
    req.batch_items = std::max<size_t>(n, 1);
    carve(nullptr, req, true, &bytes_exact);
    return std::max(bytes, bytes_exact);
}

// One rebuild: A = current contents of `table` (when the op needs them) or
// of `table2`, B = hashed batch keys (or the second table's contents).
template <int BPE>
static int rebuild(const gqf_sqf *qf, const gqf_sqf *qf2, const uint32_t *keys, uint32_t n, int op, int nodup,
                   cudaStream_t s, float *ms)
{
    const SqfGeom tg = geom_of(qf);
    const bool needA = op != OP_BUILD;
    const bool bFromTable = qf2 != nullptr;
    uint64_t nA = needA ? tg.nslots : 0;  // worst case for sizing
    uint64_t nB = bFromTable ? tg.nslots : n;
    // expected items: the table holds at most nslots
    uint64_t expect = std::min<uint64_t>((needA ? (uint64_t)(tg.nslots * 0.9) : 0) + (bFromTable ? (uint64_t)(tg.nslots * 0.9) : n),
                                         (uint64_t)tg.nslots * 2);
    // r = 5 and set semantics: remainder bitmaps (see LayoutArgs::bitmap_ok)
    const bool bitmap_ok = tg.r == 5 && (((op == OP_BUILD || op == OP_MERGE) && nodup) || op == OP_INSERT ||
                                         op == OP_DELETE);
    LayoutPlan p = plan_layout(tg.q, tg.r, expect, bFromTable ? 0 : n, bitmap_ok);
    ScratchReq req{p.g.nb, bFromTable ? 0 : (size_t)p.g.nb * p.stride, false, needA, bFromTable, tg.nslots};
    (void)nA;
    (void)nB;
    int dev = current_device();
    Arena &ar = arena(dev, s);
    std::lock_guard<std::mutex> lk(ar.mu);
    size_t bytes = 0;
    carve(nullptr, req, true, &bytes);
    // exact-mode batch needs n items at most
    size_t bytes_exact = 0;
    ScratchReq req_exact = req;
    req_exact.batch_items = std::max<size_t>(n, 1);
    carve(nullptr, req_exact, true, &bytes_exact);
    // In-place update: an insert or delete on one-byte slots with set
    // semantics decodes every bucket's old contents straight from a snapshot
    // of the table (no extraction pass, see LayoutArgs).  If a bucket cannot
    // be placed that way (a table holding duplicate fingerprints), the op
    // reruns the general way from the snapshot: a synchronous call decides
    // on the host; an asynchronous one queues the general path behind the
    // in-place kernels with every launch gated on the device-side failure
    // flag, so it costs only empty launches when the in-place path held.
    // An insert whose batch averages more than half of MERGE_ITEMS new
    // fingerprints per bucket would send buckets over the in-place merge's
    // capacity and end up on the general path anyway: it goes there directly.
    const bool merge_fits = op != OP_INSERT || (uint64_t)n * 2 <= (uint64_t)p.g.nb * MERGE_ITEMS;
    const bool fused = BPE == 1 && bitmap_ok && (op == OP_INSERT || op == OP_DELETE) && !bFromTable && merge_fits;
    ScratchReq req_fused = req_exact;
    req_fused.snap_bytes = tg.T;
    size_t bytes_fused = 0;
    if (fused) carve(nullptr, req_fused, true, &bytes_fused);
    void *base = arena_reserve(ar, std::max(std::max(bytes, bytes_exact), bytes_fused));
    if (!base) return GQF_ERR_NOMEM;
    float ms_fused = 0.0f;
    if (fused) {
        Scratch sc = carve(base, req_fused, false, &bytes);
        int st = call_begin(ar, s, ms != nullptr);
        if (st) return st;
        // the snapshot is copied on the side stream while the batch is bucketed
        cudaStream_t side = arena_side(ar);
        if (!side) return GQF_ERR_CUDA;
        GQF_CK(cudaEventRecord(ar.fork, s));
        GQF_CK(cudaStreamWaitEvent(side, ar.fork, 0));
        GQF_CK(cudaMemcpyAsync(sc.snap, qf->table, tg.T, cudaMemcpyDeviceToDevice, side));
        GQF_CK(cudaEventRecord(ar.join, side));
        GQF_CK(cudaMemsetAsync(sc.bcnt, 0, sc.ctrl_bytes, s));
        BucketSrc A{nullptr, nullptr, 0, nullptr}, B{nullptr, nullptr, 0, nullptr};
        if (n) {
            st = bucket_batch(keys, n, p, sc, true, false, ar.err, s);
            if (st) return st;
            B = BucketSrc{sc.bitems, sc.bbase, 0, sc.bcnt};
        }
        GQF_CK(cudaStreamWaitEvent(s, ar.join, 0));
        st = launch_layout<BPE>(p, tg, qf->table, A, B, op, nodup, true, nullptr, sc, ar.err, s, sc.snap);
        if (st) return st;
        if (!ms) {
            // the general path, gated on the failure flag: contents from the
            // snapshot, the bucketed batch as it stands
            const DeviceInfo &di = device_info(current_device());
            const size_t tail = (size_t)(1u << tg.q) * BPE;
            count_launches(1);
            k_fallback_prepare<<<di.sms * 4, 256, 0, s>>>(sc.fused_fail, sc.status, p.g.nb, sc.ticket, sc.fix_cnt,
                                                           sc.a_dups, ar.err, qf->table + tail,
                                                           tg.T > tail ? tg.T - tail : 0);
            GQF_CK(cudaGetLastError());
            st = extract_into<BPE>(sc.snap, tg.nslots, tg.T, tg.r, p.g, sc.tiles, sc.Q, sc.E, sc.abase, sc.acnt,
                                   sc.a_dups, s, sc.fused_fail);
            if (st) return st;
            A = BucketSrc{sc.E, sc.abase, 0, sc.acnt};
            st = launch_layout<BPE>(p, tg, qf->table, A, B, op, nodup, bitmap_ok, sc.a_dups, sc, ar.err, s, nullptr,
                                    sc.fused_fail);
            if (st) return st;
            return call_end(ar, s, nullptr);
        }
        uint32_t rep[2];
        st = call_report(ar, s, sc.fused_fail, rep);
        if (st) return st;
        const uint32_t e = rep[0], fail = rep[1];
        GQF_CK(cudaEventElapsedTime(&ms_fused, ar.ev0, ar.ev1));
        if (!fail) {
            *ms = ms_fused;
            return dev_err_to_status(e);
        }
        GQF_CK(cudaMemcpy(qf->table, sc.snap, tg.T, cudaMemcpyDeviceToDevice));
    }
    // A timed build uses speculative bucket strides (one pass over the keys)
    // and reruns with exact bucket bases if a bucket overflowed; the rerun
    // rewrites the whole table from the keys.  Updates read the table, so
    // they and all asynchronous calls bucket exactly.
    bool exact = !(op == OP_BUILD && ms != nullptr);
    for (int attempt = 0; attempt < 2; attempt++) {
        Scratch sc = carve(base, exact ? req_exact : req, false, &bytes);
        int st = call_begin(ar, s, ms != nullptr);
        if (st) return st;
        GQF_CK(cudaMemsetAsync(sc.bcnt, 0, sc.ctrl_bytes, s));  // counters, look-back, ticket, fix-ups
        BucketSrc A{nullptr, nullptr, 0, nullptr}, B{nullptr, nullptr, 0, nullptr};
        if (needA) {
            st = extract_into<BPE>(qf->table, tg.nslots, tg.T, tg.r, p.g, sc.tiles, sc.Q, sc.E, sc.abase, sc.acnt,
                                   sc.a_dups, s);
            if (st) return st;
            A = BucketSrc{sc.E, sc.abase, 0, sc.acnt};
        }
        if (bFromTable) {
            st = extract_into<BPE>(qf2->table, tg.nslots, tg.T, tg.r, p.g, sc.tiles, sc.Q, sc.E2, sc.a2base, sc.a2cnt,
                                   nullptr, s);
            if (st) return st;
            B = BucketSrc{sc.E2, sc.a2base, 0, sc.a2cnt};
        } else if (n) {
            st = bucket_batch(keys, n, p, sc, exact, false, ar.err, s);
            if (st) return st;
            B = exact ? BucketSrc{sc.bitems, sc.bbase, 0, sc.bcnt} : BucketSrc{sc.bitems, nullptr, p.stride, sc.bcnt};
        }
        st = launch_layout<BPE>(p, tg, qf->table, A, B, op, nodup, bitmap_ok,
                                (op == OP_INSERT || op == OP_DELETE) ? sc.a_dups : nullptr, sc, ar.err, s);
        if (st) return st;
        if (!ms) return call_end(ar, s, nullptr);
        // synchronous: look at the error word before deciding
        uint32_t rep[2];
        st = call_report(ar, s, nullptr, rep);
        if (st) return st;
        const uint32_t e = rep[0];
        if ((e & DEV_ERR_BUCKET_OVER) && !exact) {
            exact = true;
            continue;
        }
        GQF_CK(cudaEventElapsedTime(ms, ar.ev0, ar.ev1));
        *ms += ms_fused;
        return dev_err_to_status(e);
    }
    return GQF_ERR_FULL;
}

template <int BPE>
static int lookup_unsorted_t(const gqf_sqf *qf, int n, const uint32_t *keys, uint32_t *out, cudaStream_t s, float *ms)
{
    const SqfGeom tg = geom_of(qf);
    Arena &ar = arena(current_device(), s);
    std::lock_guard<std::mutex> lk(ar.mu);
    // one-byte slots and a batch of at least one query per 16 slots: transpose
    // the table into the bit-plane mirror first
    const bool mirror = BPE == 1 && (uint64_t)n * 16 >= tg.nslots;
    uint4 *rec = nullptr;
    if (mirror) {
        rec = static_cast<uint4 *>(arena_reserve(ar, mir_bytes(tg.nslots)));
        if (!rec) return GQF_ERR_NOMEM;
        GQF_CK(set_smem(k_sqf_mirror, 2 * (size_t)MIR_TILE));
    }
    int st = call_begin(ar, s, ms != nullptr);
    if (st) return st;
    TableView v{qf->table, tg.q, tg.r, tg.nslots, (uint32_t)tg.T, (uint32_t)(tg.T / 8)};
    if (n > 0 && mirror) {
        const DeviceInfo &di = device_info(current_device());
        const uint32_t ngroups = mir_groups(tg.nslots);
        const uint32_t ntiles = (uint32_t)(((uint64_t)(ngroups + 1) * MIR_SLOTS + MIR_TILE - 1) / MIR_TILE);
        k_sqf_mirror<<<std::min<uint32_t>(ntiles, (uint32_t)di.sms * 3), MIR_BUILD_THREADS, 2 * MIR_TILE, s>>>(
            v, rec, ngroups, ntiles, ar.err);
        const uint32_t grid = std::min<uint32_t>((n + MIR_LOOKUP_THREADS - 1) / MIR_LOOKUP_THREADS,
                                                 (uint32_t)di.sms * 32);
        k_lookup_mirror<<<grid, MIR_LOOKUP_THREADS, 0, s>>>(keys, (uint32_t)n, v, rec, out);
        count_launches(2);
    } else if (n > 0) {
        const DeviceInfo &di = device_info(current_device());
        // one-byte slots: two queries per thread (more threads in flight
        // beat more loads per thread for the dependent word walks)
        constexpr int QPT = BPE == 1 ? 2 : LOOKUP_QPT;
        const uint32_t per_block = LOOKUP_THREADS * QPT;
        const uint32_t grid = std::min<uint32_t>((n + per_block - 1) / per_block, (uint32_t)di.sms * 32);
        k_lookup_unsorted<BPE, QPT><<<grid, LOOKUP_THREADS, 0, s>>>(keys, (uint32_t)n, v, out);
        count_launches(1);
    }
    return call_end(ar, s, ms);
}

template <int BPE>
static int lookup_sorted_t(const gqf_sqf *qf, int n, const uint32_t *keys, uint32_t *out, cudaStream_t s, float *ms)
{
    const SqfGeom tg = geom_of(qf);
    // Results go to the queries' input positions either way (the reference
    // sorts them back by index, quotientFilter.cu:304-305).  On one-byte slots
    // a batch of at least one query per 16 slots is answered faster through
    // the bit-plane mirror than by bucketing the queries first.
    if (BPE == 1 && (uint64_t)n * 16 >= tg.nslots) return lookup_unsorted_t<BPE>(qf, n, keys, out, s, ms);
    LayoutPlan p = plan_layout(tg.q, tg.r, (uint64_t)tg.nslots * 8 / 10, (uint64_t)n, false);
    // query buckets: aim for ~4k queries per bucket, table-aligned
    ScratchReq req{p.g.nb, (size_t)std::max(n, 1), true, false, false, tg.nslots};
    Arena &ar = arena(current_device(), s);
    std::lock_guard<std::mutex> lk(ar.mu);
    size_t bytes = 0;
    carve(nullptr, req, true, &bytes);
    void *base = arena_reserve(ar, bytes);
    if (!base) return GQF_ERR_NOMEM;
    Scratch sc = carve(base, req, false, &bytes);
    int st = call_begin(ar, s, ms != nullptr);
    if (st) return st;
    if (n > 0) {
        GQF_CK(cudaMemsetAsync(sc.bcnt, 0, sc.ctrl_bytes, s));
        st = bucket_batch(keys, (uint32_t)n, p, sc, true, true, ar.err, s);
        if (st) return st;
        TableView v{qf->table, tg.q, tg.r, tg.nslots, (uint32_t)tg.T, (uint32_t)(tg.T / 8)};
        BucketSrc src{sc.bitems, sc.bbase, 0, sc.bcnt};
        const size_t lsm = lks_smem_bytes(p.g.tb);
        const DeviceInfo &di = device_info(current_device());
        if (BPE == 1 && (reinterpret_cast<uintptr_t>(qf->table) & 15) == 0 && p.g.tb >= 8 &&
            lsm <= (size_t)(di.smem_optin > 0 ? di.smem_optin : 48 * 1024)) {
            GQF_CK(set_smem(k_lookup_bucketed_s, lsm));
            k_lookup_bucketed_s<<<p.g.nb, LKS_THREADS, lsm, s>>>(src, sc.bidx, v, p.g.tb, out);
        } else {
            k_lookup_bucketed<BPE><<<p.g.nb, LOOKUP_THREADS, 0, s>>>(src, sc.bidx, v, out);
        }
        count_launches(1);
    }
    return call_end(ar, s, ms);
}


// ------------------------------------------------ no-allocation bulk build
// Scratch for gqf_sqf_bulk_build_noalloc: a fixed array in the library's
// device image.  Host code must not use the symbol itself as an address;
// each device's address comes from cudaGetSymbolAddress on that device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[GQF_NOALLOC_SCRATCH_BYTES];
// Per device: the array's device address (looked up on the first call, with
// that device current) and a mutex that serialises the calls on it.
struct NoallocDev {
    std::mutex mu;
    void *base = nullptr;
};
static std::mutex g_noalloc_map_mu;
static std::map<int, NoallocDev> g_noalloc_dev;

template <int BPE>
static int bulk_build_noalloc_t(const gqf_sqf *qf, uint32_t n, const uint32_t *keys, int nodup, cudaStream_t s)
{
    const int dev = current_device();
    NoallocDev *nd;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_map_mu);
        nd = &g_noalloc_dev[dev];  // std::map nodes stay put
    }
    std::lock_guard<std::mutex> lk(nd->mu);
    if (!nd->base) {
        void *ptr = nullptr;
        GQF_CK(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
        nd->base = ptr;
    }
    char *base = static_cast<char *>(nd->base);
    const SqfGeom tg = geom_of(qf);
    const bool bitmap_ok = tg.r == 5 && nodup;
    LayoutPlan p = plan_layout(tg.q, tg.r, n, n, bitmap_ok);
    ScratchReq req{p.g.nb, std::max<size_t>(n, 1), false, false, false, tg.nslots};
    size_t need = 0;
    carve(nullptr, req, true, &need);
    const size_t err_off = GQF_NOALLOC_SCRATCH_BYTES - 256;  // device error word
    if (need > err_off) return GQF_ERR_LIMIT;
    size_t got = 0;
    Scratch sc = carve(base, req, false, &got);
    uint32_t *err = reinterpret_cast<uint32_t *>(base + err_off);
    // the array keeps the previous call's contents: clear what starts at zero
    GQF_CK(cudaMemsetAsync(err, 0, sizeof(uint32_t), s));
    GQF_CK(cudaMemsetAsync(sc.bcnt, 0, sc.ctrl_bytes, s));
    BucketSrc A{nullptr, nullptr, 0, nullptr}, B{nullptr, nullptr, 0, nullptr};
    if (n) {
        int st = bucket_batch(keys, n, p, sc, true, false, err, s);
        if (st) return st;
        B = BucketSrc{sc.bitems, sc.bbase, 0, sc.bcnt};
    }
    int st = launch_layout<BPE>(p, tg, qf->table, A, B, OP_BUILD, nodup, bitmap_ok, nullptr, sc, err, s);
    if (st) return st;
    uint32_t e = 0;
    GQF_CK(cudaMemcpyAsync(&e, err, sizeof(e), cudaMemcpyDeviceToHost, s));
    GQF_CK(cudaStreamSynchronize(s));
    return dev_err_to_status(e);
}

// One warp per bucket runs the build's look-back over host-given
// descriptors, with a caller-chosen poll limit (test support).
__global__ void k_lookback_probe(unsigned long long *status, uint32_t nb, uint32_t spin_limit, uint32_t *cin,
                                 uint32_t *err)
{
    const uint32_t b = blockIdx.x;
    if (b >= nb) return;
    const uint32_t c = lookback_cin_warp(status, b, err, spin_limit);
    if ((threadIdx.x & 31) == 0) cin[b] = c;
}

}  // namespace gqf

using namespace gqf;

#define BPE_DISPATCH(qf, fn, ...) (((qf)->rbits + 3) / 8 == 1 ? fn<1>(__VA_ARGS__) : fn<2>(__VA_ARGS__))

extern "C" {

size_t gqf_sqf_table_bytes(unsigned int q, unsigned int r)
{
    // calcNumSlotsGPU, quotientFilter.cu:37-42
    size_t table_bits = (size_t)(1u << q) * (r + 3);
    size_t table_slots = table_bits / 8;
    return (size_t)((double)table_slots * 1.1);
}

unsigned int gqf_sqf_num_slots(unsigned int q) { return (unsigned int)((double)(1u << q) * 1.1); }

size_t gqf_sqf_update_workspace_bytes(unsigned int q, unsigned int r, int n)
{
    if (!qr_ok(q, r) || n < 0) return 0;
    return align_up(update_scratch_bytes(q, r, (uint32_t)n), 1u << 20);
}

int gqf_sqf_init(gqf_sqf *qf, unsigned int q, unsigned int r)
{
    if (!qf || !qr_ok(q, r)) return GQF_ERR_ARG;
    qf->qbits = q;
    qf->rbits = r;
    qf->bytesPerElement = (r + 3) / 8;
    size_t T = gqf_sqf_table_bytes(q, r);
    unsigned char *t = nullptr;
    GQF_CK(cudaMalloc(&t, align_up(T, 256)));
    GQF_CK(cudaMemset(t, 0, align_up(T, 256)));
    qf->table = t;
    return GQF_OK;
}

int gqf_sqf_free(gqf_sqf *qf)
{
    if (!qf) return GQF_ERR_ARG;
    if (qf->table) GQF_CK(cudaFree(qf->table));
    qf->table = nullptr;
    return GQF_OK;
}

// the kernels read the table in aligned 8- and 16-byte words and bulk copies
static bool table_aligned(const void *t) { return (reinterpret_cast<uintptr_t>(t) & 15u) == 0; }
static bool sqf_ok(const gqf_sqf *qf)
{
    return qf && qf->table && table_aligned(qf->table) && qr_ok(qf->qbits, qf->rbits);
}

int gqf_sqf_bulk_build(const gqf_sqf *qf, int n, const uint32_t *d_keys, int no_duplicates, void *stream, float *ms)
{
    if (!sqf_ok(qf) || n < 0 || (n > 0 && !d_keys)) return GQF_ERR_ARG;
    return BPE_DISPATCH(qf, rebuild, qf, nullptr, d_keys, (uint32_t)n, OP_BUILD, no_duplicates ? 1 : 0,
                        static_cast<cudaStream_t>(stream), ms);
}

int gqf_sqf_bulk_build_noalloc(const gqf_sqf *qf, int n, const uint32_t *d_keys, int no_duplicates, void *stream)
{
    if (!sqf_ok(qf) || n < 0 || (n > 0 && !d_keys)) return GQF_ERR_ARG;
    if ((unsigned)n > GQF_NOALLOC_MAX_KEYS || qf->qbits > GQF_NOALLOC_MAX_Q) return GQF_ERR_LIMIT;
    return BPE_DISPATCH(qf, bulk_build_noalloc_t, qf, (uint32_t)n, d_keys, no_duplicates ? 1 : 0,
                        static_cast<cudaStream_t>(stream));
}

int gqf_sqf_insert(const gqf_sqf *qf, int n, const uint32_t *d_keys, void *stream, float *ms)
{
    if (!sqf_ok(qf) || n < 0 || (n > 0 && !d_keys)) return GQF_ERR_ARG;
    return BPE_DISPATCH(qf, rebuild, qf, nullptr, d_keys, (uint32_t)n, OP_INSERT, 1, static_cast<cudaStream_t>(stream),
                        ms);
}

int gqf_sqf_delete(const gqf_sqf *qf, int n, const uint32_t *d_keys, void *stream, float *ms)
{
    if (!sqf_ok(qf) || n < 0 || (n > 0 && !d_keys)) return GQF_ERR_ARG;
    return BPE_DISPATCH(qf, rebuild, qf, nullptr, d_keys, (uint32_t)n, OP_DELETE, 0, static_cast<cudaStream_t>(stream),
                        ms);
}

int gqf_sqf_insert_via_merge(const gqf_sqf *qf, const uint32_t *d_old, int n_old, const uint32_t *d_new, int n_new,
                             int no_duplicates, void *stream, float *ms)
{
    (void)d_old;
    (void)n_old;
    if (!sqf_ok(qf) || n_new < 0 || (n_new > 0 && !d_new)) return GQF_ERR_ARG;
    return BPE_DISPATCH(qf, rebuild, qf, nullptr, d_new, (uint32_t)n_new, OP_MERGE, no_duplicates ? 1 : 0,
                        static_cast<cudaStream_t>(stream), ms);
}

int gqf_sqf_merge(const gqf_sqf *qf1, const gqf_sqf *qf2, int no_duplicates, void *stream, float *ms)
{
    if (!sqf_ok(qf1) || !sqf_ok(qf2)) return GQF_ERR_ARG;
    if (qf1->qbits != qf2->qbits || qf1->rbits != qf2->rbits) return GQF_ERR_MISMATCH;
    return BPE_DISPATCH(qf1, rebuild, qf1, qf2, nullptr, 0u, OP_MERGE, no_duplicates ? 1 : 0,
                        static_cast<cudaStream_t>(stream), ms);
}

int gqf_sqf_lookup_unsorted(const gqf_sqf *qf, int n, const uint32_t *d_keys, uint32_t *d_out, void *stream, float *ms)
{
    if (!sqf_ok(qf) || n < 0 || (n > 0 && (!d_keys || !d_out))) return GQF_ERR_ARG;
    return BPE_DISPATCH(qf, lookup_unsorted_t, qf, n, d_keys, d_out, static_cast<cudaStream_t>(stream), ms);
}

int gqf_sqf_lookup_sorted(const gqf_sqf *qf, int n, const uint32_t *d_keys, uint32_t *d_out, void *stream, float *ms)
{
    if (!sqf_ok(qf) || n < 0 || (n > 0 && (!d_keys || !d_out))) return GQF_ERR_ARG;
    return BPE_DISPATCH(qf, lookup_sorted_t, qf, n, d_keys, d_out, static_cast<cudaStream_t>(stream), ms);
}

int gqf_debug_lookback_probe(const unsigned long long *status, unsigned int nb, unsigned int spin_limit,
                             unsigned int *cin)
{
    if (!status || !cin || nb == 0 || nb > (1u << 20) || spin_limit == 0) return GQF_ERR_ARG;
    unsigned long long *d_status = nullptr;
    uint32_t *d_cin = nullptr, *d_err = nullptr;
    int st = GQF_OK;
    uint32_t e = 0;
    cudaError_t ce = cudaMalloc(&d_status, sizeof(unsigned long long) * nb);
    if (ce == cudaSuccess) ce = cudaMalloc(&d_cin, sizeof(uint32_t) * nb);
    if (ce == cudaSuccess) ce = cudaMalloc(&d_err, sizeof(uint32_t));
    if (ce == cudaSuccess) ce = cudaMemcpy(d_status, status, sizeof(unsigned long long) * nb, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemset(d_err, 0, sizeof(uint32_t));
    if (ce == cudaSuccess) {
        count_launches(1);
        k_lookback_probe<<<nb, 32>>>(d_status, nb, spin_limit, d_cin, d_err);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    if (ce == cudaSuccess) ce = cudaMemcpy(cin, d_cin, sizeof(uint32_t) * nb, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(&e, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    st = ce == cudaSuccess ? dev_err_to_status(e) : GQF_ERR_CUDA;
    cudaFree(d_status);
    cudaFree(d_cin);
    cudaFree(d_err);
    return st;
}

}  // extern "C"
