// Batched filters: many independent standard quotient filters, of any mix
// of sizes and fills, bulk built and then queried by ONE launch of each
// pipeline kernel (hash histogram, bucket scan, scatter, bucket layout,
// occupied fix-up, lookups) instead of one pipeline per filter.  Every kernel
// takes its work units from a global list (scatter chunks, buckets, query
// chunks) spanning all filters, so a small filter costs a few CTAs of a
// full-size launch instead of a mostly idle launch of its own.  The launch
// sequence of a batch is captured once into a CUDA graph and replayed.
//
// Per filter the results are exactly those of bulkBuildSegmentedLayouts and
// launchUnsortedLookups on the same inputs (same kernels' per-bucket and
// per-query code; only the work lists differ).  The same pipeline also runs
// as one persistent cooperative launch (batch_persist.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "batch.cuh"
#include "host_common.cuh"

namespace gqf {

// Slots past the last bucket's quotients only receive spill: clear them in
// every filter that is rebuilt (the single-filter path does this with a
// memset before its layout).
template <int BPE>
__global__ void k_mf_clear_tails(MfParams p)
{
    for (uint32_t fi = blockIdx.x; fi < p.nf; fi += gridDim.x) {
        const MfFilter &f = p.f[fi];
        if (!f.n_keys) continue;
        const size_t tail = (size_t)(1u << f.q) * BPE;
        for (size_t i = tail + threadIdx.x; i < f.T; i += blockDim.x) f.table[i] = 0;
    }
}

template <int THREADS, int IPT>
__global__ void __launch_bounds__(THREADS) k_mf_hist(MfParams p)
{
    __shared__ uint32_t s_f;
    if (threadIdx.x == 0) s_f = mf_owner<&MfFilter::chunk0>(p.f, p.nf, blockIdx.x);
    __syncthreads();
    const MfFilter &f = p.f[s_f];
    bucket_hist_chunk<THREADS, IPT>(blockIdx.x - f.chunk0, f.keys, f.n_keys, mf_geom(f, p.tb), p.bcnt + f.bucket0);
}

template <int THREADS, int IPT>
__global__ void __launch_bounds__(THREADS) k_mf_scatter(MfParams p)
{
    __shared__ uint32_t s_f;
    if (threadIdx.x == 0) s_f = mf_owner<&MfFilter::chunk0>(p.f, p.nf, blockIdx.x);
    __syncthreads();
    const MfFilter &f = p.f[s_f];
    hash_bucket_chunk<THREADS, IPT, false>(blockIdx.x - f.chunk0, f.keys, f.n_keys, mf_geom(f, p.tb),
                                           p.bbase + f.bucket0, 0xFFFFFFFFu, p.bfill + f.bucket0, p.items, nullptr,
                                           p.err);
}

// Exclusive scan of the bucket counts of all filters (one CTA).
__global__ void __launch_bounds__(1024) k_mf_scan(const uint32_t *__restrict__ cnt, uint32_t nb,
                                                  uint32_t *__restrict__ base)
{
    __shared__ uint32_t sw[33];
    const uint32_t per = (nb + 1023) / 1024;
    const uint32_t b0 = min(nb, threadIdx.x * per), b1 = min(nb, b0 + per);
    uint32_t sum = 0;
    for (uint32_t b = b0; b < b1; b++) sum += cnt[b];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) sw[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const uint32_t v = sw[lane];
        uint32_t iv = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, iv, o);
            if (lane >= o) iv += t;
        }
        sw[lane] = iv - v;
    }
    __syncthreads();
    uint32_t run = sw[wid] + incl - sum;
    for (uint32_t b = b0; b < b1; b++) {
        base[b] = run;
        run += cnt[b];
    }
}

template <int THREADS, int QPT, int BPE>
__global__ void __launch_bounds__(THREADS, (THREADS >= 1024 ? 1 : 2)) k_mf_layout(MfParams p)
{
    __shared__ uint32_t s_gb, s_f;
    if (threadIdx.x == 0) {
        s_gb = atomicAdd(p.ticket, 1u);  // ticket order: a bucket's predecessors started first
        s_f = mf_owner<&MfFilter::bucket0>(p.f, p.nf, s_gb);
    }
    __syncthreads();
    const uint32_t fi = s_f;
    const MfFilter &f = p.f[fi];
    LayoutArgs a;
    a.A = BucketSrc{nullptr, nullptr, 0, nullptr};
    a.B = BucketSrc{p.items, p.bbase + f.bucket0, 0, p.bcnt + f.bucket0};
    a.table = f.table;
    a.q = f.q;
    a.r = f.r;
    a.tb = p.tb;
    a.nb = f.nb;
    a.nslots = f.nslots;
    a.cap_items = p.cap_items;
    a.op = OP_BUILD;
    a.nodup = p.nodup;
    a.bitmap_ok = p.bitmap_ok;
    a.a_dups = nullptr;
    a.status = p.status + f.bucket0;
    a.ticket = p.ticket;
    a.fix_list = p.fix_list + f.fix0;
    a.fix_cnt = p.fix_cnt + fi;
    a.fix_cap = f.fix_cap;
    a.fix_soft = 1;
    a.err = p.err;
    bucket_layout_body<THREADS, QPT, BPE>(a, s_gb - f.bucket0);
}

template <int BPE>
__global__ void k_mf_fixup(MfParams p)
{
    for (uint32_t fi = blockIdx.x; fi < p.nf; fi += gridDim.x) {
        const MfFilter &f = p.f[fi];
        if (f.n_keys) mf_occupied_bits<BPE>(p, f, fi, threadIdx.x, blockDim.x);
    }
}

// Lookups of all filters: work unit = MF_QCHUNK queries of one filter, each
// thread answering LOOKUP_QPT of them as k_lookup_unsorted does.
template <int BPE>
__global__ void __launch_bounds__(LOOKUP_THREADS) k_mf_lookup(MfParams p, uint32_t total)
{
    __shared__ uint32_t s_f;
    for (uint32_t u = blockIdx.x; u < total; u += gridDim.x) {
        __syncthreads();
        if (threadIdx.x == 0) s_f = mf_owner<&MfFilter::qchunk0>(p.f, p.nf, u);
        __syncthreads();
        const MfFilter &f = p.f[s_f];
        const TableView v{f.table, f.q, f.r, f.nslots, f.T, f.T / 8};
        const uint32_t fpmask = (f.q + f.r >= 32) ? 0xFFFFFFFFu : ((1u << (f.q + f.r)) - 1u);
        const uint32_t c0 = (u - f.qchunk0) * MF_QCHUNK;
        uint32_t fp[LOOKUP_QPT], res[LOOKUP_QPT];
        bool valid[LOOKUP_QPT];
#pragma unroll
        for (int k = 0; k < LOOKUP_QPT; k++) {
            const uint32_t i = c0 + k * LOOKUP_THREADS + threadIdx.x;
            valid[k] = i < f.n_q;
            fp[k] = valid[k] ? aphash32(__ldg(f.queries + i)) & fpmask : 0u;
        }
        sqf_query_batch<BPE>(v, fp, valid, res);
#pragma unroll
        for (int k = 0; k < LOOKUP_QPT; k++)
            if (valid[k]) f.results[c0 + k * LOOKUP_THREADS + threadIdx.x] = res[k];
    }
}

// ------------------------------------------------------------------ plan
struct Batch {
    int device = 0;
    uint32_t r = 5, bpe = 1, nf = 0;
    gqf_batch_tuning tune{};
    MfParams p{};
    uint32_t total_chunks = 0, total_buckets = 0, total_qchunks = 0, nbmax = 1;
    size_t layout_smem = 0;
    bool any_build = false, any_lookup = false;
    char *mem = nullptr;
    void *ctrl = nullptr;
    size_t ctrl_bytes = 0;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // the persistent pipeline (one cooperative launch); pkernel == nullptr
    // when the tuning's shape is not one of the compiled ones
    MfPersist px{};
    const void *pkernel = nullptr;
    int pthreads = 0, pgrid = 0;
    size_t psmem = 0;
};

template <typename K>
static cudaError_t mf_smem(K kernel, size_t bytes)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Calls fn(kernel-set) for the scatter shape of the tuning.
template <typename Fn>
static cudaError_t mf_with_scatter(uint32_t chunk, Fn fn)
{
    switch (chunk) {
    case 2048: return fn(k_mf_hist<256, 8>, k_mf_scatter<256, 8>, 256u, 2048u);
    case 32768: return fn(k_mf_hist<1024, 32>, k_mf_scatter<1024, 32>, 1024u, 32768u);
    default: return fn(k_mf_hist<256, 32>, k_mf_scatter<256, 32>, 256u, 8192u);
    }
}

template <int BPE, typename Fn>
static cudaError_t mf_with_layout(uint32_t tb, Fn fn)
{
    switch (tb) {
    case 13: return fn(k_mf_layout<256, 32, BPE>, 256);
    case 12: return fn(k_mf_layout<128, 32, BPE>, 128);
    case 11: return fn(k_mf_layout<64, 32, BPE>, 64);
    default: return fn(k_mf_layout<32, 32, BPE>, 32);
    }
}

template <int BPE>
static int mf_record(Batch &b, cudaStream_t s)
{
    const DeviceInfo &di = device_info(b.device);
    GQF_CK(cudaMemsetAsync(b.ctrl, 0, b.ctrl_bytes, s));
    if (b.any_build) {
        const uint32_t fgrid = std::min<uint32_t>(b.nf, (uint32_t)di.sms * 4);
        k_mf_clear_tails<BPE><<<fgrid, 256, 0, s>>>(b.p);
        GQF_CK(mf_with_scatter(b.tune.scatter_chunk, [&](auto khist, auto kscat, uint32_t threads, uint32_t chunk) {
            khist<<<b.total_chunks, threads, (size_t)b.nbmax * 4, s>>>(b.p);
            k_mf_scan<<<1, 1024, 0, s>>>(b.p.bcnt, b.total_buckets, b.p.bbase);
            kscat<<<b.total_chunks, threads, (size_t)chunk * 4 + (size_t)b.nbmax * 8, s>>>(b.p);
            return cudaGetLastError();
        }));
        GQF_CK(mf_with_layout<BPE>(b.p.tb, [&](auto klay, int threads) {
            klay<<<b.total_buckets, threads, b.layout_smem, s>>>(b.p);
            return cudaGetLastError();
        }));
        k_mf_fixup<BPE><<<fgrid, 256, 0, s>>>(b.p);
        count_launches(6);
    }
    if (b.any_lookup) {
        const uint32_t grid = std::min<uint32_t>(b.total_qchunks, (uint32_t)di.sms * 8);
        k_mf_lookup<BPE><<<grid, LOOKUP_THREADS, 0, s>>>(b.p, b.total_qchunks);
        count_launches(1);
    }
    GQF_CK(cudaGetLastError());
    return GQF_OK;
}

static int mf_record_any(Batch &b, cudaStream_t s) { return b.bpe == 1 ? mf_record<1>(b, s) : mf_record<2>(b, s); }

static void mf_free(Batch *b)
{
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->mem) cudaFree(b->mem);
    delete b;
}

static int mf_create(Batch *b, const gqf_sqf_job *jobs, int count, int no_duplicates, const gqf_batch_tuning *tune)
{
    b->device = current_device();
    const DeviceInfo &di = device_info(b->device);
    b->nf = (uint32_t)count;
    b->r = jobs[0].filter.rbits;
    b->bpe = (b->r + 3) / 8;
    uint32_t qmin = 32;
    uint64_t n_items = 0, fix_total = 0;
    for (int i = 0; i < count; i++) {
        const gqf_sqf &f = jobs[i].filter;
        if (!f.table || (reinterpret_cast<uintptr_t>(f.table) & 15u) || f.rbits != b->r ||
            f.bytesPerElement != b->bpe || f.qbits < 7 || f.qbits + f.rbits > 31)
            return GQF_ERR_ARG;
        if (jobs[i].n_build < 0 || jobs[i].n_lookup < 0) return GQF_ERR_ARG;
        if (jobs[i].n_build > 0 && !jobs[i].d_build_keys) return GQF_ERR_ARG;
        if (jobs[i].n_lookup > 0 && (!jobs[i].d_lookup_keys || !jobs[i].d_results)) return GQF_ERR_ARG;
        if (jobs[i].n_build > 0) qmin = std::min<uint32_t>(qmin, f.qbits);
        n_items += (uint64_t)jobs[i].n_build;
    }
    b->tune.bucket_bits = tune && tune->bucket_bits ? tune->bucket_bits : 12;
    b->tune.scatter_chunk = tune && tune->scatter_chunk ? tune->scatter_chunk : 8192;
    if (b->tune.scatter_chunk != 2048 && b->tune.scatter_chunk != 8192 && b->tune.scatter_chunk != 32768)
        return GQF_ERR_ARG;
    b->tune.cta_threads = tune && tune->cta_threads ? tune->cta_threads : 256;
    b->tune.items_per_thread = tune && tune->items_per_thread ? tune->items_per_thread : 32;
    if ((b->tune.cta_threads != 128 && b->tune.cta_threads != 256) ||
        (b->tune.items_per_thread != 8 && b->tune.items_per_thread != 32))
        return GQF_ERR_ARG;
    uint32_t tb = (uint32_t)std::min<int>(std::max(b->tune.bucket_bits, 10), 13);
    if (qmin < 32 && qmin < tb) return GQF_ERR_ARG;  // every rebuilt filter spans whole buckets
    b->tune.bucket_bits = (int)tb;
    // work lists
    std::vector<MfFilter> hf(count);
    uint32_t chunks = 0, buckets = 0, qchunks = 0, fix0 = 0, pchunks = 0;
    const uint32_t pchunk = (uint32_t)b->tune.cta_threads * (uint32_t)b->tune.items_per_thread;
    double max_avg = 0;
    for (int i = 0; i < count; i++) {
        const gqf_sqf &f = jobs[i].filter;
        MfFilter &m = hf[i];
        m.table = f.table;
        m.keys = jobs[i].d_build_keys;
        m.queries = jobs[i].d_lookup_keys;
        m.results = jobs[i].d_results;
        m.q = f.qbits;
        m.r = f.rbits;
        m.nslots = gqf_sqf_num_slots(f.qbits);
        m.T = (uint32_t)gqf_sqf_table_bytes(f.qbits, f.rbits);
        m.n_keys = (uint32_t)jobs[i].n_build;
        m.n_q = (uint32_t)jobs[i].n_lookup;
        m.chunk0 = chunks;
        m.pchunk0 = pchunks;
        m.bucket0 = buckets;
        m.qchunk0 = qchunks;
        m.fix0 = fix0;
        m.nb = m.n_keys ? 1u << (f.qbits - tb) : 0u;
        m.fix_cap = m.n_keys ? std::max<uint32_t>(1024u, m.nslots / 8) : 0u;
        chunks += (m.n_keys + b->tune.scatter_chunk - 1) / b->tune.scatter_chunk;
        pchunks += (m.n_keys + pchunk - 1) / pchunk;
        buckets += m.nb;
        qchunks += (m.n_q + MF_QCHUNK - 1) / MF_QCHUNK;
        fix0 += m.fix_cap;
        if (m.nb) {
            b->nbmax = std::max(b->nbmax, m.nb);
            max_avg = std::max(max_avg, (double)m.n_keys / m.nb);
        }
    }
    fix_total = fix0;
    b->total_chunks = chunks;
    b->total_buckets = buckets;
    b->total_qchunks = qchunks;
    b->any_build = buckets > 0;
    b->any_lookup = qchunks > 0;
    if (b->nbmax > 4096) return GQF_ERR_ARG;  // scatter keeps two words per bucket of a filter in shared memory
    // layout geometry (bitmap mode for r = 5 NoDup, else the general mode
    // needs a per-bucket capacity)
    const bool bitmap = b->r == 5 && no_duplicates;
    const uint32_t S = 1u << tb;
    size_t maxsm = (size_t)(di.smem_optin > 0 ? di.smem_optin : 99 * 1024) - 4096;
    uint32_t cap = (uint32_t)std::min<double>(max_avg * 1.25 + 10.0 * std::sqrt(max_avg) + 512.0, 65520.0);
    cap = (cap + 15) & ~15u;
    size_t sm = layout_smem_bytes(tb, cap, (int)b->bpe, bitmap);
    if (sm > maxsm) return GQF_ERR_ARG;
    (void)S;
    b->layout_smem = sm;
    // one allocation: descriptors | zeroed control | bases | items | fix-ups
    Sizer z;
    z.take<MfFilter>(count);
    const size_t ctrl0 = align_up(z.off, 256);
    z.take<uint32_t>(std::max(buckets, 1u));             // bcnt
    z.take<uint32_t>(std::max(buckets, 1u));             // bfill
    z.take<unsigned long long>(std::max(buckets, 1u));   // status
    z.take<uint32_t>(1);                                 // ticket
    z.take<uint32_t>(count);                             // fix_cnt
    z.take<uint32_t>(1);                                 // err
    z.take<uint32_t>(4);                                 // grid barrier of the persistent pipeline
    const size_t ctrl1 = z.off;
    z.take<uint32_t>(std::max(buckets, 1u));             // bbase
    z.take<uint32_t>(std::max<uint64_t>(n_items, 1));    // items
    z.take<uint32_t>(std::max<uint64_t>(fix_total, 1));  // fix lists
    GQF_CK(cudaMalloc(reinterpret_cast<void **>(&b->mem), z.off));
    Carver c(b->mem);
    MfFilter *d_f = c.take<MfFilter>(count);
    b->p.bcnt = c.take<uint32_t>(std::max(buckets, 1u));
    b->p.bfill = c.take<uint32_t>(std::max(buckets, 1u));
    b->p.status = c.take<unsigned long long>(std::max(buckets, 1u));
    b->p.ticket = c.take<uint32_t>(1);
    b->p.fix_cnt = c.take<uint32_t>(count);
    b->p.err = c.take<uint32_t>(1);
    b->px.bar = c.take<uint32_t>(4);
    b->p.bbase = c.take<uint32_t>(std::max(buckets, 1u));
    b->p.items = c.take<uint32_t>(std::max<uint64_t>(n_items, 1));
    b->p.fix_list = c.take<uint32_t>(std::max<uint64_t>(fix_total, 1));
    b->ctrl = b->mem + ctrl0;
    b->ctrl_bytes = ctrl1 - ctrl0;
    GQF_CK(cudaMemcpy(d_f, hf.data(), sizeof(MfFilter) * count, cudaMemcpyHostToDevice));
    b->p.f = d_f;
    b->p.nf = b->nf;
    b->p.tb = tb;
    b->p.cap_items = cap;
    b->p.nodup = no_duplicates ? 1 : 0;
    b->p.bitmap_ok = bitmap ? 1 : 0;
    b->p.total_buckets = buckets;
    // kernel attributes, then the graph
    GQF_CK(mf_with_scatter(b->tune.scatter_chunk, [&](auto khist, auto kscat, uint32_t, uint32_t chunk) {
        cudaError_t e = mf_smem(khist, (size_t)b->nbmax * 4);
        return e != cudaSuccess ? e : mf_smem(kscat, (size_t)chunk * 4 + (size_t)b->nbmax * 8);
    }));
    if (b->bpe == 1)
        GQF_CK(mf_with_layout<1>(tb, [&](auto klay, int) { return mf_smem(klay, b->layout_smem); }));
    else
        GQF_CK(mf_with_layout<2>(tb, [&](auto klay, int) { return mf_smem(klay, b->layout_smem); }));
    // the persistent shape: quotients per layout thread = 2^tb / threads
    b->px.total_chunks = pchunks;
    b->px.total_buckets = buckets;
    b->px.total_qchunks = qchunks;
    b->px.any_build = b->any_build ? 1 : 0;
    b->px.any_lookup = b->any_lookup ? 1 : 0;
    {
        const int threads = b->tune.cta_threads, ipt = b->tune.items_per_thread, qpt = (1 << tb) / threads;
        const size_t sm = std::max({(size_t)b->nbmax * 4, (size_t)pchunk * 4 + (size_t)b->nbmax * 8, b->layout_smem});
        auto setup = [&](const void *kern, int t) -> cudaError_t {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (e != cudaSuccess) return e;
            int per_sm = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, t, sm);
            if (e != cudaSuccess) return e;
            if (per_sm > 0) {
                b->pkernel = kern;
                b->pthreads = t;
                b->pgrid = per_sm * di.sms;
                b->psmem = sm;
            }
            return cudaSuccess;
        };
        const void *kern = mf_persistent_kernel((int)b->bpe, threads, ipt, qpt);
        if (kern) GQF_CK(setup(kern, threads));
    }
    GQF_CK(cudaEventCreate(&b->ev0));
    GQF_CK(cudaEventCreate(&b->ev1));
    GQF_CK(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
    GQF_CK(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
    int st = mf_record_any(*b, b->cap);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->cap, &g);
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    GQF_CK(e);
    b->graph = g;
    GQF_CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
    return GQF_OK;
}

}  // namespace gqf

using namespace gqf;

extern "C" {

int gqf_batch_create(gqf_batch **out, const gqf_sqf_job *jobs, int count, int no_duplicates,
                     const gqf_batch_tuning *tuning)
{
    if (!out || !jobs || count <= 0) return GQF_ERR_ARG;
    *out = nullptr;
    Batch *b = new Batch();
    int st = mf_create(b, jobs, count, no_duplicates, tuning);
    if (st) {
        mf_free(b);
        return st;
    }
    *out = reinterpret_cast<gqf_batch *>(b);
    return GQF_OK;
}

int gqf_batch_run(gqf_batch *batch, int use_graph, void *stream, float *ms)
{
    Batch *b = reinterpret_cast<Batch *>(batch);
    if (!b) return GQF_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (use_graph == GQF_BATCH_PERSISTENT && !b->pkernel) return GQF_ERR_ARG;
    if (ms) GQF_CK(cudaEventRecord(b->ev0, s));
    if (use_graph == GQF_BATCH_PERSISTENT) {
        GQF_CK(cudaMemsetAsync(b->ctrl, 0, b->ctrl_bytes, s));
        void *args[] = {&b->p, &b->px};
        GQF_CK(cudaLaunchCooperativeKernel(b->pkernel, dim3(b->pgrid), dim3(b->pthreads), args, b->psmem, s));
        count_launches(1);
    } else if (use_graph) {
        GQF_CK(cudaGraphLaunch(b->exec, s));
        count_launches(1);
    } else {
        int st = mf_record_any(*b, s);
        if (st) return st;
    }
    if (!ms) return GQF_OK;
    GQF_CK(cudaEventRecord(b->ev1, s));
    GQF_CK(cudaEventSynchronize(b->ev1));
    GQF_CK(cudaEventElapsedTime(ms, b->ev0, b->ev1));
    uint32_t e = 0;
    GQF_CK(cudaMemcpy(&e, b->p.err, sizeof e, cudaMemcpyDeviceToHost));
    return dev_err_to_status(e);
}

int gqf_batch_tuning_of(const gqf_batch *batch, gqf_batch_tuning *out)
{
    const Batch *b = reinterpret_cast<const Batch *>(batch);
    if (!b || !out) return GQF_ERR_ARG;
    *out = b->tune;
    return GQF_OK;
}

int gqf_batch_destroy(gqf_batch *batch)
{
    mf_free(reinterpret_cast<Batch *>(batch));
    return GQF_OK;
}

}  // extern "C"
