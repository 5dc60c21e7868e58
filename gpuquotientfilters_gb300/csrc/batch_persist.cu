// Batched filters as ONE persistent cooperative launch (gqf_batch_run with
// GQF_BATCH_PERSISTENT): the pipeline of batch.cu -- tails, histogram, scan,
// scatter, layout, fix-ups, lookups -- walked by every CTA of a co-resident
// grid, phases separated by a bounded grid barrier.  Per filter the results
// are exactly those of the kernel-per-phase pipeline (same per-unit code).
#include "batch.cuh"

namespace gqf {

// ------------------------------------------------------------ persistent
// The whole pipeline as ONE cooperative launch: every CTA walks the phases
// (tails, histogram, scan, scatter, layout, fix-ups, lookups) taking work
// units from the same lists as the kernels above, and the phases are
// separated by a grid barrier.  The layout's buckets are taken by ticket, so
// a bucket's predecessors were taken by CTAs that are running.
// Grid-wide barrier for a co-resident grid: thread 0 of each CTA arrives,
// the last one opens the next generation.  The wait is bounded; a CTA that
// gives up records DEV_ERR_TIMEOUT and the abort word, and every CTA leaves
// at the next barrier.  Returns false when the pipeline must stop.
__device__ __forceinline__ bool mf_grid_sync(uint32_t *bar, uint32_t *err)
{
    __shared__ uint32_t s_go;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t go = 1;
        volatile uint32_t *vbar = bar;
        const uint32_t gen = vbar[1];
        __threadfence();  // this CTA's phase writes before its arrival
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            vbar[0] = 0u;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            uint32_t i = 0;
            while (vbar[1] == gen) {
                if (++i > SPIN_LIMIT) {
                    atomicOr(err, DEV_ERR_TIMEOUT);
                    atomicExch(bar + 2, 1u);
                    break;
                }
            }
        }
        __threadfence();
        if (vbar[2]) go = 0;
        s_go = go;
    }
    __syncthreads();
    return s_go != 0;
}

template <int THREADS, int IPT, int QPT, int BPE>
__global__ void __launch_bounds__(THREADS, 512 / THREADS) k_mf_persistent(MfParams p, MfPersist x)
{
    __shared__ uint32_t s_u, s_f;
    const uint32_t tid = threadIdx.x;
    if (x.any_build) {
        // slots past the last bucket's quotients only receive spill
        for (uint32_t fi = blockIdx.x; fi < p.nf; fi += gridDim.x) {
            const MfFilter &f = p.f[fi];
            if (!f.n_keys) continue;
            const size_t tail = (size_t)(1u << f.q) * BPE;
            for (size_t i = tail + tid; i < f.T; i += THREADS) f.table[i] = 0;
        }
        for (uint32_t u = blockIdx.x; u < x.total_chunks; u += gridDim.x) {
            __syncthreads();
            if (tid == 0) s_f = mf_owner<&MfFilter::pchunk0>(p.f, p.nf, u);
            __syncthreads();
            const MfFilter &f = p.f[s_f];
            bucket_hist_chunk<THREADS, IPT>(u - f.pchunk0, f.keys, f.n_keys, mf_geom(f, p.tb), p.bcnt + f.bucket0);
        }
        if (!mf_grid_sync(x.bar, p.err)) return;
        // exclusive scan of all bucket counts (one CTA)
        if (blockIdx.x == 0) {
            __shared__ uint32_t sw[THREADS / 32];
            const uint32_t nb = x.total_buckets, per = (nb + THREADS - 1) / THREADS;
            const uint32_t b0 = min(nb, tid * per), b1 = min(nb, b0 + per);
            uint32_t sum = 0;
            for (uint32_t b = b0; b < b1; b++) sum += p.bcnt[b];
            const uint32_t lane = tid & 31, wid = tid >> 5;
            uint32_t incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane == 31) sw[wid] = incl;
            __syncthreads();
            uint32_t run = incl - sum;
            for (uint32_t w = 0; w < wid; w++) run += sw[w];
            for (uint32_t b = b0; b < b1; b++) {
                p.bbase[b] = run;
                run += p.bcnt[b];
            }
        }
        if (!mf_grid_sync(x.bar, p.err)) return;
        for (uint32_t u = blockIdx.x; u < x.total_chunks; u += gridDim.x) {
            __syncthreads();
            if (tid == 0) s_f = mf_owner<&MfFilter::pchunk0>(p.f, p.nf, u);
            __syncthreads();
            const MfFilter &f = p.f[s_f];
            hash_bucket_chunk<THREADS, IPT, false>(u - f.pchunk0, f.keys, f.n_keys, mf_geom(f, p.tb),
                                                   p.bbase + f.bucket0, 0xFFFFFFFFu, p.bfill + f.bucket0, p.items,
                                                   nullptr, p.err);
        }
        if (!mf_grid_sync(x.bar, p.err)) return;
        for (;;) {
            __syncthreads();
            if (tid == 0) {
                s_u = atomicAdd(p.ticket, 1u);
                s_f = s_u < x.total_buckets ? mf_owner<&MfFilter::bucket0>(p.f, p.nf, s_u) : 0u;
            }
            __syncthreads();
            const uint32_t gb = s_u;
            if (gb >= x.total_buckets) break;
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
            bucket_layout_body<THREADS, QPT, BPE>(a, gb - f.bucket0);
        }
        if (!mf_grid_sync(x.bar, p.err)) return;
        for (uint32_t fi = blockIdx.x; fi < p.nf; fi += gridDim.x) {
            const MfFilter &f = p.f[fi];
            if (f.n_keys) mf_occupied_bits<BPE>(p, f, fi, tid, THREADS);
        }
        if (!mf_grid_sync(x.bar, p.err)) return;
    }
    if (x.any_lookup) {
        for (uint32_t u = blockIdx.x; u < x.total_qchunks; u += gridDim.x) {
            __syncthreads();
            if (tid == 0) s_f = mf_owner<&MfFilter::qchunk0>(p.f, p.nf, u);
            __syncthreads();
            const MfFilter &f = p.f[s_f];
            const TableView v{f.table, f.q, f.r, f.nslots, f.T, f.T / 8};
            const uint32_t fpmask = (f.q + f.r >= 32) ? 0xFFFFFFFFu : ((1u << (f.q + f.r)) - 1u);
            for (uint32_t c0 = (u - f.qchunk0) * MF_QCHUNK, c1 = c0 + MF_QCHUNK; c0 < c1;
                 c0 += THREADS * LOOKUP_QPT) {
                uint32_t fp[LOOKUP_QPT], res[LOOKUP_QPT];
                bool valid[LOOKUP_QPT];
#pragma unroll
                for (int k = 0; k < LOOKUP_QPT; k++) {
                    const uint32_t i = c0 + k * THREADS + tid;
                    valid[k] = i < f.n_q;
                    fp[k] = valid[k] ? aphash32(__ldg(f.queries + i)) & fpmask : 0u;
                }
                sqf_query_batch<BPE>(v, fp, valid, res);
#pragma unroll
                for (int k = 0; k < LOOKUP_QPT; k++)
                    if (valid[k]) f.results[c0 + k * THREADS + tid] = res[k];
            }
        }
    }
}

const void *mf_persistent_kernel(int bpe, int threads, int ipt, int qpt)
{
#define MF_P(T, I, Q)                                                                              \
    if (threads == T && ipt == I && qpt == Q)                                                      \
        return bpe == 1 ? reinterpret_cast<const void *>(k_mf_persistent<T, I, Q, 1>)             \
                        : reinterpret_cast<const void *>(k_mf_persistent<T, I, Q, 2>);
    MF_P(256, 32, 32) MF_P(256, 32, 16) MF_P(256, 8, 32) MF_P(256, 8, 16)
    MF_P(128, 32, 32) MF_P(128, 32, 16) MF_P(128, 8, 32) MF_P(128, 8, 16)
#undef MF_P
    return nullptr;
}

}  // namespace gqf
