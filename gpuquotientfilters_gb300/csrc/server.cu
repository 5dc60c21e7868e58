// Served filters: a request loop with continuous batching over resident
// standard quotient filters.
//
// Requests (lookup / insert / delete batches of host keys on one filter) are
// queued per filter.  A dispatcher thread keeps up to `streams` ops on the
// device: whenever a stream slot is free it serves the filter whose oldest
// queued request has waited longest and that has no op in flight, building
// one op from all of that filter's queued requests of the head request's
// kind (up to max_op_keys keys).  Coalescing consecutive same-kind requests
// gives exactly the table and results of applying them one at a time:
// lookups see the same table; inserts skip fingerprints already present, so
// inserting A then B equals inserting A and B together; deletes remove one
// copy per occurrence up to the copies present, so deleting A then B equals
// deleting A and B together.  One op per filter at a time keeps every
// filter's requests in submission order while ops of different filters
// overlap on separate streams, each stream with its own workspace and
// staging buffers.  Requests arriving while ops run wait in the queues and
// join the next op of their filter: continuous batching.
//
// The HBM budget covers the filters' tables, and per stream the workspace
// of the largest update plus key and result staging; it fixes the number of
// streams.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "host_common.cuh"

namespace gqf {

struct SrvReq {
    uint64_t id;
    int filter, op;
    const uint32_t *keys;
    int n;
    uint32_t *results;
    double t_submit, t_start;
};

struct SrvSlot {
    cudaStream_t s = nullptr;
    uint32_t *d_keys = nullptr, *d_out = nullptr;
    uint32_t *h_err = nullptr;  // pinned: the op's latched device error word
    cudaEvent_t done = nullptr;
    bool busy = false;
    int filter = -1;
    int status = GQF_OK;
    std::vector<SrvReq> reqs;
};

struct Server {
    int device = 0;
    std::vector<gqf_sqf> filters;
    gqf_server_config cfg{};
    size_t hbm = 0;
    std::vector<SrvSlot> slots;
    std::chrono::steady_clock::time_point t0;
    // submissions and completions, shared with callers
    std::mutex mu;
    std::condition_variable cv;
    std::deque<SrvReq> incoming;
    std::vector<gqf_completion> completed;
    uint64_t next_id = 1, submitted = 0, finished = 0;
    bool stop = false;
    std::thread worker;
    // dispatcher-owned
    std::vector<std::deque<SrvReq>> queues;
    std::vector<char> in_flight;

    double now_us() const
    {
        return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
    }
};

static int srv_launch(Server &S, SrvSlot &slot)
{
    const gqf_sqf &qf = S.filters[slot.filter];
    const int op = slot.reqs.front().op;
    size_t off = 0;
    for (const SrvReq &r : slot.reqs) {
        GQF_CK(cudaMemcpyAsync(slot.d_keys + off, r.keys, (size_t)r.n * 4, cudaMemcpyHostToDevice, slot.s));
        off += (size_t)r.n;
    }
    int st = GQF_OK;
    if (op == GQF_SERVE_LOOKUP)
        st = gqf_sqf_lookup_unsorted(&qf, (int)off, slot.d_keys, slot.d_out, slot.s, nullptr);
    else if (op == GQF_SERVE_INSERT)
        st = gqf_sqf_insert(&qf, (int)off, slot.d_keys, slot.s, nullptr);
    else
        st = gqf_sqf_delete(&qf, (int)off, slot.d_keys, slot.s, nullptr);
    if (st) return st;
    if (op == GQF_SERVE_LOOKUP) {
        off = 0;
        for (const SrvReq &r : slot.reqs) {
            if (r.results)
                GQF_CK(cudaMemcpyAsync(r.results, slot.d_out + off, (size_t)r.n * 4, cudaMemcpyDeviceToHost, slot.s));
            off += (size_t)r.n;
        }
    }
    // the op's device error word (latched per stream by the entry point)
    Arena &a = arena(S.device, slot.s);
    GQF_CK(cudaMemcpyAsync(slot.h_err, a.latch, sizeof(uint32_t), cudaMemcpyDeviceToHost, slot.s));
    GQF_CK(cudaMemsetAsync(a.latch, 0, sizeof(uint32_t), slot.s));
    GQF_CK(cudaEventRecord(slot.done, slot.s));
    return GQF_OK;
}

static void srv_loop(Server *SP)
{
    Server &S = *SP;
    cudaSetDevice(S.device);
    const size_t cap = (size_t)S.cfg.max_op_keys;
    for (;;) {
        bool progressed = false;
        {
            std::unique_lock<std::mutex> lk(S.mu);
            while (!S.incoming.empty()) {
                SrvReq r = S.incoming.front();
                S.incoming.pop_front();
                S.queues[r.filter].push_back(r);
                progressed = true;
            }
            if (S.stop && S.submitted == S.finished) return;
        }
        // completions
        std::vector<gqf_completion> done;
        for (SrvSlot &slot : S.slots) {
            if (!slot.busy || cudaEventQuery(slot.done) != cudaSuccess) continue;
            const double t = S.now_us();
            if (slot.status == GQF_OK) slot.status = dev_err_to_status(*slot.h_err);
            for (const SrvReq &r : slot.reqs) done.push_back(gqf_completion{r.id, slot.status, r.t_submit, r.t_start, t});
            S.in_flight[slot.filter] = 0;
            slot.busy = false;
            slot.reqs.clear();
            progressed = true;
        }
        // dispatch: free slots to the filters whose head request is oldest
        for (SrvSlot &slot : S.slots) {
            if (slot.busy) continue;
            int best = -1;
            double oldest = 0;
            for (size_t f = 0; f < S.queues.size(); f++) {
                if (S.in_flight[f] || S.queues[f].empty()) continue;
                if (best < 0 || S.queues[f].front().t_submit < oldest) {
                    best = (int)f;
                    oldest = S.queues[f].front().t_submit;
                }
            }
            if (best < 0) break;
            std::deque<SrvReq> &q = S.queues[best];
            const int op = q.front().op;
            size_t keys = 0;
            const double t = S.now_us();
            do {
                SrvReq r = q.front();
                q.pop_front();
                r.t_start = t;
                keys += (size_t)r.n;
                slot.reqs.push_back(r);
            } while (S.cfg.coalesce && !q.empty() && q.front().op == op && keys + (size_t)q.front().n <= cap);
            slot.filter = best;
            slot.busy = true;
            *slot.h_err = 0;
            S.in_flight[best] = 1;
            slot.status = srv_launch(S, slot);
            if (slot.status) {  // nothing (more) runs for this op: complete it with the error
                cudaEventRecord(slot.done, slot.s);
            }
            progressed = true;
        }
        if (!done.empty()) {
            std::lock_guard<std::mutex> lk(S.mu);
            S.completed.insert(S.completed.end(), done.begin(), done.end());
            S.finished += done.size();
            S.cv.notify_all();
        }
        if (!progressed) {
            std::unique_lock<std::mutex> lk(S.mu);
            S.cv.wait_for(lk, std::chrono::microseconds(20),
                          [&] { return !S.incoming.empty() || (S.stop && S.submitted == S.finished); });
        }
    }
}

static void srv_free(Server *S)
{
    if (!S) return;
    if (S->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->stop = true;
            S->cv.notify_all();
        }
        S->worker.join();
    }
    for (SrvSlot &slot : S->slots) {
        if (slot.s) {
            cudaStreamSynchronize(slot.s);
            gqf_workspace_release(slot.s);
            cudaStreamDestroy(slot.s);
        }
        if (slot.d_keys) cudaFree(slot.d_keys);
        if (slot.d_out) cudaFree(slot.d_out);
        if (slot.h_err) cudaFreeHost(slot.h_err);
        if (slot.done) cudaEventDestroy(slot.done);
    }
    delete S;
}

static int srv_create(Server *S, const gqf_sqf *filters, int nf, const gqf_server_config *cfg)
{
    S->device = current_device();
    S->filters.assign(filters, filters + nf);
    S->cfg.hbm_budget_bytes = cfg ? cfg->hbm_budget_bytes : 0;
    S->cfg.max_streams = cfg && cfg->max_streams > 0 ? cfg->max_streams : 8;
    S->cfg.max_op_keys = cfg && cfg->max_op_keys > 0 ? cfg->max_op_keys : (1 << 22);
    S->cfg.coalesce = cfg ? cfg->coalesce : 1;
    size_t tables = 0, ws = 0;
    for (int i = 0; i < nf; i++) {
        const gqf_sqf &f = filters[i];
        if (!f.table || (reinterpret_cast<uintptr_t>(f.table) & 15u)) return GQF_ERR_ARG;
        tables += align_up(gqf_sqf_table_bytes(f.qbits, f.rbits), 256);
        ws = std::max(ws, gqf_sqf_update_workspace_bytes(f.qbits, f.rbits, S->cfg.max_op_keys));
    }
    const size_t staging = 2 * align_up((size_t)S->cfg.max_op_keys * 4, 256);
    const size_t per_stream = ws + staging;
    int streams = S->cfg.max_streams;
    if (S->cfg.hbm_budget_bytes) {
        if (S->cfg.hbm_budget_bytes < tables + per_stream) return GQF_ERR_NOMEM;
        streams = (int)std::min<size_t>((size_t)streams, (S->cfg.hbm_budget_bytes - tables) / per_stream);
    }
    S->slots.resize(streams);
    for (SrvSlot &slot : S->slots) {
        GQF_CK(cudaStreamCreateWithFlags(&slot.s, cudaStreamNonBlocking));
        GQF_CK(cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming));
        GQF_CK(cudaMalloc(&slot.d_keys, (size_t)S->cfg.max_op_keys * 4));
        GQF_CK(cudaMalloc(&slot.d_out, (size_t)S->cfg.max_op_keys * 4));
        GQF_CK(cudaMallocHost(&slot.h_err, sizeof(uint32_t)));
        int st = gqf_workspace_reserve(slot.s, ws, nullptr);
        if (st) return st;
    }
    S->hbm = tables + (size_t)streams * per_stream;
    S->queues.resize(nf);
    S->in_flight.assign(nf, 0);
    S->t0 = std::chrono::steady_clock::now();
    S->worker = std::thread(srv_loop, S);
    return GQF_OK;
}

}  // namespace gqf

using namespace gqf;

extern "C" {

int gqf_server_create(gqf_server **out, const gqf_sqf *filters, int nfilters, const gqf_server_config *cfg)
{
    if (!out || !filters || nfilters <= 0) return GQF_ERR_ARG;
    *out = nullptr;
    Server *S = new Server();
    int st = srv_create(S, filters, nfilters, cfg);
    if (st) {
        srv_free(S);
        return st;
    }
    *out = reinterpret_cast<gqf_server *>(S);
    return GQF_OK;
}

int gqf_server_submit(gqf_server *srv, int filter, int op, const uint32_t *keys, int n, uint32_t *results,
                      uint64_t *id)
{
    Server *S = reinterpret_cast<Server *>(srv);
    if (!S || filter < 0 || filter >= (int)S->filters.size() || op < 0 || op > 2 || n < 0 ||
        n > S->cfg.max_op_keys || (n > 0 && !keys) || (op == GQF_SERVE_LOOKUP && n > 0 && !results))
        return GQF_ERR_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return GQF_ERR_ARG;
    SrvReq r{S->next_id++, filter, op, keys, n, results, S->now_us(), 0.0};
    if (id) *id = r.id;
    S->incoming.push_back(r);
    S->submitted++;
    S->cv.notify_all();
    return GQF_OK;
}

int gqf_server_poll(gqf_server *srv, gqf_completion *out, int max, int *count)
{
    Server *S = reinterpret_cast<Server *>(srv);
    if (!S || !count || (max > 0 && !out)) return GQF_ERR_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    const int k = std::min<int>(max, (int)S->completed.size());
    std::copy(S->completed.begin(), S->completed.begin() + k, out);
    S->completed.erase(S->completed.begin(), S->completed.begin() + k);
    *count = k;
    return GQF_OK;
}

int gqf_server_drain(gqf_server *srv)
{
    Server *S = reinterpret_cast<Server *>(srv);
    if (!S) return GQF_ERR_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv.wait(lk, [&] { return S->submitted == S->finished; });
    return GQF_OK;
}

int gqf_server_info(const gqf_server *srv, int *streams, size_t *hbm_bytes)
{
    const Server *S = reinterpret_cast<const Server *>(srv);
    if (!S) return GQF_ERR_ARG;
    if (streams) *streams = (int)S->slots.size();
    if (hbm_bytes) *hbm_bytes = S->hbm;
    return GQF_OK;
}

int gqf_server_destroy(gqf_server *srv)
{
    srv_free(reinterpret_cast<Server *>(srv));
    return GQF_OK;
}

}  // extern "C"
