"""Benchmark: the q=26, r=5, fill-0.8 standard quotient filter workload
(53,687,091 MT19937 keys, seed 2) through the reference's host API.

One step = bulkBuildSegmentedLayouts (NoDup) of all keys, 2^24 unsorted
lookups, 2^24 sorted lookups (50% inserted keys, 50% fresh draws), an
insert of 2^20 fresh keys and 2^20 deletes of present keys.  `value` is the
step's operations (keys built + queries + inserts + deletes) per second of
device time, summed over ranks (each rank runs an independent filter:
replicas, weak scaling).  Every op is a synchronous call (it returns its
status) timed on its stream with CUDA events, with L2 flushed before each
op.  `e2e` repeats the step through the same API from pinned host buffers,
host<->device copies inside the timed region, the ops queued asynchronously.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import concurrent.futures
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "M ops/s build/lookup/insert at q=26 r=5 fill .8 (%HBM roofline); served p50/p99"
Q, R, SEED = 26, 5, 2
N_KEYS = 53687091
N_LOOKUP = 1 << 24
N_INSERT = 1 << 20
N_DELETE = 1 << 20
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one q=26 r=5 NoDup build of
# N_KEYS keys, from one `ncu --set full` capture: k_hash_bucket 384,808,192 + k_bucket_layout
# 261,271,808 (k_fixup_occ touches a few KB).
BUILD_DRAM_BYTES = 384808192 + 261271808
# ops timed in every step but not counted in `value`
EXTRA_OPS = ("build_dup",)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(op: str, n: int, T: int) -> float:
    """Bytes one op must move at minimum (per-op model of the design notes)."""
    if op in ("build", "build_dup"):
        return 12.0 * n + T       # keys in, one fingerprint permutation, table out
    if op == "lookup_unsorted":
        return 40.0 * n           # key + result + one 32-B table sector
    if op == "lookup_sorted":
        return 24.0 * n + T       # key + result + (fp, idx) pair out and back + table sweep
    return 68.0 * n               # insert / delete: key + one sector read + written


class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(
                        ["nvidia-smi", "-i", str(self.index),
                         "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                         "clocks_event_reasons.sw_power_cap",
                         "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                    if out.returncode == 0 and out.stdout.strip():
                        self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 2 + i and "Active" in r[2 + i]
                          and r[2 + i] != "Not Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        import torch
        if not torch.cuda.is_available():
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x: float, device) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, world, rank, local):
    import torch

    import gpuquotientfilters_gb300 as G
    from gpuquotientfilters_gb300 import workload as W

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    G.lib()
    q = args.q
    n_keys = N_KEYS if q == Q else W.n_keys(q, 0.8)
    c = W.config2(seed=SEED, q=q, n=n_keys, n_lookup=N_LOOKUP >> (Q - q), n_insert=N_INSERT >> (Q - q),
                  n_delete=N_DELETE >> (Q - q))
    n_look, n_ins, n_del = c["lookups"].size, c["inserts"].size, c["deletes"].size
    T = G.calcNumSlotsGPU(q, R)

    def dev_u32(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)

    d_keys = dev_u32(c["keys"])
    d_look = dev_u32(c["lookups"])
    d_ins = dev_u32(c["inserts"])
    d_del = dev_u32(c["deletes"])
    d_out = torch.empty(n_look, dtype=torch.int32, device=dev)
    d_out2 = torch.empty(n_look, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2
    qf = G.initFilterGPU(q, R)
    stream = torch.cuda.current_stream(dev)

    # Config 2 builds with both Dup and NoDup.  The Dup build is timed in every
    # step and reported in per_op, but kept out of `value` (the NoDup build
    # right after it overwrites the table, and the step's ops are counted once).
    ops = [
        ("build_dup", n_keys, lambda: G.bulkBuildSegmentedLayouts(qf, n_keys, d_keys, False, stream=stream)),
        ("build", n_keys, lambda: G.bulkBuildSegmentedLayouts(qf, n_keys, d_keys, True, stream=stream)),
        ("lookup_unsorted", n_look, lambda: G.launchUnsortedLookups(qf, n_look, d_look, d_out, stream=stream)),
        ("lookup_sorted", n_look, lambda: G.launchSortedLookups(qf, n_look, d_look, d_out2, stream=stream)),
        ("insert", n_ins, lambda: G.insert(qf, n_ins, d_ins, stream=stream)),
        ("delete", n_del, lambda: G.superclusterDeletes(qf, n_del, d_del, stream=stream)),
    ]
    wanted = args.ops.split(",") if args.ops else None
    if wanted:
        ops = [o for o in ops if o[0] in wanted or o[0] == "build"]

    def step(record):
        tot = 0.0
        for name, n, fn in ops:
            flush.fill_(1)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            fn()
            ev1.record(stream)
            ev1.synchronize()
            ms = ev0.elapsed_time(ev1)
            if name not in EXTRA_OPS:
                tot += ms
            if record is not None:
                record.setdefault(name, []).append(ms)
        return tot

    for _ in range(args.warmup):
        step(None)
    # correctness guard on the measured path: sorted == unsorted
    if not wanted:
        assert torch.equal(d_out, d_out2), "sorted and unsorted lookups disagree"

    clocks = ClockSampler(local)
    rec = {}
    launches0 = G.lib().gqf_kernel_launches()
    barrier(world)
    torch.cuda.synchronize(dev)
    clocks.start()
    t_dev = 0.0
    for _ in range(args.steps):
        t_dev += step(rec)
    torch.cuda.synchronize(dev)
    barrier(world)
    clk = clocks.stop()
    launches = G.lib().gqf_kernel_launches() - launches0
    t_max = max_over_ranks(world, t_dev, dev)
    ops_per_step = sum(n for name, n, _ in ops if name not in EXTRA_OPS)
    value = world * ops_per_step * args.steps / (t_max / 1e3) / 1e6
    peak, peak_kind = peaks()
    per_op = {}
    for name, n, _ in ops:
        ms = float(np.mean(rec[name]))
        gbs = algorithmic_bytes(name, n, T) / (ms / 1e3) / 1e9
        per_op[name] = {"n": n, "ms": round(ms, 4), "mops": round(n / ms / 1e3, 1),
                        "alg_GBps": round(gbs, 1), "frac_hbm": round(gbs / peak, 4)}
    b = per_op["build"]

    # end to end through the same API from pinned host buffers
    e2e = e2e_step(args, G, torch, dev, stream, c, qf) if not wanted and q == Q else None
    G.freeFilterGPU(qf)
    del d_keys, d_look, d_ins, d_del, d_out, d_out2
    rsqf = rsqf_ops(args, G, torch, dev, stream, flush, peak) if args.rsqf and not wanted else None
    batched = batched_ops(args, G, torch, dev, stream, flush, peak) if args.batched and not wanted else None
    served = served_ops(args, G, torch, dev) if args.served and not wanted else None
    return {
        "value": value, "ms_per_step": t_max / args.steps, "per_op": per_op, "clocks": clk,
        "gpu_launches": int(launches), "peak": peak, "peak_kind": peak_kind, "e2e": e2e, "rsqf": rsqf,
        "batched": batched, "served": served,
        "roofline": {"bound": "hbm", "kernel": "bulk build pipeline (hash+bucket scatter, bucket layout, fixup)",
                     "achieved": b["alg_GBps"], "peak": peak, "unit": "GB/s", "frac": b["frac_hbm"],
                     "traffic": BUILD_DRAM_BYTES if q == Q else None,
                     "traffic_source": "ncu capture of the same build (k_hash_bucket + k_bucket_layout)",
                     "peak_source": peak_kind},
    }


def rsqf_ops(args, G, torch, dev, stream, flush, peak):
    """The rank-and-select filter (64-slot blocks): build to 0.9 fill by
    insertGPU of MT19937 seed-3 keys into an empty filter, 2^24 sorted
    lookups (50% positive), then 2^20 incremental inserts -- with 5-bit
    remainders at q=26 (60,397,976 keys), and with 8-bit remainders at q=23,
    the largest width whose q + 8 fingerprint bits fit the hash's 31
    (7,549,747 keys, batches scaled to 2^21 lookups and 2^17 inserts so the
    filter stays within its slots).  Reported beside the headline, not
    counted in it."""
    from gpuquotientfilters_gb300 import workload as W
    out = {}
    for rbits, q, tag in ((5, args.q, "rsqf"), (8, args.q - 3, "rsqf8")):
        n = W.n_keys(q, 0.9, reference_arithmetic=True)
        n_look, n_ins = N_LOOKUP >> (Q - q), N_INSERT >> (Q - q)  # the batches scale with the filter
        keys = G.mt19937(3, n + n_ins)
        look = W.mixed_lookups(keys[:n], n_look, 3, skip=n + n_ins)

        def dev_u32(a):
            return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)

        d_keys, d_ins, d_look = dev_u32(keys[:n]), dev_u32(keys[n:]), dev_u32(look)
        d_ret = torch.empty(n, dtype=torch.int32, device=dev)
        d_out = torch.empty(n_look, dtype=torch.int32, device=dev)
        rec = {}
        for it in range(args.warmup + args.steps):
            cqf = G.initCQFGPU(q, rbits)
            torch.cuda.synchronize(dev)
            for name, fn in (("build", lambda: G.insertGPU(cqf, n, d_keys, d_ret, stream=stream)),
                             ("lookup_sorted", lambda: G.launchLookups(cqf, n_look, d_look, d_out, stream=stream)),
                             ("insert", lambda: G.insertGPU(cqf, n_ins, d_ins, d_ret, stream=stream))):
                flush.fill_(1)
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
                fn()
                ev1.record(stream)
                ev1.synchronize()
                if it >= args.warmup:
                    rec.setdefault(name, []).append(ev0.elapsed_time(ev1))
            G.freeCQFGPU(cqf)
        nb = G.calcNumBlocksGPU(q)
        bb = 17 + 8 * rbits
        # build: key in, slot out, one fingerprint permutation, blocks written
        # once; lookup: key, result, the 32-B sectors of one block (two for
        # 57 bytes, three for 81); insert: key, slot, those sectors read and
        # written
        sect = 64 if rbits == 5 else 96
        for name, cnt, nbytes in (("build", n, 16.0 * n + bb * (nb + 1.0)),
                                  ("lookup_sorted", n_look, (8.0 + sect) * n_look),
                                  ("insert", n_ins, (8.0 + 2 * sect) * n_ins)):
            ms = float(np.mean(rec[name]))
            gbs = nbytes / (ms / 1e3) / 1e9
            out[tag + "_" + name] = {"n": cnt, "ms": round(ms, 4), "mops": round(cnt / ms / 1e3, 1),
                                     "alg_GBps": round(gbs, 1), "frac_hbm": round(gbs / peak, 4)}
        out[tag + "_workload"] = ("RSQF q=%d RBITS %d: insertGPU of %d keys (0.9 fill, MT19937 seed 3) into an empty "
                                  "filter, %d sorted lookups, %d incremental inserts" % (q, rbits, n, n_look, n_ins))
        del d_keys, d_ins, d_look, d_ret, d_out
    return out


def batched_ops(args, G, torch, dev, stream, flush, peak):
    """256 independent filters (q uniform in [12, 22], fill in [0.5, 0.9],
    Pareto(1.5) lookup batches, MT19937 seed 4 substreams): every filter
    bulk built (NoDup) and then queried, (a) as one batch -- the whole
    pipeline as one persistent cooperative kernel or one launch per pipeline
    kernel replayed from a CUDA graph, form and launch shape from the
    autotuner -- and (b) one bulkBuildSegmentedLayouts +
    launchUnsortedLookups call per filter.  Both timed with CUDA events on
    the stream, L2 flushed before each repetition; the tables of (a) and (b)
    are compared."""
    from gpuquotientfilters_gb300 import autotune
    from gpuquotientfilters_gb300 import workload as W
    c = W.config4()

    def dev_u32(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)

    jobs, jobs_ref = [], []
    for f in c:
        dk, dl = dev_u32(f["keys"]), dev_u32(f["lookups"])
        res = torch.empty(f["lookups"].size, dtype=torch.int32, device=dev)
        jobs.append((G.initFilterGPU(f["q"], 5), dk, dl, res))
        jobs_ref.append((G.initFilterGPU(f["q"], 5), dk, dl, torch.empty_like(res)))
    choice, sweep = autotune.tune(G, jobs, True, use_cache=False, cache=None, stream=stream)
    b = autotune.make_batch(G, jobs, True, choice)

    def timed(fn):
        out = []
        for it in range(args.warmup + args.steps):
            flush.fill_(1)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            fn()
            ev1.record(stream)
            ev1.synchronize()
            if it >= args.warmup:
                out.append(ev0.elapsed_time(ev1))
        return float(np.mean(out))

    launches0 = G.lib().gqf_kernel_launches()
    ms_batch = timed(lambda: autotune.run_batch(b, choice, stream))
    batch_launches = (G.lib().gqf_kernel_launches() - launches0) // (args.warmup + args.steps)

    def per_filter():
        for (qf, dk, dl, res) in jobs_ref:
            G.bulkBuildSegmentedLayouts(qf, dk.numel(), dk, True, stream=stream)
            G.launchUnsortedLookups(qf, dl.numel(), dl, res, stream=stream)

    launches0 = G.lib().gqf_kernel_launches()
    ms_plain = timed(per_filter)
    plain_launches = (G.lib().gqf_kernel_launches() - launches0) // (args.warmup + args.steps)
    same = all(torch.equal(j[3], r[3]) for j, r in zip(jobs, jobs_ref)) and all(
        np.array_equal(G.table_bytes(j[0]), G.table_bytes(r[0])) for j, r in zip(jobs[:16], jobs_ref[:16]))
    n_keys = sum(f["keys"].size for f in c)
    n_look = sum(f["lookups"].size for f in c)
    T = sum(G.calcNumSlotsGPU(f["q"], 5) for f in c)
    nbytes = 12.0 * n_keys + T + 40.0 * n_look
    b.close()
    for j in jobs + jobs_ref:
        G.freeFilterGPU(j[0])
    gbs = nbytes / (ms_batch / 1e3) / 1e9
    return {"workload": "256 SQFs r=5, q U[12,22], fill U[0.5,0.9], NoDup build + Pareto(1.5) lookups in "
                        "[2^8,2^20] (50% positive), MT19937 seed 4 substreams",
            "keys": int(n_keys), "lookups": int(n_look),
            "batched_ms": round(ms_batch, 4), "per_filter_calls_ms": round(ms_plain, 4),
            "speedup": round(ms_plain / ms_batch, 2), "mops": round((n_keys + n_look) / ms_batch / 1e3, 1),
            "alg_GBps": round(gbs, 1), "frac_hbm": round(gbs / peak, 4), "tuning": choice,
            "best_graph_ms": round(min(v for k, v in sweep.items() if k[0] == "graph"), 4),
            "best_persistent_ms": round(min([v for k, v in sweep.items() if k[0] == "persistent"] or [0.0]), 4),
            "tuning_sweep_ms": {autotune.label(k): round(v, 4) for k, v in sweep.items()},
            "launches_batched": int(batch_launches), "launches_per_filter": int(plain_launches),
            "results_identical": bool(same)}


def served_ops(args, G, torch, dev):
    """Served stream (64 resident r=5 filters, q in [16,24], fill 0.6; 400
    requests of log-uniform size in [2^8, 2^20], 70% lookups / 20% inserts /
    10% deletes, Zipf(1.1) keys over 2^30, deletes of present keys): the
    continuous-batching server against the plain path (each request in turn:
    copy keys in, one synchronous API call, copy results out), both from
    pinned host buffers, wall-clock timed.  Saturation: all requests offered
    at once.  Latency: Poisson arrivals at fractions of the saturation rate
    (filters rebuilt before each run).  Results and final tables of the
    saturation run are compared with the plain path's."""
    import time as _t
    from gpuquotientfilters_gb300 import workload as W
    filters, reqs = W.config5()
    budget = 8 << 30

    def build_all():
        qfs = [G.initFilterGPU(f["q"], 5) for f in filters]
        keys = [torch.from_numpy(f["keys"].view(np.int32)).to(dev) for f in filters]
        b = G.Batch([(qf, k, None, None) for qf, k in zip(qfs, keys)], True)
        b.run()
        b.close()
        torch.cuda.synchronize(dev)
        return qfs

    h_keys = [torch.from_numpy(r["keys"].view(np.int32)).pin_memory() for r in reqs]
    nkeys = sum(r["keys"].size for r in reqs)

    def new_outs():
        return [torch.zeros(max(r["keys"].size, 1), dtype=torch.int32).pin_memory() if r["op"] == 0 else None
                for r in reqs]

    def run_served(qfs, outs, arrivals=None):
        srv = G.Server(qfs, hbm_budget=budget)
        info = srv.info()
        t0 = _t.perf_counter()
        for i, (r, k, o) in enumerate(zip(reqs, h_keys, outs)):
            if arrivals is not None:
                while _t.perf_counter() - t0 < arrivals[i]:
                    pass
            srv.submit(r["filter"], r["op"], k, o)
        srv.drain()
        wall = _t.perf_counter() - t0
        done = srv.poll(len(reqs) + 16)
        srv.close()
        lat = np.array([d["done_us"] - d["submit_us"] for d in done])
        return wall, lat, info, all(d["status"] == 0 for d in done)

    # saturation
    served_q = build_all()
    outs_s = new_outs()
    wall_s, lat_s, info, ok_s = run_served(served_q, outs_s)
    # plain path on a second copy
    plain_q = build_all()
    outs_p = new_outs()
    d_keys = torch.empty(max(r["keys"].size for r in reqs), dtype=torch.int32, device=dev)
    d_out = torch.empty_like(d_keys)
    lat_p = []
    t0 = _t.perf_counter()
    for r, k, o in zip(reqs, h_keys, outs_p):
        ts = _t.perf_counter()
        n = r["keys"].size
        d_keys[:n].copy_(k)
        qf = plain_q[r["filter"]]
        if r["op"] == 0:
            G.launchUnsortedLookups(qf, n, d_keys, d_out)
            o[:n].copy_(d_out[:n])
        elif r["op"] == 1:
            G.insert(qf, n, d_keys)
        else:
            G.superclusterDeletes(qf, n, d_keys)
        lat_p.append((_t.perf_counter() - t0) * 1e6)  # all offered at t0: completion time = latency
    wall_p = _t.perf_counter() - t0
    same = all(torch.equal(a, b) for a, b in zip(outs_s, outs_p) if a is not None) and all(
        np.array_equal(G.table_bytes(a), G.table_bytes(b)) for a, b in zip(served_q, plain_q))
    for qf in served_q + plain_q:
        G.freeFilterGPU(qf)
    sat_rps = len(reqs) / wall_s
    sweep = []
    rng = np.random.Generator(np.random.PCG64(55))
    for frac in (0.25, 0.5, 0.75):
        rate = frac * sat_rps
        arr = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
        qfs = build_all()
        wall, lat, _, ok = run_served(qfs, new_outs(), arr)
        for qf in qfs:
            G.freeFilterGPU(qf)
        sweep.append({"offered_req_per_s": round(rate, 1), "achieved_Mkeys_per_s": round(nkeys / wall / 1e6, 1),
                      "p50_ms": round(float(np.percentile(lat, 50)) / 1e3, 3),
                      "p99_ms": round(float(np.percentile(lat, 99)) / 1e3, 3), "ok": bool(ok)})
    return {"workload": "64 SQFs r=5 q U[16,24] fill 0.6; 400 requests log-uniform [2^8,2^20] keys, 70/20/10 "
                        "lookup/insert/delete, Zipf(1.1) over 2^30, seed 5; HBM budget 8 GiB",
            "requests": len(reqs), "keys": int(nkeys), "streams": info["streams"],
            "hbm_bytes": info["hbm_bytes"],
            "served_Mkeys_per_s": round(nkeys / wall_s / 1e6, 1), "plain_Mkeys_per_s": round(nkeys / wall_p / 1e6, 1),
            "throughput_ratio": round(wall_p / wall_s, 2),
            "saturation_p50_ms": round(float(np.percentile(lat_s, 50)) / 1e3, 3),
            "saturation_p99_ms": round(float(np.percentile(lat_s, 99)) / 1e3, 3),
            "plain_p50_ms": round(float(np.percentile(lat_p, 50)) / 1e3, 3),
            "plain_p99_ms": round(float(np.percentile(lat_p, 99)) / 1e3, 3),
            "poisson_sweep": sweep, "results_identical": bool(same and ok_s)}


def e2e_step(args, G, torch, dev, stream, c, qf):
    """The same step from pinned host memory: copies in, ops, results out.

    Copies run on their own streams and overlap the ops, as a serving host
    would run them: a step's inputs go up on the copy stream (double-buffered,
    so the next step's inputs load while this step computes), each op waits
    only for its own input, and each lookup's results come back on a third
    stream while the later ops run.  The ops are queued asynchronously
    (sync=False: the C ABI with no timing pointer), so the host runs ahead of
    the device.  The timed region runs from before the first copy to after
    the last result is on the host."""
    def pinned(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).pin_memory()

    h_keys, h_look, h_ins, h_del = pinned(c["keys"]), pinned(c["lookups"]), pinned(c["inserts"]), pinned(c["deletes"])
    h_out = torch.empty(N_LOOKUP, dtype=torch.int32).pin_memory()
    h_out2 = torch.empty(N_LOOKUP, dtype=torch.int32).pin_memory()
    up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def buffers():
        b = {k: torch.empty(n, dtype=torch.int32, device=dev)
             for k, n in (("keys", N_KEYS), ("look", N_LOOKUP), ("ins", N_INSERT), ("del", N_DELETE),
                          ("out", N_LOOKUP), ("out2", N_LOOKUP))}
        b["free"] = torch.cuda.Event()      # the ops are done with the inputs
        b["fetched"] = torch.cuda.Event()   # the results are on the host
        b["free"].record(stream)
        b["fetched"].record(down)
        return b

    bufs = [buffers(), buffers()]
    bi = 4 * (N_KEYS + N_LOOKUP + N_INSERT + N_DELETE)
    bo = 4 * 2 * N_LOOKUP

    pending = {}

    def load(step):
        """Issue step's input copies (the host does not wait for them)."""
        b = bufs[step % 2]
        ev = {k: torch.cuda.Event() for k in ("keys", "look", "ins", "del")}
        up.wait_event(b["free"])
        with torch.cuda.stream(up):
            for name, h in (("keys", h_keys), ("look", h_look), ("ins", h_ins), ("del", h_del)):
                b[name].copy_(h, non_blocking=True)
                ev[name].record(up)
        pending[step] = ev

    def run(step):
        b, ev = bufs[step % 2], pending.pop(step)
        lu, ls = torch.cuda.Event(), torch.cuda.Event()
        stream.wait_event(ev["keys"])
        G.bulkBuildSegmentedLayouts(qf, N_KEYS, b["keys"], True, stream=stream, sync=False)
        stream.wait_event(ev["look"])
        stream.wait_event(b["fetched"])
        G.launchUnsortedLookups(qf, N_LOOKUP, b["look"], b["out"], stream=stream, sync=False)
        lu.record(stream)
        G.launchSortedLookups(qf, N_LOOKUP, b["look"], b["out2"], stream=stream, sync=False)
        ls.record(stream)
        down.wait_event(lu)
        with torch.cuda.stream(down):
            h_out.copy_(b["out"], non_blocking=True)
            down.wait_event(ls)
            h_out2.copy_(b["out2"], non_blocking=True)
            b["fetched"].record(down)
        stream.wait_event(ev["ins"])
        G.insert(qf, N_INSERT, b["ins"], stream=stream, sync=False)
        stream.wait_event(ev["del"])
        G.superclusterDeletes(qf, N_DELETE, b["del"], stream=stream, sync=False)
        b["free"].record(stream)

    def steps(n):
        # the next step's inputs load while this step computes
        load(0)
        for k in range(n):
            if k + 1 < n:
                load(k + 1)
            run(k)

    steps(max(1, args.warmup))
    torch.cuda.synchronize(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    up.wait_event(ev0)
    steps(args.steps)
    stream.wait_event(bufs[(args.steps - 1) % 2]["fetched"])
    ev1.record(stream)
    ev1.synchronize()
    G.stream_status(stream)  # a device-side error of any queued op fails the run
    ms = ev0.elapsed_time(ev1) / args.steps
    ops = N_KEYS + 2 * N_LOOKUP + N_INSERT + N_DELETE
    return {"value": ops / ms / 1e3, "unit": "M ops/s", "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo,
            "ms_per_step": ms, "copies": "overlapped with the ops (copy-in, compute and copy-out streams)"}


# -------------------------------------------------------------- CPU baseline
# The whole step (about 15 s on the host: the build, inserts and deletes are
# sequential, the lookups run on every host thread).
CPU_SAMPLE = dict(q=Q, n_build=N_KEYS, n_lookup=N_LOOKUP, n_insert=N_INSERT, n_delete=N_DELETE)


def _oracle_mixed_lookups(O, keys, n, seed, skip):
    """The lookup batch of workload.mixed_lookups (the same array), drawn
    with the oracle's MT19937 so the CPU legs load nothing of the product."""
    rng = np.random.Generator(np.random.PCG64(seed))
    npos = n // 2
    pos = keys[:npos] if npos == keys.size else keys[rng.choice(keys.size, npos, replace=False)]
    neg = O.mt_keys(seed, n - npos, skip=skip)
    out = np.concatenate([pos, neg]).astype(np.uint32)
    return out[rng.permutation(n)]


def cpu_workload(sample=CPU_SAMPLE):
    import oracle as O
    keys = O.mt_keys(SEED, sample["n_build"])
    look = _oracle_mixed_lookups(O, keys, sample["n_lookup"], SEED, skip=sample["n_build"] + sample["n_insert"])
    ins = O.mt_keys(SEED, sample["n_insert"], skip=sample["n_build"])
    return keys, look, ins, keys[: sample["n_delete"]]


def cpu_sample_run(sample=CPU_SAMPLE, work=None):
    """The oracle port (the sequential algorithm of the reference's
    CPU_version on the GPU table format and hash) on the workload: build by
    sequential insertItem of n_build keys into an empty q-bit table, then the
    lookups (50% present), inserts of fresh keys and deletes of present keys.
    Returns (M ops/s, seconds, description, threads, per-op seconds)."""
    import oracle as O
    q = sample["q"]
    keys, look, ins, dels = work if work is not None else cpu_workload(sample)
    t = O.sqf_new(q, R)
    threads = max(1, os.cpu_count() or 1)
    parts = np.array_split(look, threads)
    per = {}
    t0 = time.perf_counter()
    O.sqf_insert(t, q, R, keys)
    t1 = time.perf_counter()
    # lookups are independent reads of the table: one slice per host thread
    # (the C calls run without the interpreter lock)
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda a: O.sqf_lookup(t, q, R, a), parts))
    t2 = time.perf_counter()
    O.sqf_insert(t, q, R, ins)
    t3 = time.perf_counter()
    O.sqf_delete(t, q, R, dels)
    t4 = time.perf_counter()
    dt = t4 - t0
    per = {"build": {"s": round(t1 - t0, 3), "cores": 1}, "lookup": {"s": round(t2 - t1, 3), "cores": threads},
           "insert": {"s": round(t3 - t2, 3), "cores": 1}, "delete": {"s": round(t4 - t3, 3), "cores": 1}}
    nops = sample["n_build"] + sample["n_lookup"] + sample["n_insert"] + sample["n_delete"]
    desc = ("oracle port: insertItem of %d keys into an empty q=%d r=5 table, %d inserts and %d deletes on one "
            "thread (the reference CPU algorithm shifts in order), %d lookups on %d threads"
            % (sample["n_build"], q, sample["n_insert"], sample["n_delete"], sample["n_lookup"], threads))
    return nops / dt / 1e6, dt, desc, threads, per


def reference_gpu_kernels(args):
    """The reference's own standard-filter GPU kernels (quotientFilter.cu,
    compiled unmodified into oracle/_ref/ref_sqf_gpu.cubin when the reference
    sources were present at build time) on the same q=26 workload, each op
    timed with CUDA events around the whole reference entry point as the
    reference times it (its host-side sorts and scans restated with torch,
    its round loops' host syncs included).  One warm-up and one timed run;
    L2 flushed before each op.  None when the cubin is absent."""
    from oracle import ref_gpu as RG
    if not RG.available():
        return None
    import torch
    keys, look, ins, dels = [RG.device_keys(a) for a in cpu_workload()]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    res = {}
    for it in range(2):
        f = RG.RefFilter(Q, R)
        for name, n, fn in (
                ("build", keys.numel(), lambda: RG.bulk_build_segmented_layouts(f, keys, True)),
                ("lookup_unsorted", look.numel(), lambda: RG.unsorted_lookups(f, look)),
                ("lookup_sorted", look.numel(), lambda: RG.sorted_lookups(f, look)),
                ("insert", ins.numel(), lambda: RG.insert(f, ins)),
                ("delete", dels.numel(), lambda: RG.supercluster_deletes(f, dels))):
            flush.fill_(1)
            torch.cuda.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record()
            fn()
            ev1.record()
            ev1.synchronize()
            if it == 1:
                ms = ev0.elapsed_time(ev1)
                res[name] = {"n": int(n), "ms": round(ms, 3), "mops": round(n / ms / 1e3, 1)}
        del f
    tot_ms = sum(v["ms"] for v in res.values())
    nops = sum(v["n"] for v in res.values())
    res["step"] = {"ms": round(tot_ms, 3), "mops": round(nops / tot_ms / 1e3, 1)}
    res["what"] = ("reference quotientFilter.cu kernels from a cubin; thrust/CUB host steps restated with torch; "
                   "bulkBuildSegmentedLayouts NoDup, launchUnsortedLookups, launchSortedLookups, insert, "
                   "superclusterDeletes; keys and results stay on the device (no copies timed)")
    return res


def run_reference(args, world, rank):
    """The reference arm: the reference's CPU algorithm (the oracle port: the
    reference's own CPU_version sources are not on the GPU machine, and
    binaries compiled from them here are x86 while the GPU machine is Arm) on
    the full q=26 workload, plus the reference's own GPU kernels on the same
    workload as a second comparator."""
    if rank != 0:
        return None
    import oracle as O
    O.build()
    work = cpu_workload()
    for _ in range(args.warmup):
        cpu_sample_run(CPU_SAMPLE, work)
    vals, secs, per = [], 0.0, None
    for _ in range(args.steps):
        v, dt, desc, threads, per = cpu_sample_run(CPU_SAMPLE, work)
        vals.append(v)
        secs += dt
    value = float(np.mean(vals))
    try:
        ref_gpu = reference_gpu_kernels(args)
    except Exception as e:  # the comparator never decides the arm's line
        ref_gpu = {"error": repr(e)[:300]}
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "M ops/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": "SQF q=26 r=5 fill 0.8: build 53,687,091 keys NoDup + 2^24 unsorted + 2^24 sorted "
                                   "lookups (50% positive) + 2^20 inserts + 2^20 deletes",
                       "q": Q, "r": R, "n_keys": N_KEYS, "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": "M ops/s", "cores": threads, "cores_per_op": per,
                             "kind": "port", "sample": desc + " (the whole q=26 step)"},
            "e2e": {"value": value, "unit": "M ops/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_gpu_kernels": ref_gpu}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gqf", choices=["gqf", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--q", type=int, default=Q, help="quotient bits (26 = the benchmark workload; smaller "
                    "values scale every batch by 2^(q-26), for profiling small cases)")
    ap.add_argument("--no-rsqf", dest="rsqf", action="store_false", help="skip the RSQF ops")
    ap.add_argument("--no-batched", dest="batched", action="store_false", help="skip the batched-filter ops")
    ap.add_argument("--no-served", dest="served", action="store_false", help="skip the served-stream ops")
    ap.add_argument("--ops", default="", help="comma list of ops to run (build always runs)")
    args = ap.parse_args()
    world, rank, local = dist_init()
    if args.impl == "reference":
        out = run_reference(args, world, rank)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    r = run_gpu(args, world, rank, local)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        v, dt, desc, threads, per = cpu_sample_run()
        cpu = {"value": v, "unit": "M ops/s", "cores": threads, "cores_per_op": per, "kind": "port",
               "sample": desc, "seconds": round(dt, 2)}
    out = {
        "metric": METRIC, "value": r["value"], "unit": "M ops/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (MT19937 seed 2 keys)",
        "config": {"workload": "SQF q=26 r=5 fill 0.8: build 53,687,091 keys NoDup + 2^24 unsorted + 2^24 sorted "
                               "lookups (50% positive) + 2^20 inserts + 2^20 deletes",
                   "q": Q, "r": R, "n_keys": N_KEYS, "l2": "flushed (256 MB write) before every op",
                   "parallelism": "replicas x%d" % world},
        "per_op": r["per_op"], "roofline": r["roofline"], "cpu_baseline": cpu, "e2e": r["e2e"],
        "clocks": r["clocks"], "gpu_launches": r["gpu_launches"], "rsqf": r["rsqf"], "batched": r["batched"],
        "served": r["served"],
    }
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
