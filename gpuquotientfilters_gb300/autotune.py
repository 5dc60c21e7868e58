"""Launch-shape autotuner for batched filters.

A batch (gqf_batch_*) runs either as one launch per pipeline kernel replayed
from a CUDA graph, or as one persistent cooperative kernel.  The graph form
has two launch parameters: the bucket size of the layout kernel
(bucket_bits: 2^bits quotients per CTA, which sets the CTA width, 2^(bits-5)
threads of 32 quotients each) and the scatter chunk (keys per scatter CTA:
2048, 8192 or 32768, i.e. 256 threads x 8, 256 x 32 or 1024 x 32 items per
thread).  The persistent form has three: the CTA size (128 or 256 threads,
the same for every phase), the keys per thread of a scatter chunk (8 or
32) and the bucket bits (each layout thread owning 16 or 32 quotients).
The best shape depends on the filters' sizes and fills: small filters want
small chunks (fewer idle threads per CTA), large ones want fewer, fuller
CTAs.  tune() times every admissible shape of both forms on the caller's
own batch (CUDA events, after warm-up) and returns the fastest; results are
cached per class of batch -- (r, smallest q, largest q, mean fill to 0.1,
log2 of the key count) -- in a JSON file, so a later batch of the same class
starts from the cached choice without measuring.
"""
from __future__ import annotations

import json
import math
import os

BUCKET_BITS = (10, 11, 12, 13)
SCATTER_CHUNKS = (2048, 8192, 32768)
CTA_THREADS = (128, 256)
ITEMS_PER_THREAD = (8, 32)
QUOTIENTS_PER_THREAD = (16, 32)  # persistent layout threads (compiled shapes)
DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "gpuquotientfilters_gb300", "tuning.json")


def batch_class(shapes, r: int) -> str:
    """shapes: [(q, n_build_keys), ...] of the filters that are rebuilt."""
    qs = [q for q, n in shapes if n > 0]
    if not qs:
        return "r%d:lookups-only" % r
    fills = [n / float(1 << q) for q, n in shapes if n > 0]
    total = sum(n for _, n in shapes)
    return "r%d:q%d-%d:f%.1f:n2^%d" % (r, min(qs), max(qs), sum(fills) / len(fills), int(math.log2(max(total, 1))))


def candidates(shapes):
    """Admissible shapes: ('graph', bucket_bits, scatter_chunk) and
    ('persistent', bucket_bits, cta_threads, items_per_thread)."""
    qmin = min([q for q, n in shapes if n > 0] or [32])
    out = [("graph", bb, ch) for bb in BUCKET_BITS if bb <= qmin for ch in SCATTER_CHUNKS]
    out += [("persistent", bb, t, i) for t in CTA_THREADS for i in ITEMS_PER_THREAD for bb in BUCKET_BITS
            if bb <= qmin and (1 << bb) // t in QUOTIENTS_PER_THREAD]
    return out


def choice_of(cand):
    """The Batch arguments and run mode of a candidate."""
    if cand[0] == "graph":
        return {"mode": "graph", "bucket_bits": cand[1], "scatter_chunk": cand[2], "cta_threads": 0,
                "items_per_thread": 0}
    return {"mode": "persistent", "bucket_bits": cand[1], "scatter_chunk": 0, "cta_threads": cand[2],
            "items_per_thread": cand[3]}


def label(cand):
    return "/".join(str(x) for x in cand)


def make_batch(G, jobs, no_duplicates, choice):
    return G.Batch(jobs, no_duplicates, choice["bucket_bits"], choice["scatter_chunk"], choice["cta_threads"],
                   choice["items_per_thread"])


def run_batch(b, choice, stream=None):
    return b.run(True, stream, persistent=choice["mode"] == "persistent")


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, table):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune(G, jobs, no_duplicates=True, r=5, reps=3, warmup=1, cache=DEFAULT_CACHE, use_cache=True, stream=None):
    """Returns (choice, {candidate: ms}) for the batch `jobs` (the argument of
    gpuquotientfilters_gb300.Batch); choice = {'mode', 'bucket_bits',
    'scatter_chunk', 'cta_threads', 'items_per_thread'}."""
    shapes = [(qf.qbits, 0 if bk is None else (bk[1] if isinstance(bk, tuple) else int(bk.numel())))
              for (qf, bk, _lk, _res) in jobs]
    key = batch_class(shapes, r)
    table = _load(cache) if (cache and use_cache) else {}
    if key in table:
        return dict(table[key]["best"]), {}
    times = {}
    for cand in candidates(shapes):
        choice = choice_of(cand)
        b = make_batch(G, jobs, no_duplicates, choice)
        try:
            for _ in range(warmup):
                run_batch(b, choice, stream)
            times[cand] = min(run_batch(b, choice, stream) for _ in range(reps))
        finally:
            b.close()
    best = min(times, key=times.get)
    choice = choice_of(best)
    if cache:
        table = _load(cache)
        table[key] = {"best": choice, "ms": {label(k): round(v, 4) for k, v in times.items()}}
        _store(cache, table)
    return choice, times
