"""Synthetic workloads of the benchmark configurations (MT19937 keys, as the
reference drivers draw them: init_genrand(seed) then genrand_int32()).

Lookup batches mix inserted keys and further draws and are shuffled with
numpy's PCG64 generator seeded with the config seed (a seeded, documented
permutation; the reference drivers do not shuffle).
"""
from __future__ import annotations

import numpy as np

from . import mt19937


def n_keys(q: int, alpha: float, reference_arithmetic: bool = False) -> int:
    """Key count for fill alpha.  The benchmark counts round alpha*2^q to
    nearest; the reference drivers compute `int numValues = alpha * (1 << q)`
    with a float alpha (e.g. bulkBuildSegmentedLayoutTest.cu:83)."""
    if reference_arithmetic:
        return int(np.float32(alpha) * np.float32(1 << q))
    return int(round(alpha * (1 << q)))


def mixed_lookups(keys: np.ndarray, n: int, seed: int, skip: int) -> np.ndarray:
    """n lookups: n//2 inserted keys (sampled), the rest fresh MT draws
    taken after `skip` draws of the same stream, shuffled."""
    rng = np.random.Generator(np.random.PCG64(seed))
    npos = n // 2
    if npos <= keys.size:
        pos = keys[:npos] if npos == keys.size else keys[rng.choice(keys.size, npos, replace=False)]
    else:
        pos = keys[rng.integers(0, keys.size, npos)]
    neg = mt19937(seed, n - npos, skip=skip)
    out = np.concatenate([pos, neg]).astype(np.uint32)
    return out[rng.permutation(n)]


def config1(seed: int = 1, q: int = 15, r: int = 5, n: int = 19661):
    """Plain SQF: n keys, n mixed lookups, delete the first 4096 keys."""
    keys = mt19937(seed, n)
    look = mixed_lookups(keys, n, seed, skip=n)
    return dict(q=q, r=r, keys=keys, lookups=look, deletes=keys[:4096].copy())


def config2(seed: int = 2, q: int = 26, r: int = 5, n: int = 53687091, n_insert: int = 1 << 20,
            n_lookup: int = 1 << 24, n_delete: int = 1 << 20):
    """SQF at scale: build keys, fresh insert batch (the next draws),
    mixed lookups, deletes of present keys."""
    keys = mt19937(seed, n)
    ins = mt19937(seed, n_insert, skip=n)
    look = mixed_lookups(keys, n_lookup, seed, skip=n + n_insert)
    return dict(q=q, r=r, keys=keys, inserts=ins, lookups=look, deletes=keys[:n_delete].copy())


def config4(seed: int = 4, nfilters: int = 256, q_lo: int = 12, q_hi: int = 22):
    """Batched multi-filter workload: nfilters independent r=5 filters,
    q uniform in [q_lo, q_hi], fill uniform in [0.5, 0.9]; filter i draws its
    keys from MT19937 seeded seed*1000 + i (one substream per filter; its
    next draws are the negative lookups); lookup batch size Pareto(1.5)
    clipped to [2^8, 2^20], 50% positive.  Shapes from numpy PCG64(seed)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(nfilters):
        q = int(rng.integers(q_lo, q_hi + 1))
        fill = float(rng.uniform(0.5, 0.9))
        n = int(round(fill * (1 << q)))
        nl = int(np.clip((rng.pareto(1.5) + 1.0) * 256.0, 256, 1 << 20))
        keys = mt19937(seed * 1000 + i, n + nl - nl // 2)
        pos = keys[rng.integers(0, n, nl // 2)]
        look = np.concatenate([pos, keys[n:]]).astype(np.uint32)
        look = look[rng.permutation(nl)]
        out.append(dict(q=q, r=5, fill=fill, keys=keys[:n].copy(), lookups=look))
    return out


def zipf_keys(rng, n: int, s: float = 1.1, universe_bits: int = 30) -> np.ndarray:
    """n keys from a Zipf(s) law over a 2^universe_bits universe: rank v
    (numpy's zipf sampler, v >= 1) is scrambled by an odd multiplier mod
    2^32 and kept to universe_bits bits, so hot keys are spread over the
    key space."""
    v = rng.zipf(s, n).astype(np.uint64)
    return (((v * np.uint64(0x9E3779B1)) & np.uint64(0xFFFFFFFF)) >> np.uint64(32 - universe_bits)).astype(np.uint32)


def config5(seed: int = 5, nfilters: int = 64, q_lo: int = 16, q_hi: int = 24, fill: float = 0.6,
            nreq: int = 400, size_lo: int = 1 << 8, size_hi: int = 1 << 20, mix=(0.7, 0.2, 0.1)):
    """Served stream: nfilters resident r=5 filters (q uniform in
    [q_lo, q_hi]), each bulk built to `fill` from MT19937 seed*1000+i keys;
    nreq requests, each on a uniformly chosen filter, kind drawn by `mix`
    (lookup, insert, delete), size log-uniform in [size_lo, size_hi].
    Lookup and insert keys are Zipf(1.1) over a 2^30 universe; delete keys
    are present keys (the filter's initial keys, each deleted at most once).
    An insert batch is capped at 2^(q-4) keys of its filter (1/16 of the
    slots), so the smallest filters do not overflow their 1.1 * 2^q slots.
    Shapes and draws from numpy PCG64(seed)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    filters = []
    order, cursor = [], []
    for i in range(nfilters):
        q = int(rng.integers(q_lo, q_hi + 1))
        keys = mt19937(seed * 1000 + i, int(round(fill * (1 << q))))
        filters.append(dict(q=q, r=5, keys=keys))
        order.append(rng.permutation(keys.size))
        cursor.append(0)
    reqs = []
    kinds = rng.choice(3, size=nreq, p=np.asarray(mix, float) / sum(mix))
    for k in kinds:
        f = int(rng.integers(0, nfilters))
        n = int(np.exp(rng.uniform(np.log(size_lo), np.log(size_hi + 1))))
        n = min(max(n, size_lo), size_hi)
        if k == 1:
            n = min(n, 1 << (filters[f]["q"] - 4))
        if k == 2:
            c = cursor[f]
            n = min(n, filters[f]["keys"].size - c)
            keys = filters[f]["keys"][order[f][c:c + n]]
            cursor[f] = c + n
        else:
            keys = zipf_keys(rng, n)
        reqs.append(dict(filter=f, op=int(k), keys=np.ascontiguousarray(keys, np.uint32)))
    return filters, reqs
