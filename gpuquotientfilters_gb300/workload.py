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
