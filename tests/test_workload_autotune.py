"""Host-side logic, no GPU: the workload generators the bench and the tests
draw from, and the batch autotuner's class, candidates and cache."""
import json

import numpy as np

from gpuquotientfilters_gb300 import autotune as A
from gpuquotientfilters_gb300 import workload as W


def test_config2_small_shapes():
    c = W.config2(seed=2, q=14, n=int(0.8 * (1 << 14)), n_insert=1 << 10, n_lookup=1 << 12, n_delete=1 << 10)
    assert c["keys"].dtype == np.uint32 and c["keys"].size == int(0.8 * (1 << 14))
    assert c["inserts"].size == 1 << 10 and c["lookups"].size == 1 << 12 and c["deletes"].size == 1 << 10
    # deletes are present keys; half the lookups are present keys
    assert np.isin(c["deletes"], c["keys"]).all()
    frac = np.isin(c["lookups"], c["keys"]).mean()
    assert 0.45 <= frac <= 0.6


def test_config4_shapes():
    fs = W.config4(seed=4, nfilters=32)
    assert len(fs) == 32
    for f in fs:
        assert 12 <= f["q"] <= 22 and f["r"] == 5 and 0.5 <= f["fill"] <= 0.9
        assert f["keys"].size == int(round(f["fill"] * (1 << f["q"])))
        assert 256 <= f["lookups"].size <= 1 << 20
        assert np.isin(f["lookups"], f["keys"]).sum() >= f["lookups"].size // 2


def test_config5_stream():
    filters, reqs = W.config5(seed=5, nfilters=8, q_lo=12, q_hi=14, nreq=300, size_lo=16, size_hi=4096)
    assert len(filters) == 8 and len(reqs) == 300
    deleted = [set() for _ in filters]
    kinds = np.bincount([r["op"] for r in reqs], minlength=3) / len(reqs)
    assert abs(kinds[0] - 0.7) < 0.1 and abs(kinds[1] - 0.2) < 0.1 and abs(kinds[2] - 0.1) < 0.07
    for r in reqs:
        f = filters[r["filter"]]
        k = r["keys"]
        assert k.dtype == np.uint32 and k.size <= 4096
        if r["op"] == 1:
            assert k.size <= 1 << (f["q"] - 4)  # an insert never overflows its filter
        if r["op"] == 2:  # deletes hit present keys, each at most once
            assert np.isin(k, f["keys"]).all()
            s = set(k.tolist())
            assert not (s & deleted[r["filter"]])
            deleted[r["filter"]] |= s
        else:
            assert (k < (1 << 30)).all()


def test_zipf_keys_are_skewed():
    rng = np.random.Generator(np.random.PCG64(1))
    k = W.zipf_keys(rng, 20000)
    _, counts = np.unique(k, return_counts=True)
    assert counts.max() > 100  # heavy hitters
    assert (k < (1 << 30)).all()


def test_batch_class_and_candidates():
    shapes = [(12, 3000), (16, 50000), (14, 0)]
    cls = A.batch_class(shapes, 5)
    assert cls.startswith("r5:q12-16:")
    assert A.batch_class([(14, 0)], 5) == "r5:lookups-only"
    cands = A.candidates(shapes)
    assert all(c[1] <= 12 for c in cands)  # every rebuilt filter spans whole buckets
    assert {c[2] for c in cands if c[0] == "graph"} == set(A.SCATTER_CHUNKS)
    pers = [c for c in cands if c[0] == "persistent"]
    assert {(c[2], c[3]) for c in pers} == {(t, i) for t in A.CTA_THREADS for i in A.ITEMS_PER_THREAD}
    assert all((1 << c[1]) // c[2] in A.QUOTIENTS_PER_THREAD for c in pers)


class _FakeQF:
    def __init__(self, q):
        self.qbits = q


class _FakeBatch:
    """Stands in for G.Batch: run() returns a time that depends on the shape."""
    calls = []

    def __init__(self, jobs, no_duplicates, bb, ch, threads=0, ipt=0):
        self.bb, self.ch, self.threads, self.ipt = bb, ch, threads, ipt
        _FakeBatch.calls.append((bb, ch, threads, ipt))

    def run(self, use_graph=True, stream=None, persistent=False):
        if persistent:  # the persistent form wins at 256 threads x 32 keys, 12 bucket bits
            return 0.5 + abs(self.bb - 12) + (0.0 if (self.threads, self.ipt) == (256, 32) else 0.3)
        return 1.0 + abs(self.bb - 11) + (0.0 if self.ch == 8192 else 0.5)

    def close(self):
        pass


class _FakeG:
    Batch = _FakeBatch


def test_tune_picks_fastest_and_caches(tmp_path):
    cache = str(tmp_path / "tuning.json")
    jobs = [(_FakeQF(13), (0, 40000), None, None), (_FakeQF(15), (0, 90000), None, None)]
    _FakeBatch.calls = []
    choice, times = A.tune(_FakeG, jobs, cache=cache)
    assert choice == {"mode": "persistent", "bucket_bits": 12, "scatter_chunk": 0, "cta_threads": 256,
                      "items_per_thread": 32}
    assert len(times) == len(A.candidates([(13, 40000), (15, 90000)]))
    table = json.load(open(cache))
    assert list(table.values())[0]["best"] == choice
    # a second batch of the same class starts from the cache without measuring
    _FakeBatch.calls = []
    choice2, times2 = A.tune(_FakeG, jobs, cache=cache)
    assert choice2 == choice and times2 == {} and _FakeBatch.calls == []
