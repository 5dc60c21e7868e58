"""Batched filters (one launch per pipeline kernel for many filters, CUDA
graph replay, or the whole pipeline as one persistent cooperative kernel):
every filter's table and lookup results are identical to the oracle's and to
the single-filter API's, for every launch shape."""
import numpy as np
import pytest

import oracle as O
from conftest import from_dev, to_dev

pytestmark = pytest.mark.gpu


def make_jobs(G, torch, spec, seed, r=5, nodup=True):
    rng = np.random.default_rng(seed)
    jobs, host = [], []
    for i, (q, fill, nlook) in enumerate(spec):
        n = int(fill * (1 << q))
        keys = O.mt_keys(seed * 1000 + i, n)
        if not nodup:
            keys = np.concatenate([keys, keys[: n // 7]])
        look = np.concatenate([keys[: nlook // 2], O.mt_keys(seed * 1000 + i, nlook - nlook // 2, skip=n)])
        look = look[rng.permutation(look.size)] if look.size else look
        qf = G.initFilterGPU(q, r)
        dk = to_dev(torch, keys) if n else None
        dl = to_dev(torch, look) if nlook else None
        res = torch.empty(max(nlook, 1), dtype=torch.int32, device="cuda") if nlook else None
        jobs.append((qf, dk, dl, res))
        host.append((q, keys, look))
    return jobs, host


def check(G, torch, jobs, host, r=5, nodup=True):
    for (qf, dk, dl, res), (q, keys, look) in zip(jobs, host):
        t = O.sqf_new(q, r)
        if keys.size:
            O.sqf_bulk_build(t, q, r, keys, nodup)
        assert np.array_equal(G.table_bytes(qf), t), "table of q=%d" % q
        if look.size:
            assert np.array_equal(from_dev(res)[: look.size], O.sqf_lookup(t, q, r, look)), "lookups of q=%d" % q


SPEC = [(12, 0.5, 300), (13, 0.9, 5000), (17, 0.7, 20000), (12, 0.85, 0), (15, 0.6, 256), (16, 0.9, 70000),
        (14, 0.75, 1000), (18, 0.55, 3000), (12, 0.9, 4096), (13, 0.5, 1)]


@pytest.mark.parametrize("bucket_bits,chunk", [(0, 0), (10, 2048), (11, 32768), (12, 8192)])
def test_batch_build_and_lookup(gqf, cuda, bucket_bits, chunk):
    G, torch = gqf, cuda
    jobs, host = make_jobs(G, torch, SPEC, 4)
    b = G.Batch(jobs, True, bucket_bits, chunk)
    for use_graph in (True, False, True):
        b.run(use_graph)
        check(G, torch, jobs, host)
    b.close()
    for qf, *_ in jobs:
        G.freeFilterGPU(qf)


def check_tables(G, jobs, want, look_want):
    for (qf, dk, dl, res), t, lw in zip(jobs, want, look_want):
        assert np.array_equal(G.table_bytes(qf), t)
        if lw is not None:
            assert np.array_equal(from_dev(res)[: lw.size], lw)


# nearly full filters included: (13, 0.95) and, with duplicates, more items than quotients
SPEC_P = [(12, 0.5, 300), (13, 0.95, 5000), (12, 0.85, 0), (15, 0.6, 256), (16, 0.9, 7000), (14, 0.75, 1000),
          (12, 0.9, 4096), (13, 0.5, 1)]


@pytest.mark.parametrize("threads,ipt,bucket_bits", [(256, 32, 13), (256, 8, 12), (128, 32, 12), (128, 8, 11)])
@pytest.mark.parametrize("nodup", [True, False])
def test_batch_persistent(gqf, cuda, threads, ipt, bucket_bits, nodup):
    """The whole pipeline as one cooperative launch: same tables and results
    as the oracle, run after run, interleaved with the graph replay.  With
    duplicates some filters hold more items than quotients, so most of their
    buckets start in the previous bucket's spill and their occupied-bit
    fix-up list overflows: the filter's bits are then set from its items."""
    G, torch = gqf, cuda
    spec = [s for s in SPEC_P if s[0] >= bucket_bits]
    jobs, host = make_jobs(G, torch, spec, 8 + threads + ipt, nodup=nodup)
    want, look_want = [], []
    for q, keys, look in host:
        t = O.sqf_new(q, 5)
        assert O.sqf_bulk_build(t, q, 5, keys, nodup) == 0
        want.append(t)
        look_want.append(O.sqf_lookup(t, q, 5, look) if look.size else None)
    b = G.Batch(jobs, nodup, bucket_bits, 0, threads, ipt)
    assert b.tuning()["cta_threads"] == threads and b.tuning()["items_per_thread"] == ipt
    for persistent in (True, False, True):
        b.run(True, persistent=persistent)
        check_tables(G, jobs, want, look_want)
    b.close()
    for qf, *_ in jobs:
        G.freeFilterGPU(qf)


def test_batch_persistent_r13_and_lookup_only(gqf, cuda):
    G, torch = gqf, cuda
    spec = [(13, 0.7, 2000), (14, 0.8, 3000), (12, 0.6, 0)]
    jobs, host = make_jobs(G, torch, spec, 9, r=13)
    G.Batch(jobs, True).run(persistent=True)
    check(G, torch, jobs, host, r=13)
    jobs2 = [(qf, None, dl, torch.empty(max(1, dl.numel() if dl is not None else 1), dtype=torch.int32,
                                        device="cuda") if dl is not None else None)
             for (qf, dk, dl, res) in jobs]
    G.Batch(jobs2, True).run(persistent=True)
    for (qf, _, dl, res2), (q, keys, look) in zip(jobs2, host):
        if look.size:
            t = O.sqf_new(q, 13)
            O.sqf_bulk_build(t, q, 13, keys, True)
            assert np.array_equal(from_dev(res2)[: look.size], O.sqf_lookup(t, q, 13, look))


def test_batch_persistent_shape_not_compiled(gqf, cuda):
    """A shape whose layout threads would own 64 quotients has no persistent
    kernel: the graph replay still runs, the persistent mode is refused."""
    G, torch = gqf, cuda
    jobs, host = make_jobs(G, torch, [(14, 0.6, 500)], 10)
    b = G.Batch(jobs, True, 13, 0, 128, 32)
    b.run(True)
    check(G, torch, jobs, host)
    with pytest.raises(G.GQFError):
        b.run(True, persistent=True)
    b.close()


def test_batch_equals_single_filter_api(gqf, cuda):
    G, torch = gqf, cuda
    spec = [(14, 0.8, 2000), (16, 0.6, 9000), (12, 0.9, 100)]
    jobs, host = make_jobs(G, torch, spec, 5)
    G.Batch(jobs, True).run()
    for (qf, dk, dl, res), (q, keys, look) in zip(jobs, host):
        qf2 = G.initFilterGPU(q, 5)
        G.bulkBuildSegmentedLayouts(qf2, keys.size, dk, True)
        assert np.array_equal(G.table_bytes(qf2), G.table_bytes(qf))
        out = torch.empty(look.size, dtype=torch.int32, device="cuda")
        G.launchUnsortedLookups(qf2, look.size, dl, out)
        assert np.array_equal(from_dev(out), from_dev(res)[: look.size])
        G.freeFilterGPU(qf2)


def test_batch_dup_and_lookup_only_filters(gqf, cuda):
    G, torch = gqf, cuda
    spec = [(13, 0.7, 3000), (15, 0.8, 6000), (12, 0.6, 500)]
    jobs, host = make_jobs(G, torch, spec, 6, nodup=False)
    G.Batch(jobs, False).run()
    check(G, torch, jobs, host, nodup=False)
    # a second batch that only looks up in the built filters (no build keys)
    jobs2 = [(qf, None, dl, torch.empty(res.numel(), dtype=torch.int32, device="cuda")) for (qf, dk, dl, res) in jobs]
    G.Batch(jobs2, False).run()
    for (qf, _, dl, res2), (q, keys, look) in zip(jobs2, host):
        t = O.sqf_new(q, 5)
        O.sqf_bulk_build(t, q, 5, keys, False)
        assert np.array_equal(from_dev(res2)[: look.size], O.sqf_lookup(t, q, 5, look))


def test_batch_r13(gqf, cuda):
    G, torch = gqf, cuda
    spec = [(13, 0.7, 2000), (14, 0.8, 3000)]
    jobs, host = make_jobs(G, torch, spec, 7, r=13)
    G.Batch(jobs, True).run()
    check(G, torch, jobs, host, r=13)


def test_batch_rejects_bad_jobs(gqf, cuda):
    G, torch = gqf, cuda
    a, b = G.initFilterGPU(12, 5), G.initFilterGPU(12, 13)
    k = to_dev(torch, O.mt_keys(1, 100))
    with pytest.raises(G.GQFError):
        G.Batch([(a, k, None, None), (b, k, None, None)])  # mixed r
    with pytest.raises(G.GQFError):
        G.Batch([(a, k, None, None)], True, 13)  # q below the bucket bits
