"""SQF parity on the GPU: every op through the C ABI, compared with the oracle
(table slot arrays bit-exact, lookup results exact)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as O
from conftest import from_dev, to_dev

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


class Filter:
    def __init__(self, G, torch, q, r):
        self.G, self.torch, self.q, self.r = G, torch, q, r
        self.qf = G.initFilterGPU(q, r)

    def __del__(self):
        try:
            self.G.freeFilterGPU(self.qf)
        except Exception:
            pass

    def build(self, keys, nodup=True):
        return self.G.bulkBuildSegmentedLayouts(self.qf, keys.size, to_dev(self.torch, keys), nodup)

    def slots(self):
        return O.sqf_slots(self.G.table_bytes(self.qf), self.q, self.r)

    def raw(self):
        return self.G.table_bytes(self.qf)

    def lookup(self, keys, sorted_=False):
        out = self.torch.empty(keys.size, dtype=self.torch.int32, device="cuda")
        fn = self.G.launchSortedLookups if sorted_ else self.G.launchUnsortedLookups
        fn(self.qf, keys.size, to_dev(self.torch, keys), out)
        return from_dev(out)

    def insert(self, keys):
        return self.G.insert(self.qf, keys.size, to_dev(self.torch, keys))

    def delete(self, keys):
        return self.G.superclusterDeletes(self.qf, keys.size, to_dev(self.torch, keys))


def oracle_build(q, r, keys, nodup=True):
    t = O.sqf_new(q, r)
    assert O.sqf_bulk_build(t, q, r, keys, nodup) == 0
    return t


def assert_same_table(f, t):
    raw = f.raw()
    if not np.array_equal(raw, t):
        d = np.nonzero(raw != t)[0]
        raise AssertionError("%d bytes differ, first at %d: gpu %s oracle %s" %
                             (d.size, d[0], raw[d[0]:d[0] + 8], t[d[0]:d[0] + 8]))


def test_config1_build_lookup_delete(gqf, cuda):
    from gpuquotientfilters_gb300 import workload as W
    c = W.config1()
    q, r = c["q"], c["r"]
    f = Filter(gqf, cuda, q, r)
    f.build(c["keys"], True)
    t = oracle_build(q, r, c["keys"])
    assert_same_table(f, t)
    g = GOLDEN["sqf_cpu_version"][0]
    assert (g["q"], g["n"]) == (15, 19661)
    assert sha(f.slots().astype(np.uint32)) == g["aphash"]["slots_sha256"]
    want = O.sqf_lookup(t, q, r, c["lookups"])
    assert np.array_equal(f.lookup(c["lookups"]), want)
    assert np.array_equal(f.lookup(c["lookups"], sorted_=True), want)
    f.delete(c["deletes"])
    O.sqf_delete(t, q, r, c["deletes"])
    assert_same_table(f, t)
    assert np.array_equal(f.lookup(c["lookups"]), O.sqf_lookup(t, q, r, c["lookups"]))


@pytest.mark.parametrize("q,r,alpha,seed,nodup", [
    (15, 5, 0.6, 1, False), (12, 5, 0.9, 2, True), (16, 5, 0.95, 3, True), (18, 5, 0.8, 4, False),
    (20, 5, 0.5, 5, True), (14, 13, 0.8, 6, True), (16, 13, 0.9, 7, False), (7, 5, 0.8, 8, True),
    (10, 5, 1.0, 9, True), (22, 5, 0.85, 10, True),
])
def test_build_and_lookups(gqf, cuda, q, r, alpha, seed, nodup):
    n = int(alpha * (1 << q))
    keys = O.mt_keys(seed, n)
    f = Filter(gqf, cuda, q, r)
    f.build(keys, nodup)
    t = oracle_build(q, r, keys, nodup)
    assert_same_table(f, t)
    look = np.concatenate([keys[: n // 2], O.mt_keys(seed, n // 2 + 7, skip=n)])
    want = O.sqf_lookup(t, q, r, look)
    assert np.array_equal(f.lookup(look), want)
    assert np.array_equal(f.lookup(look, sorted_=True), want)
    assert (want[: n // 2] != O.NOT_FOUND).all()
    # a batch under one query per 16 slots takes the other paths (direct walk,
    # bucketed queries): same answers
    m = max(1, O.sqf_num_slots(q) // 32)
    small = np.concatenate([look[: m // 2], look[-(m - m // 2):]])
    ws = O.sqf_lookup(t, q, r, small)
    assert np.array_equal(f.lookup(small), ws)
    assert np.array_equal(f.lookup(small, sorted_=True), ws)


@pytest.mark.parametrize("q,alpha,nodup", [(17, 0.8, True), (19, 0.95, False)])
def test_large_lookups_and_table_alignment(gqf, cuda, q, alpha, nodup):
    """Large one-byte-slot batches go through the bit-plane mirror (its
    records are read and written as 32-byte sectors, the table by bulk
    copies).  A filter whose table is not 16-byte aligned (a drop-in caller's
    own buffer at an odd address) is refused on the host with GQF_ERR_ARG
    before any kernel runs."""
    r = 5
    n = int(alpha * (1 << q))
    keys = O.mt_keys(40 + q, n)
    f = Filter(gqf, cuda, q, r)
    f.build(keys, nodup)
    t = oracle_build(q, r, keys, nodup)
    look = np.concatenate([keys[: n // 2], O.mt_keys(41 + q, n // 2, skip=n)])
    want = O.sqf_lookup(t, q, r, look)
    assert np.array_equal(f.lookup(look), want)
    assert np.array_equal(f.lookup(look, sorted_=True), want)
    # the same table at an offset of 16 bytes answers the same
    T = t.size
    buf = cuda.zeros(T + 64, dtype=cuda.uint8, device="cuda")
    buf[16:16 + T] = cuda.from_numpy(t).cuda()
    moved = gqf.quotient_filter(q, r, 1, buf.data_ptr() + 16)
    out = cuda.empty(look.size, dtype=cuda.int32, device="cuda")
    gqf.launchUnsortedLookups(moved, look.size, to_dev(cuda, look), out)
    assert np.array_equal(from_dev(out), want)
    # an odd address is refused
    odd = gqf.quotient_filter(q, r, 1, buf.data_ptr() + 1)
    for call in (lambda: gqf.launchUnsortedLookups(odd, look.size, to_dev(cuda, look), out),
                 lambda: gqf.launchSortedLookups(odd, look.size, to_dev(cuda, look), out),
                 lambda: gqf.insert(odd, 16, to_dev(cuda, keys[:16])),
                 lambda: gqf.bulkBuildSegmentedLayouts(odd, 16, to_dev(cuda, keys[:16]), True)):
        with pytest.raises(gqf.GQFError) as ei:
            call()
        assert ei.value.status == 1


def test_build_reference_arithmetic_count(gqf, cuda):
    from gpuquotientfilters_gb300 import workload as W
    q, r = 15, 5
    n = W.n_keys(q, 0.6, reference_arithmetic=True)
    keys = O.mt_keys(1, n)
    f = Filter(gqf, cuda, q, r)
    f.build(keys, True)
    assert sha(f.slots().astype(np.uint32)) == GOLDEN["sqf_cpu_version"][1]["aphash"]["slots_sha256"]


def test_build_heavy_duplicates(gqf, cuda):
    q, r = 14, 5
    base = O.mt_keys(11, 2000)
    keys = np.repeat(base, 5)  # every fingerprint 5 times
    keys = np.concatenate([keys, O.mt_keys(12, 3000)])
    for nodup in (False, True):
        f = Filter(gqf, cuda, q, r)
        f.build(keys, nodup)
        assert_same_table(f, oracle_build(q, r, keys, nodup))


def test_build_empty_and_rebuild_clears(gqf, cuda):
    q, r = 12, 5
    f = Filter(gqf, cuda, q, r)
    f.build(O.mt_keys(1, 3000), True)
    f.build(np.zeros(0, np.uint32), True)
    assert not f.raw().any()
    keys = O.mt_keys(2, 1000)
    f.build(keys, True)
    assert_same_table(f, oracle_build(q, r, keys))


def test_build_overfull_reports_full(gqf, cuda):
    q, r = 10, 5
    f = Filter(gqf, cuda, q, r)
    with pytest.raises(gqf.GQFError) as e:
        f.build(O.mt_keys(3, 2000), True)
    assert e.value.status == gqf.GQF_ERR_FULL


def test_invalid_arguments(gqf, cuda):
    with pytest.raises(gqf.GQFError):
        gqf.initFilterGPU(12, 6)  # (r + 3) % 8 != 0
    with pytest.raises(gqf.GQFError):
        gqf.initFilterGPU(27, 5)  # q + r > 31


@pytest.mark.parametrize("q,r,alpha,seed,nodup_build", [(14, 5, 0.6, 21, True), (16, 5, 0.8, 22, False),
                                                        (13, 13, 0.7, 23, True), (18, 5, 0.9, 24, True)])
def test_insert_and_delete(gqf, cuda, q, r, alpha, seed, nodup_build):
    n = int(alpha * (1 << q))
    keys = O.mt_keys(seed, n)
    if not nodup_build:
        keys = np.concatenate([keys, keys[: n // 20]])
    f = Filter(gqf, cuda, q, r)
    f.build(keys, nodup_build)
    t = oracle_build(q, r, keys, nodup_build)
    new = np.concatenate([O.mt_keys(seed, n // 8, skip=n), keys[:100], O.mt_keys(seed, 50, skip=n)])
    f.insert(new)
    O.sqf_insert(t, q, r, new)
    assert_same_table(f, t)
    dels = np.concatenate([keys[: n // 5], new[:200], O.mt_keys(seed + 99, 300), keys[:10]])
    f.delete(dels)
    O.sqf_delete(t, q, r, dels)
    assert_same_table(f, t)
    look = np.concatenate([keys[: n // 4], new])
    assert np.array_equal(f.lookup(look), O.sqf_lookup(t, q, r, look))


@pytest.mark.parametrize("q,nodup_build", [(14, True), (16, False), (18, True)])
def test_insert_and_delete_async(gqf, cuda, q, nodup_build):
    """Asynchronous inserts and deletes (no ms pointer: only enqueued on a
    stream) take the in-place path too; on a table holding duplicate
    fingerprints it cannot place the buckets and the general path queued
    behind it runs instead, decided on the device.  Tables equal the
    oracle's either way; the stream's error latch stays clear."""
    import ctypes as C
    r = 5
    n = int(0.8 * (1 << q))
    keys = O.mt_keys(40 + q, n)
    if not nodup_build:
        keys = np.concatenate([keys, keys[: n // 20]])
    f = Filter(gqf, cuda, q, r)
    f.build(keys, nodup_build)
    t = oracle_build(q, r, keys, nodup_build)
    s = cuda.cuda.Stream()
    sp = C.c_void_p(s.cuda_stream)
    L = gqf.lib()
    # a small insert batch fits the in-place merge; a large one (more new
    # fingerprints per bucket than it holds) goes to the general path directly
    for it, frac in enumerate((64, 8)):
        new = np.concatenate([O.mt_keys(41 + q, max(200, n // frac), skip=n + it * n), keys[:100]])
        dels = np.concatenate([keys[it * n // 10:(it + 1) * n // 10], new[:200], O.mt_keys(42 + q, 300)])
        d_new, d_dels = to_dev(cuda, new), to_dev(cuda, dels)
        cuda.cuda.synchronize()
        assert L.gqf_sqf_insert(C.byref(f.qf), new.size, d_new.data_ptr(), sp, None) == 0
        assert L.gqf_sqf_delete(C.byref(f.qf), dels.size, d_dels.data_ptr(), sp, None) == 0
        s.synchronize()
        assert L.gqf_stream_status(sp) == 0
        O.sqf_insert(t, q, r, new)
        O.sqf_delete(t, q, r, dels)
        assert_same_table(f, t)


def test_insert_into_empty_and_empty_batches(gqf, cuda):
    q, r = 12, 5
    f = Filter(gqf, cuda, q, r)
    t = O.sqf_new(q, r)
    keys = O.mt_keys(5, 2500)
    f.insert(keys)
    O.sqf_insert(t, q, r, keys)
    assert_same_table(f, t)
    f.insert(np.zeros(0, np.uint32))
    f.delete(np.zeros(0, np.uint32))
    assert_same_table(f, t)
    f.delete(keys)
    assert not f.raw().any()


@pytest.mark.parametrize("nodup", [True, False])
def test_insert_via_merge_and_merge_two(gqf, cuda, nodup):
    q, r = 15, 5
    a = O.mt_keys(31, 12000)
    b = np.concatenate([O.mt_keys(32, 9000), a[:500]])
    fa = Filter(gqf, cuda, q, r)
    fa.build(a, False)
    ta = oracle_build(q, r, a, False)
    gqf.insertViaMerge(fa.qf, None, 0, to_dev(cuda, b), b.size, nodup)
    O.sqf_insert_via_merge(ta, q, r, b, nodup)
    assert_same_table(fa, ta)
    f1, f2 = Filter(gqf, cuda, q, r), Filter(gqf, cuda, q, r)
    f1.build(a, True)
    f2.build(b, False)
    t1, t2 = oracle_build(q, r, a, True), oracle_build(q, r, b, False)
    gqf.mergeTwoFilters(f1.qf, f2.qf, nodup)
    O.sqf_merge_two(t1, t2, q, r, nodup)
    assert_same_table(f1, t1)
    assert_same_table(f2, t2)  # second filter untouched


def test_merge_size_mismatch(gqf, cuda):
    f1, f2 = Filter(gqf, cuda, 12, 5), Filter(gqf, cuda, 13, 5)
    with pytest.raises(gqf.GQFError) as e:
        gqf.mergeTwoFilters(f1.qf, f2.qf, True)
    assert e.value.status == gqf.GQF_ERR_MISMATCH


def test_key_equal_to_not_found_sentinel(gqf, cuda):
    """A key of 0xFFFFFFFF is an ordinary key here (the reference's insert
    loop never retires it: superclusterBidding returns before bidding,
    quotientFilter.cu:431-433)."""
    q, r = 12, 5
    keys = np.array([0xFFFFFFFF, 1, 2, 3], np.uint32)
    f = Filter(gqf, cuda, q, r)
    f.insert(keys)
    t = O.sqf_new(q, r)
    O.sqf_insert(t, q, r, keys)
    assert_same_table(f, t)
    assert (f.lookup(keys) != O.NOT_FOUND).all()


def test_config2_full_size_parity(gqf, cuda):
    """q=26, r=5, 53,687,091 keys: the whole 73.8 MB table bit-exact with the
    oracle after the build, a 2^20 insert batch and 2^20 deletes; 2^22 mixed
    lookups exact (sorted and unsorted)."""
    from gpuquotientfilters_gb300 import workload as W
    c = W.config2(n_lookup=1 << 22)
    q, r = c["q"], c["r"]
    f = Filter(gqf, cuda, q, r)
    f.build(c["keys"], True)
    t = oracle_build(q, r, c["keys"], True)
    assert_same_table(f, t)
    want = O.sqf_lookup(t, q, r, c["lookups"])
    assert np.array_equal(f.lookup(c["lookups"]), want)
    assert np.array_equal(f.lookup(c["lookups"], sorted_=True), want)
    f.insert(c["inserts"])
    O.sqf_insert(t, q, r, c["inserts"])
    assert_same_table(f, t)
    f.delete(c["deletes"])
    O.sqf_delete(t, q, r, c["deletes"])
    assert_same_table(f, t)


def test_config2_full_size_dup_parity(gqf, cuda):
    """q=26, r=5, 53,687,091 keys built with duplicates kept (Dup): every
    copy of a repeated fingerprint stored, the whole table bit-exact with the
    oracle; then 2^20 deletes (one copy per occurrence) and a 2^20 insert
    batch (skipping fingerprints already stored), table exact after each."""
    from gpuquotientfilters_gb300 import workload as W
    c = W.config2(n_lookup=1 << 16)
    q, r = c["q"], c["r"]
    f = Filter(gqf, cuda, q, r)
    f.build(c["keys"], False)
    t = oracle_build(q, r, c["keys"], False)
    fps = O.aphash(c["keys"], q, r)
    assert np.unique(fps).size < fps.size  # the build does hold duplicates
    assert_same_table(f, t)
    want = O.sqf_lookup(t, q, r, c["lookups"])
    assert np.array_equal(f.lookup(c["lookups"]), want)
    f.delete(c["deletes"])
    O.sqf_delete(t, q, r, c["deletes"])
    assert_same_table(f, t)
    f.insert(c["inserts"])
    O.sqf_insert(t, q, r, c["inserts"])
    assert_same_table(f, t)


def test_skewed_bucket_set_semantics(gqf, cuda):
    """Thousands of fingerprints in one narrow quotient range (one bucket far
    over its average): the set-semantics paths handle any bucket size."""
    q, r = 16, 5
    cand = O.mt_keys(77, 400000)
    fps = O.aphash(cand, q, r)
    sel = cand[(fps >> r) < 3000][:2500]  # quotients 0..2999, ~0.83 per slot
    keys = np.concatenate([sel, O.mt_keys(78, 20000)])
    f = Filter(gqf, cuda, q, r)
    f.build(keys, True)
    t = oracle_build(q, r, keys, True)
    assert_same_table(f, t)
    more = cand[(fps >> r) < 3000][2500:3000]
    f.insert(more)
    O.sqf_insert(t, q, r, more)
    assert_same_table(f, t)
    f.delete(sel[:1000])
    O.sqf_delete(t, q, r, sel[:1000])
    assert_same_table(f, t)


def test_python_async_calls(gqf, cuda):
    """sync=False queues each op on the stream without waiting (the C ABI
    with no timing pointer); stream_status() then reports any deferred
    device-side error.  The results equal the synchronous calls' (oracle)."""
    q, r = 16, 5
    n = int(0.8 * (1 << q))
    keys = O.mt_keys(91, n)
    look = np.concatenate([keys[: n // 2], O.mt_keys(92, n // 2)])
    ins, dels = O.mt_keys(93, 3000), keys[:2000].copy()
    s = cuda.cuda.Stream()
    qf = gqf.initFilterGPU(q, r)
    try:
        out = cuda.empty(look.size, dtype=cuda.int32, device="cuda")
        dk, dl, di, dd = to_dev(cuda, keys), to_dev(cuda, look), to_dev(cuda, ins), to_dev(cuda, dels)
        cuda.cuda.synchronize()
        assert gqf.bulkBuildSegmentedLayouts(qf, keys.size, dk, True, stream=s, sync=False) is None
        gqf.launchUnsortedLookups(qf, look.size, dl, out, stream=s, sync=False)
        gqf.insert(qf, ins.size, di, stream=s, sync=False)
        gqf.superclusterDeletes(qf, dels.size, dd, stream=s, sync=False)
        gqf.stream_status(s)
        t = oracle_build(q, r, keys)
        assert np.array_equal(from_dev(out), O.sqf_lookup(t, q, r, look))
        O.sqf_insert(t, q, r, ins)
        O.sqf_delete(t, q, r, dels)
        assert np.array_equal(gqf.table_bytes(qf), t)
    finally:
        gqf.freeFilterGPU(qf)
