"""RSQF parity on the GPU: packed blocks byte-identical to the oracle (the
reference CPU_version restated, pinned by its golden digests) after every
insert batch, return slots identical, lookups identical."""
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


class RSQF:
    def __init__(self, G, torch, q, rbits=5):
        self.G, self.torch, self.q = G, torch, q
        self.cqf = G.initCQFGPU(q, rbits)

    def __del__(self):
        try:
            self.G.freeCQFGPU(self.cqf)
        except Exception:
            pass

    def insert(self, keys):
        ret = self.torch.empty(max(keys.size, 1), dtype=self.torch.int32, device="cuda")
        self.G.insertGPU(self.cqf, keys.size, to_dev(self.torch, keys), ret)
        return ret.cpu().numpy()[: keys.size]

    def lookup(self, keys, sorted_=True):
        out = self.torch.empty(keys.size, dtype=self.torch.int32, device="cuda")
        fn = self.G.launchLookups if sorted_ else self.G.launchUnsortedLookupsRSQF
        fn(self.cqf, keys.size, to_dev(self.torch, keys), out)
        return out.cpu().numpy()

    def blocks(self):
        return self.G.rsqf_blocks_bytes(self.cqf)


def assert_same_blocks(g, o, bb=57):
    if not np.array_equal(g, o):
        d = np.nonzero(g != o)[0]
        raise AssertionError("%d bytes differ, first at %d (block %d byte %d)" % (d.size, d[0], d[0] // bb, d[0] % bb))


@pytest.mark.parametrize("case", GOLDEN["rsqf_cpu_version"], ids=lambda c: "q%d_n%d" % (c["q"], c["n"]))
def test_rsqf_golden(gqf, cuda, case):
    q, n, batch, seed = case["q"], case["n"], case["batch"], case["seed"]
    f = RSQF(gqf, cuda, q)
    keys = O.mt_keys(seed, n)
    ret = f.insert(keys)
    assert sha(f.blocks()) == case["build_blocks_sha256"]
    assert sha(ret) == case["build_rets_sha256"]
    bret = f.insert(O.mt_keys(seed, batch, skip=n))
    assert sha(f.blocks()) == case["batch_blocks_sha256"]
    assert sha(bret) == case["batch_rets_sha256"]
    look = np.concatenate([keys[: case["lookup_n"] // 2],
                           O.mt_keys(seed, case["lookup_n"] - case["lookup_n"] // 2, skip=n)]).astype(np.uint32)
    assert sha(f.lookup(look)) == case["lookup_sha256"]


@pytest.mark.parametrize("q,alpha,seed", [(10, 0.9, 1), (12, 0.5, 2), (14, 0.9, 3), (16, 0.9, 4), (12, 0.92, 5),
                                          (18, 0.9, 6), (13, 0.96, 7)])
def test_rsqf_build_and_batches(gqf, cuda, q, alpha, seed):
    """Fills stay below capacity (the reference's run-end search has no bound
    past it, RSQF.cpp:444-454)."""
    n = int(alpha * (1 << q))
    keys = O.mt_keys(seed, n)
    f = RSQF(gqf, cuda, q)
    o = O.rsqf_new(q)
    ret = f.insert(keys)
    want = O.rsqf_insert_sorted(o, q, keys)
    assert_same_blocks(f.blocks(), o)
    assert np.array_equal(ret, want)
    for k in range(2):  # incremental batches (order-sensitive reference code)
        b = O.mt_keys(seed + 10 + k, max(64, n // 64))
        ret = f.insert(b)
        want = O.rsqf_insert_sorted(o, q, b)
        assert_same_blocks(f.blocks(), o)
        assert np.array_equal(ret, want)
    look = np.concatenate([keys[: n // 2], O.mt_keys(seed + 20, n // 2)])
    want = O.rsqf_lookup(o, q, look)
    assert np.array_equal(f.lookup(look, sorted_=True), want)
    assert np.array_equal(f.lookup(look, sorted_=False), want)
    # under one query per 16 slots the sorted call groups the queries by block
    small = look[: max(1, (1 << q) // 32)]
    assert np.array_equal(f.lookup(small, sorted_=True), O.rsqf_lookup(o, q, small))


def test_rsqf_duplicates_and_empty_batch(gqf, cuda):
    q = 12
    keys = O.mt_keys(7, 1500)
    keys = np.concatenate([keys, keys[:300], keys[:50]])  # RSQF stores duplicates
    f = RSQF(gqf, cuda, q)
    o = O.rsqf_new(q)
    assert np.array_equal(f.insert(keys), O.rsqf_insert_sorted(o, q, keys))
    assert_same_blocks(f.blocks(), o)
    assert f.insert(np.zeros(0, np.uint32)).size == 0
    assert_same_blocks(f.blocks(), o)


def test_rsqf_overfull(gqf, cuda):
    """Past capacity items that cannot be placed get -1.  (The reference
    returns -1 on some of these paths and reads outside its block array on
    others; the engine and the oracle bound every search at the guard
    block.)"""
    q = 8
    keys = O.mt_keys(9, 400)  # 256 quotients + 64 spare slots
    f = RSQF(gqf, cuda, q)
    o = O.rsqf_new(q)
    ret = f.insert(keys)
    want = O.rsqf_insert_sorted(o, q, keys)
    assert (want < 0).any()
    assert np.array_equal(ret, want)
    assert_same_blocks(f.blocks(), o)


@pytest.mark.parametrize("q,seed", [(12, 31), (14, 32), (16, 33)])
def test_rsqf_long_spills_replayed(gqf, cuda, q, seed):
    """Hot quotient ranges push block offsets past 62, where the reference's
    findFirstUnusedSlot departs from the canonical positions: those clusters
    go through the exact replay, the rest is written from positions."""
    cand = O.mt_keys(seed, 60 << q >> 6 << 6)
    fps = O.aphash(cand, q, 5)
    hot = []
    for k in range(4):
        lo = (k + 1) * (1 << q) // 5
        hot.append(cand[((fps >> 5) >= lo) & ((fps >> 5) < lo + 40)][:150 + 20 * k])
    keys = np.concatenate([O.mt_keys(seed + 1, int(0.6 * (1 << q)))] + hot)
    f = RSQF(gqf, cuda, q)
    o = O.rsqf_new(q)
    ret = f.insert(keys)
    want = O.rsqf_insert_sorted(o, q, keys)
    assert_same_blocks(f.blocks(), o)
    assert np.array_equal(ret, want)
    more = np.concatenate([O.mt_keys(seed + 2, 1 << (q - 5)), hot[0][:30]])
    assert np.array_equal(f.insert(more), O.rsqf_insert_sorted(o, q, more))
    assert_same_blocks(f.blocks(), o)


def test_rsqf_config3_full_size(gqf, cuda):
    """q=26, 60,397,976 MT19937 seed-3 keys (fill 0.9) into an empty filter:
    all 59.8 MB of blocks and every return slot identical to the sequential
    reference semantics; then 2^20 incremental inserts and 2^22 lookups."""
    from gpuquotientfilters_gb300 import workload as W
    q = 26
    n = W.n_keys(q, 0.9, reference_arithmetic=True)
    keys = O.mt_keys(3, n + (1 << 20))
    f = RSQF(gqf, cuda, q)
    o = O.rsqf_new(q)
    ret = f.insert(keys[:n])
    want = O.rsqf_insert_sorted(o, q, keys[:n])
    assert_same_blocks(f.blocks(), o)
    assert np.array_equal(ret, want)
    ret = f.insert(keys[n:])
    want = O.rsqf_insert_sorted(o, q, keys[n:])
    assert_same_blocks(f.blocks(), o)
    assert np.array_equal(ret, want)
    look = W.mixed_lookups(keys[:n], 1 << 22, 3, skip=n + (1 << 20))
    assert np.array_equal(f.lookup(look), O.rsqf_lookup(o, q, look))


@pytest.mark.parametrize("case", GOLDEN["rsqf8_cpu_version"], ids=lambda c: "q%d_n%d" % (c["q"], c["n"]))
def test_rsqf8_golden(gqf, cuda, case):
    """8-bit remainders (81-byte blocks): the digests of the reference
    CPU_version compiled with RBITS 8."""
    q, n, batch, seed = case["q"], case["n"], case["batch"], case["seed"]
    f = RSQF(gqf, cuda, q, 8)
    keys = O.mt_keys(seed, n)
    ret = f.insert(keys)
    assert sha(f.blocks()) == case["build_blocks_sha256"]
    assert sha(ret) == case["build_rets_sha256"]
    bret = f.insert(O.mt_keys(seed, batch, skip=n))
    assert sha(f.blocks()) == case["batch_blocks_sha256"]
    assert sha(bret) == case["batch_rets_sha256"]
    look = np.concatenate([keys[: case["lookup_n"] // 2],
                           O.mt_keys(seed, case["lookup_n"] - case["lookup_n"] // 2, skip=n)]).astype(np.uint32)
    assert sha(f.lookup(look)) == case["lookup_sha256"]


@pytest.mark.parametrize("q,alpha,seed", [(12, 0.9, 61), (16, 0.94, 62), (20, 0.9, 63), (23, 0.9, 64)])
def test_rsqf8_build_batches_lookups(gqf, cuda, q, alpha, seed):
    """8-bit remainders against the oracle: a build into an empty filter,
    two incremental batches, sorted and unsorted lookups.  q = 23 is the
    largest width whose q + 8 fingerprint bits fit the 31 the hash uses."""
    n = int(alpha * (1 << q))
    keys = O.mt_keys(seed, n)
    f = RSQF(gqf, cuda, q, 8)
    o = O.rsqf_new(q, 8)
    assert np.array_equal(f.insert(keys), O.rsqf_insert_sorted(o, q, keys, 8))
    assert_same_blocks(f.blocks(), o, 81)
    for k in range(2):
        b = O.mt_keys(seed + 10 + k, max(64, n // 64))
        assert np.array_equal(f.insert(b), O.rsqf_insert_sorted(o, q, b, 8))
        assert_same_blocks(f.blocks(), o, 81)
    look = np.concatenate([keys[: n // 2], O.mt_keys(seed + 20, n // 2)])
    want = O.rsqf_lookup(o, q, look, 8)
    assert np.array_equal(f.lookup(look, sorted_=True), want)
    assert np.array_equal(f.lookup(look, sorted_=False), want)
    small = look[: max(1, (1 << q) // 32)]
    assert np.array_equal(f.lookup(small, sorted_=True), O.rsqf_lookup(o, q, small, 8))


def test_rsqf8_width_limits(gqf, cuda):
    with pytest.raises(gqf.GQFError):
        gqf.initCQFGPU(24, 8)  # q + 8 > 31
    with pytest.raises(gqf.GQFError):
        gqf.initCQFGPU(12, 6)
