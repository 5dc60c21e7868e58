"""The bulk build that allocates no device memory.

Some callers cannot call cudaMalloc while they run -- a process whose own
pool allocator already reserved the GPU's memory, a latency-critical stream
that must not be stalled by cudaMalloc's implicit synchronisation, a service
whose memory budget is fixed after start-up.  gqf_sqf_bulk_build_noalloc
serves them from a fixed scratch array compiled into libgqf.so.  This test
calls it through the C ABI, twice in a row on the same filter with different
key sets (the second call must not see the first call's scratch contents),
and checks each table byte-for-byte against the ordinary entry point
gqf_sqf_bulk_build on the same keys.  It also checks that the calls leave
free device memory unchanged, that empty and maximum-size batches work, and
that a batch beyond the fixed maximum is refused with GQF_ERR_LIMIT.

The file name sorts last so a run that stops at the first failure has run
every other test before this one.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from conftest import to_dev

pytestmark = pytest.mark.gpu


def noalloc_build(G, torch, qf, keys, nodup):
    d = to_dev(torch, keys)
    st = G.lib().gqf_sqf_bulk_build_noalloc(C.byref(qf), int(keys.size), d.data_ptr(), int(nodup), None)
    torch.cuda.synchronize()
    return st


def reference_build(G, torch, q, r, keys, nodup):
    qf = G.initFilterGPU(q, r)
    try:
        G.bulkBuildSegmentedLayouts(qf, keys.size, to_dev(torch, keys), nodup)
        return G.table_bytes(qf)
    finally:
        G.freeFilterGPU(qf)


@pytest.mark.parametrize("q,r,nodup", [(20, 5, True), (18, 5, False), (16, 13, True)])
def test_noalloc_build_matches_regular_build_twice(gqf, cuda, q, r, nodup):
    G, torch = gqf, cuda
    qf = G.initFilterGPU(q, r)
    try:
        first = O.mt_keys(41, int(0.8 * (1 << q)))
        second = np.concatenate([O.mt_keys(42, int(0.5 * (1 << q))), first[:1000]])
        for keys in (first, second):
            assert noalloc_build(G, torch, qf, keys, nodup) == G.GQF_OK
            got = G.table_bytes(qf)
            want = reference_build(G, torch, q, r, keys, nodup)
            assert np.array_equal(got, want)
    finally:
        G.freeFilterGPU(qf)


def test_noalloc_build_allocates_nothing(gqf, cuda):
    """Free device memory is the same before and after calls on a stream that
    no other entry point has used (after one warm-up call that loads the
    kernels, which lazy module loading may place in device memory)."""
    G, torch = gqf, cuda
    q, r = 20, 5
    keys = O.mt_keys(44, int(0.7 * (1 << q)))
    d = to_dev(torch, keys)
    qf = G.initFilterGPU(q, r)
    s = torch.cuda.Stream()
    try:
        L = G.lib()
        assert L.gqf_sqf_bulk_build_noalloc(C.byref(qf), keys.size, d.data_ptr(), 1, None) == G.GQF_OK
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(2):
            st = L.gqf_sqf_bulk_build_noalloc(C.byref(qf), keys.size, d.data_ptr(), 1, C.c_void_p(s.cuda_stream))
            assert st == G.GQF_OK
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0
        assert np.array_equal(G.table_bytes(qf), reference_build(G, torch, q, r, keys, True))
    finally:
        G.freeFilterGPU(qf)


def test_noalloc_build_edge_sizes(gqf, cuda):
    """An empty batch gives the empty table of the ordinary build (twice,
    after a full one, so the array's old contents do not leak); exactly
    GQF_NOALLOC_MAX_KEYS keys at the largest q fit; two-byte slots at their
    largest q (q + r <= 32) either fit and match or are refused with
    GQF_ERR_LIMIT."""
    G, torch = gqf, cuda
    L = G.lib()
    qf = G.initFilterGPU(16, 5)
    try:
        assert noalloc_build(G, torch, qf, O.mt_keys(45, 50000), True) == G.GQF_OK
        for _ in range(2):
            st = L.gqf_sqf_bulk_build_noalloc(C.byref(qf), 0, None, 1, None)
            assert st == G.GQF_OK
            assert np.array_equal(G.table_bytes(qf), reference_build(G, torch, 16, 5, np.zeros(0, np.uint32), True))
    finally:
        G.freeFilterGPU(qf)
    kmax = O.mt_keys(46, 1 << 20)
    for q, r, nodup, keys in ((22, 5, True, kmax), (22, 5, False, kmax), (18, 13, True, kmax[: int(0.8 * (1 << 18))])):
        qf = G.initFilterGPU(q, r)
        try:
            st = noalloc_build(G, torch, qf, keys, nodup)
            if r == 13 and st == G.GQF_ERR_LIMIT:
                continue
            assert st == G.GQF_OK, (q, r, nodup, st)
            assert np.array_equal(G.table_bytes(qf), reference_build(G, torch, q, r, keys, nodup))
        finally:
            G.freeFilterGPU(qf)


def test_noalloc_build_rejects_oversized_requests(gqf, cuda):
    G, torch = gqf, cuda
    L = G.lib()
    qf = G.initFilterGPU(23, 5)  # more quotient bits than the fixed scratch covers
    try:
        keys = O.mt_keys(43, 1000)
        st = L.gqf_sqf_bulk_build_noalloc(C.byref(qf), 1000, to_dev(torch, keys).data_ptr(), 1, None)
        assert st == G.GQF_ERR_LIMIT
        big = 2 << 20  # more keys than GQF_NOALLOC_MAX_KEYS
        d = torch.zeros(big, dtype=torch.int32, device="cuda")
        st = L.gqf_sqf_bulk_build_noalloc(C.byref(qf), big, d.data_ptr(), 1, None)
        assert st == G.GQF_ERR_LIMIT
        assert b"no-allocation" in L.gqf_status_string(st)
    finally:
        G.freeFilterGPU(qf)
