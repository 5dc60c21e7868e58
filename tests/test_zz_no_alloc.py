"""The bulk build that allocates no device memory.

Some callers cannot call cudaMalloc while they run -- a process whose own
pool allocator already reserved the GPU's memory, a latency-critical stream
that must not be stalled by cudaMalloc's implicit synchronisation, a service
whose memory budget is fixed after start-up.  gqf_sqf_bulk_build_noalloc
serves them from a fixed scratch array compiled into libgqf.so.  This test
calls it through the C ABI, twice in a row on the same filter with different
key sets (the second call must not see the first call's scratch contents),
and checks each table byte-for-byte against the ordinary entry point
gqf_sqf_bulk_build on the same keys.  It also checks that a batch beyond the
fixed maximum is refused with GQF_ERR_LIMIT.

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
