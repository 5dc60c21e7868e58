"""Bounded device-side waits: the bulk build's decoupled look-back gives up
after a bounded number of polls, reports GQF_ERR_TIMEOUT, and leaves the
device usable.

gqf_debug_lookback_probe runs the build's own look-back (one warp per
bucket) over descriptors written by the host.  A descriptor left
unpublished is a flag that nothing ever sets, so the buckets that have to
read it wait until their poll limit runs out.
"""
import time

import numpy as np
import pytest

AGG, INC = 1, 2
VMAX = 0x7FFFFFFF


def pack(flag, n=0, v=0):
    return (flag << 62) | ((n & VMAX) << 31) | (v & VMAX)


def model(desc):
    """Entry slot of every bucket, or None where the look-back must wait on an
    unpublished descriptor: windows of 32 predecessors, nearest first, each
    waited on in full before its nearest inclusive descriptor is used; a
    predecessor index below 0 reads as inclusive slot 0."""
    out = []
    for b in range(len(desc)):
        j = b - 1
        res = "pending"
        while res == "pending":
            win = [(desc[i] if i >= 0 else pack(INC, 0, 0)) for i in range(j, j - 32, -1)]
            if any((d >> 62) == 0 for d in win):
                res = None
                break
            incs = [k for k, d in enumerate(win) if (d >> 62) == INC]
            if incs:
                L = incs[0]
                c = win[L] & VMAX
                for k in range(L - 1, -1, -1):  # nearer buckets apply later
                    n, F = (win[k] >> 31) & VMAX, win[k] & VMAX
                    c = max(c + n, F)
                # the windows nearer than this one are aggregates only
                for i in range(j + 1, b):
                    n, F = (desc[i] >> 31) & VMAX, desc[i] & VMAX
                    c = max(c + n, F)
                res = c
            else:
                j -= 32
        out.append(res)
    return out


def descriptors(nb, seed, unpublished=()):
    rng = np.random.default_rng(seed)
    d, c = [], 0
    for b in range(nb):
        n = int(rng.integers(0, 3000))
        x0 = b * 2048
        F = max(x0 + n, int(rng.integers(x0, x0 + 2200)))
        c = max(c + n, F)
        if b in unpublished:
            d.append(0)
        elif rng.random() < 0.15:
            d.append(pack(INC, 0, c))
        else:
            d.append(pack(AGG, n, F))
    return d


def run_probe(G, desc, spin_limit):
    import ctypes as C
    st = np.array(desc, dtype=np.uint64)
    cin = np.zeros(len(desc), dtype=np.uint32)
    t = time.time()
    rc = G.lib().gqf_debug_lookback_probe(st.ctypes.data_as(C.c_void_p), len(desc), spin_limit,
                                          cin.ctypes.data_as(C.c_void_p))
    return rc, cin, time.time() - t


def test_model_folds_like_a_sequential_scan():
    d = descriptors(300, 1)
    got = model(d)
    c, ref = 0, []
    for i, x in enumerate(d):
        ref.append(c)
        if (x >> 62) == INC:
            c = x & VMAX
        else:
            c = max(c + ((x >> 31) & VMAX), x & VMAX)
    assert got == ref


@pytest.mark.gpu
def test_lookback_all_published(gqf, cuda):
    d = descriptors(600, 2)
    rc, cin, _ = run_probe(gqf, d, 1 << 12)
    assert rc == 0
    assert list(cin) == model(d)


@pytest.mark.gpu
def test_lookback_wait_runs_out(gqf, cuda):
    """Bucket 200's descriptor is never published: buckets that must read it
    time out after 4096 polls; the others get their exact entry slot."""
    d = descriptors(600, 3, unpublished={200})
    want = model(d)
    assert any(w is None for w in want) and any(w is not None for w in want[201:])
    rc, cin, secs = run_probe(gqf, d, 1 << 12)
    assert rc == 4  # GQF_ERR_TIMEOUT
    assert secs < 10
    for b, w in enumerate(want):
        assert cin[b] == (0 if w is None else w), b
    # the device is still usable: a build right after is exact
    import oracle as O
    from conftest import to_dev
    q, r = 12, 5
    keys = O.mt_keys(21, 3000)
    qf = gqf.initFilterGPU(q, r)
    try:
        gqf.bulkBuildSegmentedLayouts(qf, keys.size, to_dev(cuda, keys), True)
        t = O.sqf_new(q, r)
        O.sqf_bulk_build(t, q, r, keys, True)
        assert (gqf.table_bytes(qf) == t).all()
    finally:
        gqf.freeFilterGPU(qf)
