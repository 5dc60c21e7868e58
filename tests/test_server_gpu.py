"""Served filters: a mixed stream of lookup / insert / delete requests on
many resident filters, submitted at once and served with continuous
batching over concurrent streams, gives every request the result it gets
when the requests are applied one at a time in submission order through
the plain API (and the same final tables); the same with coalescing off."""
import numpy as np
import pytest

import oracle as O
from conftest import from_dev, to_dev

pytestmark = pytest.mark.gpu


def build_filters(G, torch, filters):
    out = []
    for f in filters:
        qf = G.initFilterGPU(f["q"], 5)
        G.bulkBuildSegmentedLayouts(qf, f["keys"].size, to_dev(torch, f["keys"]), True)
        out.append(qf)
    return out


def sequential(G, torch, qfs, reqs):
    res = []
    for r in reqs:
        qf, k = qfs[r["filter"]], r["keys"]
        if r["op"] == G.SERVE_LOOKUP:
            out = torch.empty(max(k.size, 1), dtype=torch.int32, device="cuda")
            if k.size:
                G.launchUnsortedLookups(qf, k.size, to_dev(torch, k), out)
            res.append(from_dev(out)[: k.size])
        elif r["op"] == G.SERVE_INSERT:
            if k.size:
                G.insert(qf, k.size, to_dev(torch, k))
            res.append(None)
        else:
            if k.size:
                G.superclusterDeletes(qf, k.size, to_dev(torch, k))
            res.append(None)
    return res


@pytest.mark.parametrize("coalesce,streams", [(True, 0), (False, 3), (True, 1)])
def test_served_stream_equals_sequential(gqf, cuda, coalesce, streams):
    G, torch = gqf, cuda
    from gpuquotientfilters_gb300 import workload as W
    filters, reqs = W.config5(seed=11, nfilters=6, q_lo=12, q_hi=15, nreq=240, size_lo=16, size_hi=4096)
    served = build_filters(G, torch, filters)
    plain = build_filters(G, torch, filters)
    srv = G.Server(served, max_streams=streams, coalesce=coalesce)
    keys = [torch.from_numpy(r["keys"].view(np.int32)).pin_memory() for r in reqs]
    outs = [torch.zeros(max(r["keys"].size, 1), dtype=torch.int32).pin_memory() if r["op"] == 0 else None
            for r in reqs]
    for r, k, o in zip(reqs, keys, outs):
        srv.submit(r["filter"], r["op"], k, o)
    srv.drain()
    done = srv.poll(10000)
    assert len(done) == len(reqs) and all(d["status"] == 0 for d in done)
    assert all(d["done_us"] >= d["start_us"] >= d["submit_us"] for d in done)
    srv.close()
    want = sequential(G, torch, plain, reqs)
    for r, o, w in zip(reqs, outs, want):
        if r["op"] == 0:
            assert np.array_equal(o.numpy().view(np.uint32)[: r["keys"].size], w)
    for a, b in zip(served, plain):
        assert np.array_equal(G.table_bytes(a), G.table_bytes(b))
    # and the plain path is the oracle's sequential application
    f0 = filters[0]
    t = O.sqf_new(f0["q"], 5)
    O.sqf_bulk_build(t, f0["q"], 5, f0["keys"], True)
    for r in reqs:
        if r["filter"] != 0 or not r["keys"].size:
            continue
        if r["op"] == 1:
            O.sqf_insert(t, f0["q"], 5, r["keys"])
        elif r["op"] == 2:
            O.sqf_delete(t, f0["q"], 5, r["keys"])
    assert np.array_equal(G.table_bytes(served[0]), t)
    for qf in served + plain:
        G.freeFilterGPU(qf)


def test_server_budget(gqf, cuda):
    G, torch = gqf, cuda
    qf = G.initFilterGPU(14, 5)
    with pytest.raises(G.GQFError) as e:
        G.Server([qf], hbm_budget=1 << 20)  # not even one stream's workspace fits
    assert e.value.status == G.GQF_ERR_NOMEM
    big = G.Server([qf], hbm_budget=1 << 34, max_streams=4)
    assert big.info()["streams"] == 4
    big.close()
    G.freeFilterGPU(qf)
