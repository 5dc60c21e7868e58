"""Filter images (checkpoint / restore): a saved SQF or RSQF restores bit
for bit and answers lookups as before; damaged or mismatched images are
refused with GQF_ERR_FORMAT, missing files with GQF_ERR_IO."""
import os
import struct

import numpy as np
import pytest

import oracle as O
from conftest import from_dev, to_dev


@pytest.mark.gpu
def test_sqf_image_round_trip(gqf, cuda, tmp_path):
    G, torch = gqf, cuda
    for q, r in ((16, 5), (14, 13)):
        keys = O.mt_keys(51, int(0.7 * (1 << q)))
        qf = G.initFilterGPU(q, r)
        G.bulkBuildSegmentedLayouts(qf, keys.size, to_dev(torch, keys), False)
        path = str(tmp_path / ("sqf_%d_%d.gqf" % (q, r)))
        G.saveFilter(qf, path)
        assert os.path.getsize(path) == 64 + G.calcNumSlotsGPU(q, r)
        qf2 = G.loadFilter(path)
        assert (qf2.qbits, qf2.rbits, qf2.bytesPerElement) == (q, r, qf.bytesPerElement)
        assert np.array_equal(G.table_bytes(qf2), G.table_bytes(qf))
        out = torch.empty(keys.size, dtype=torch.int32, device="cuda")
        G.launchUnsortedLookups(qf2, keys.size, to_dev(torch, keys), out)
        t = O.sqf_new(q, r)
        O.sqf_bulk_build(t, q, r, keys, False)
        assert np.array_equal(from_dev(out), O.sqf_lookup(t, q, r, keys))
        img = G.filter_image(qf)
        qf3 = G.filter_from_image(img)
        assert np.array_equal(G.table_bytes(qf3), G.table_bytes(qf))
        for f in (qf, qf2, qf3):
            G.freeFilterGPU(f)


@pytest.mark.gpu
def test_rsqf_image_round_trip(gqf, cuda, tmp_path):
    G, torch = gqf, cuda
    q = 14
    keys = O.mt_keys(52, int(0.8 * (1 << q)))
    cqf = G.initCQFGPU(q)
    ret = torch.empty(keys.size, dtype=torch.int32, device="cuda")
    G.insertGPU(cqf, keys.size, to_dev(torch, keys), ret)
    path = str(tmp_path / "rsqf.gqf")
    G.saveCQF(cqf, path)
    assert os.path.getsize(path) == 64 + cqf.numBlocks * 57
    c2 = G.loadCQF(path)
    assert np.array_equal(G.rsqf_blocks_bytes(c2), G.rsqf_blocks_bytes(cqf))
    G.freeCQFGPU(cqf)
    G.freeCQFGPU(c2)


@pytest.mark.gpu
def test_damaged_images_are_refused(gqf, cuda, tmp_path):
    G, torch = gqf, cuda
    qf = G.initFilterGPU(12, 5)
    keys = O.mt_keys(53, 2000)
    G.bulkBuildSegmentedLayouts(qf, keys.size, to_dev(torch, keys), True)
    img = bytearray(G.filter_image(qf))
    G.freeFilterGPU(qf)
    bad = [bytes(img[:-1]),                       # truncated
           bytes(img[:100]) + bytes([img[100] ^ 4]) + bytes(img[101:]),  # payload bit flip
           b"XQFSQF01" + bytes(img[8:]),           # magic
           bytes(img[:12]) + struct.pack("<I", 13) + bytes(img[16:])]  # q changed
    for b in bad:
        with pytest.raises(G.GQFError) as e:
            G.filter_from_image(b)
        assert e.value.status == G.GQF_ERR_FORMAT
    with pytest.raises(G.GQFError) as e:
        G.loadFilter(str(tmp_path / "missing.gqf"))
    assert e.value.status == G.GQF_ERR_IO
    # an SQF image is not an RSQF image
    p = str(tmp_path / "sqf.gqf")
    open(p, "wb").write(bytes(img))
    with pytest.raises(G.GQFError) as e:
        G.loadCQF(p)
    assert e.value.status == G.GQF_ERR_FORMAT
