"""The reference's own GPU kernels as the checker for the standard filter.

``tests/golden/golden_refgpu.json`` holds digests of every step of the
cases in ``tests/golden/make_golden_refgpu.py`` -- bulk builds (segmented
layouts, sequential shifts, parallel merging; NoDup and Dup), unsorted and
sorted lookups, superclusterDeletes and insert -- produced by running the
reference's ``quotientFilter.cu`` kernels on a GPU.

* CPU: the oracle reproduces every digest (its delete, a sequential
  restatement of ``deleteItemGPU``, included).
* GPU: the product reproduces every digest through the C ABI; and where the
  reference cubin is present, the reference kernels run live beside it and
  every table and lookup array is compared byte for byte.
"""
import importlib.util
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
_spec = importlib.util.spec_from_file_location(
    "make_golden_refgpu", os.path.join(HERE, "golden", "make_golden_refgpu.py"))
MG = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(MG)
GOLD_PATH = os.path.join(HERE, "golden", "golden_refgpu.json")
GOLD = json.load(open(GOLD_PATH)) if os.path.exists(GOLD_PATH) else None
CASES = {c[0]: c for c in MG.cases()}


def _gold(name):
    if GOLD is None:
        pytest.fail("tests/golden/golden_refgpu.json is missing")
    return GOLD["cases"][name]


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_gpu(oracle_lib, name):
    got = MG.run_case(CASES[name], "oracle")
    want = _gold(name)
    bad = [s for s in want if got.get(s) != want[s]]
    assert not bad, "oracle differs from the reference GPU kernels at %s" % bad


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_product_matches_reference_gpu_digests(gqf, cuda, name):
    got = MG.run_case(CASES[name], "gqf")
    want = _gold(name)
    bad = [s for s in want if got.get(s) != want[s]]
    assert not bad, "libgqf differs from the reference GPU kernels at %s" % bad


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_kernels_live(gqf, cuda, name):
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("reference cubin not built (oracle/build_ref_gpu.sh needs the reference sources)")
    arrays = {}
    MG.run_case(CASES[name], "gqf", record=lambda s, a: arrays.__setitem__(s, a.copy()))
    mism = []

    def check(step, a):
        if not np.array_equal(arrays[step], a):
            mism.append(step)

    got = MG.run_case(CASES[name], "ref", record=check)
    assert not mism, "libgqf and the reference kernels differ at %s" % mism
    assert got == _gold(name), "reference kernels no longer give the committed digests"
