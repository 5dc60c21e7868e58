"""The drop-in boundary: the reference-named C++ API in include/*.cuh.

CPU: every GPU driver of the reference (its tests and perf programs)
compiles against its own header and links against libgqf.so unchanged
(needs the reference checkout; skipped elsewhere).
GPU: a driver written against include/quotientFilter.cuh and RSQF.cuh runs
build, lookups, deletes, re-insert and RSQF insert/lookups; every result is
compared with the oracle."""
import concurrent.futures as cf
import glob
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = O.reference_dir()
NVCC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def ref_drivers():
    out = []
    for d in ("standardQuotientFilter/GPU_version", "rankSelectQuotientFilter/GPU_version"):
        for f in sorted(glob.glob(os.path.join(REF, d, "*.cu"))):
            if os.path.basename(f) not in ("quotientFilter.cu", "RSQF.cu"):
                out.append(f)
    return out


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout absent")
def test_reference_drivers_link_against_libgqf(gqf):
    drivers = ref_drivers()
    assert len(drivers) >= 20
    lib_dir = os.path.dirname(gqf.LIB_PATH)
    with tempfile.TemporaryDirectory() as tmp:
        mt = os.path.join(tmp, "mt.o")
        subprocess.check_call(["g++", "-O2", "-c", os.path.join(REF, "mt19937ar.cpp"), "-o", mt])

        def build(src):
            exe = os.path.join(tmp, os.path.basename(src)[:-3])
            # insertViaMergePerf.cu and merge2FiltersTest.cu use std::string
            # without including <string> (it arrived transitively with older
            # toolkits); pre-including it changes no source.
            r = subprocess.run([NVCC] + ARCH + ["-w", "-include", "string", "-o", exe, src, mt,
                                "-L" + lib_dir, "-lgqf"],
                               capture_output=True, text=True)
            return src, r.returncode, r.stdout + r.stderr

        with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
            results = list(ex.map(build, drivers))
    bad = [(os.path.basename(s), out[-400:]) for s, rc, out in results if rc != 0]
    assert not bad, bad


def build_dropin_driver(gqf, exe):
    lib_dir = os.path.dirname(gqf.LIB_PATH)
    subprocess.check_call([NVCC] + ARCH + ["-w", "-I", os.path.join(ROOT, "include"), "-o", exe,
                           os.path.join(ROOT, "tests", "drivers", "dropin_driver.cu"),
                           "-L" + lib_dir, "-lgqf", "-Xlinker", "-rpath=" + lib_dir])


def test_dropin_driver_builds(gqf):
    """include/quotientFilter.cuh and include/RSQF.cuh compile together and
    every reference-named function they declare resolves in libgqf.so."""
    with tempfile.TemporaryDirectory() as tmp:
        build_dropin_driver(gqf, os.path.join(tmp, "dropin_driver"))


@pytest.mark.gpu
def test_dropin_driver_matches_oracle(gqf, cuda):
    from gpuquotientfilters_gb300 import workload as W
    c = W.config1()
    q, r = 15, 5
    with tempfile.TemporaryDirectory() as tmp:
        c["keys"].astype(np.uint32).tofile(os.path.join(tmp, "keys.u32"))
        c["lookups"].astype(np.uint32).tofile(os.path.join(tmp, "lookups.u32"))
        c["deletes"].astype(np.uint32).tofile(os.path.join(tmp, "deletes.u32"))
        exe = os.path.join(tmp, "dropin_driver")
        build_dropin_driver(gqf, exe)
        subprocess.check_call([exe, tmp])
        rd = lambda n, dt: np.fromfile(os.path.join(tmp, n), dt)
        t = O.sqf_new(q, r)
        O.sqf_bulk_build(t, q, r, c["keys"], True)
        assert np.array_equal(rd("table_build.u8", np.uint8), t)
        want = O.sqf_lookup(t, q, r, c["lookups"])
        assert np.array_equal(rd("lookup_unsorted.u32", np.uint32), want)
        assert np.array_equal(rd("lookup_sorted.u32", np.uint32), want)
        O.sqf_delete(t, q, r, c["deletes"])
        assert np.array_equal(rd("table_delete.u8", np.uint8), t)
        O.sqf_insert(t, q, r, c["deletes"])
        assert np.array_equal(rd("table_reinsert.u8", np.uint8), t)
        b = O.rsqf_new(12)
        ret = O.rsqf_insert_sorted(b, 12, c["keys"][:3600])
        assert np.array_equal(rd("rsqf_ret.i32", np.int32), ret)
        assert np.array_equal(rd("rsqf_blocks.u8", np.uint8), b)
        assert np.array_equal(rd("rsqf_lookup.i32", np.int32), O.rsqf_lookup(b, 12, c["lookups"]))
