"""libgqf.so loads without a GPU, exports every symbol include/*.h declares,
and its host-only helpers agree with the oracle."""
import ctypes as C
import glob
import os
import re

import numpy as np

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b(gqf_[a-z0-9_]+)\s*\(", src):
            syms.add(m.group(1))
    return syms


def test_library_exports_every_declared_symbol(gqf):
    L = C.CDLL(gqf.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in sorted(syms) if not hasattr(L, s)]
    assert not missing, missing


def test_host_helpers_match_oracle(gqf, oracle_lib):
    for q, r in [(15, 5), (26, 5), (18, 13), (7, 5)]:
        assert gqf.calcNumSlotsGPU(q, r) == O.sqf_table_bytes(q, r)
        assert gqf.num_slots(q) == O.sqf_num_slots(q)
    for q in (10, 20, 26):
        assert gqf.calcNumBlocksGPU(q) == O.rsqf_num_blocks(q)
    for seed in (1, 2, 3):
        assert np.array_equal(gqf.mt19937(seed, 3000, 17), O.mt_keys(seed, 3000, 17))
    keys = O.mt_keys(4, 500)
    for b in (6, 20, 31):
        assert all(gqf.Normal_APHash(int(k), 1 << b) == O.lib().or_aphash(int(k), 1 << b) for k in keys)


def test_status_strings(gqf):
    L = gqf.lib()
    for st in range(7):
        assert L.gqf_status_string(st)


def test_workload_config1_shapes(gqf):
    from gpuquotientfilters_gb300 import workload as W
    c = W.config1()
    assert c["keys"].size == 19661 and c["lookups"].size == 19661 and c["deletes"].size == 4096
    assert np.array_equal(c["keys"], O.mt_keys(1, 19661))
    # half of the lookups are inserted keys
    assert np.isin(c["lookups"], c["keys"]).sum() >= 19661 // 2
    assert W.n_keys(15, 0.6) == 19661 and W.n_keys(15, 0.6, reference_arithmetic=True) == 19660
    assert W.n_keys(26, 0.8) == 53687091 and W.n_keys(26, 0.8, reference_arithmetic=True) == 53687092


def test_unaligned_table_refused_before_any_device_call(gqf):
    """A table pointer that is not 16-byte aligned is refused with
    GQF_ERR_ARG by the argument check itself (no CUDA call is made, so this
    runs without a GPU)."""
    L = gqf.lib()
    for addr in (0x10001, 0x10008, 0x1000C):
        qf = gqf.quotient_filter(20, 5, 1, addr)
        keys, out = 0x20000, 0x30000
        assert L.gqf_sqf_lookup_unsorted(C.byref(qf), 1 << 20, C.c_void_p(keys), C.c_void_p(out), None, None) == 1
        assert L.gqf_sqf_lookup_sorted(C.byref(qf), 16, C.c_void_p(keys), C.c_void_p(out), None, None) == 1
        assert L.gqf_sqf_insert(C.byref(qf), 16, C.c_void_p(keys), None, None) == 1
        assert L.gqf_sqf_delete(C.byref(qf), 16, C.c_void_p(keys), None, None) == 1
        assert L.gqf_sqf_bulk_build(C.byref(qf), 16, C.c_void_p(keys), 1, None, None) == 1
