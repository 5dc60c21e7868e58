"""Digests of the reference's own GPU kernels on fixed workloads.

Runs the reference's standard-filter kernels (``oracle/_ref/ref_sqf_gpu.cubin``,
built by ``oracle/build_ref_gpu.sh`` from ``quotientFilter.cu``; driven by
``oracle/ref_gpu.py``) through every step of the cases below, and records the
SHA-256 of each table and lookup result in ``tests/golden/golden_refgpu.json``.
It needs a GPU and the cubin, so it runs on a GPU machine:

    python tests/golden/make_golden_refgpu.py [out.json]

The same ``run_case`` drives the product (``backend="gqf"``) and the CPU
oracle (``backend="oracle"``) in the tests, so all three are compared step
by step.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_refgpu.json")
BUILDS = ("segmented", "sequential", "parallel")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _fresh(seed: int, n: int, avoid: np.ndarray) -> np.ndarray:
    k = O.mt_keys(seed, n + 64)
    k = k[~np.isin(k, avoid)]
    return k[:n].astype(np.uint32)


def cases():
    """Seeded cases: (name, q, r, keys, lookups, deletes, inserts)."""
    out = []
    # config 1: q=15 r=5, 19,661 keys of MT19937 seed 1; lookups half
    # inserted keys, half further draws; delete the first 4,096 keys
    k1 = O.mt_keys(1, 19661)
    look1 = np.concatenate([k1[:9830], O.mt_keys(1, 19661 - 9830, skip=19661)]).astype(np.uint32)
    out.append(("q15r5", 15, 5, k1, look1, k1[:4096].copy(),
                np.concatenate([_fresh(9, 2048, k1), k1[100:164]]).astype(np.uint32)))
    # q=18 r=5 at fill 0.8; deletes mix present keys (some twice) and absent ones
    n2 = int(0.8 * (1 << 18))
    k2 = O.mt_keys(2, n2)
    absent = _fresh(12, 2048, k2)
    del2 = np.concatenate([k2[:12000], k2[:1000], absent]).astype(np.uint32)
    look2 = np.concatenate([k2[5000:13192], absent]).astype(np.uint32)
    out.append(("q18r5", 18, 5, k2, look2, del2, _fresh(13, 8192, k2)))
    # two-byte slots: q=14 r=13 at fill 0.7
    n3 = int(0.7 * (1 << 14))
    k3 = O.mt_keys(6, n3)
    out.append(("q14r13", 14, 13, k3, np.concatenate([k3[:4000], _fresh(16, 4000, k3)]).astype(np.uint32),
                k3[:3000].copy(), _fresh(17, 1500, k3)))
    for _, _, _, *arrs in out:
        for a in arrs:
            assert not (a == 0xFFFFFFFF).any()
    return out


class _Gqf:
    def __init__(self, q, r):
        import torch
        import gpuquotientfilters_gb300 as G
        self.G, self.torch, self.q, self.r = G, torch, q, r
        self.qf = G.initFilterGPU(q, r)

    def _d(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32)).cuda()

    def build(self, how, keys, nodup):
        fn = {"segmented": self.G.bulkBuildSegmentedLayouts,
              "sequential": self.G.bulkBuildSequentialShifts,
              "parallel": self.G.bulkBuildParallelMerging}[how]
        fn(self.qf, keys.size, self._d(keys), nodup)

    def lookups(self, keys, sorted_):
        out = self.torch.empty(keys.size, dtype=self.torch.int32, device="cuda")
        fn = self.G.launchSortedLookups if sorted_ else self.G.launchUnsortedLookups
        fn(self.qf, keys.size, self._d(keys), out)
        return out.cpu().numpy().view(np.uint32)

    def delete(self, keys):
        self.G.superclusterDeletes(self.qf, keys.size, self._d(keys))

    def insert(self, keys):
        self.G.insert(self.qf, keys.size, self._d(keys))

    def table(self):
        return self.G.table_bytes(self.qf)

    def close(self):
        self.G.freeFilterGPU(self.qf)


class _Ref:
    def __init__(self, q, r):
        from oracle import ref_gpu as R
        self.R, self.f = R, R.RefFilter(q, r)

    def build(self, how, keys, nodup):
        {"segmented": self.R.bulk_build_segmented_layouts,
         "sequential": self.R.bulk_build_sequential_shifts,
         "parallel": self.R.bulk_build_parallel_merging}[how](self.f, keys, nodup)

    def lookups(self, keys, sorted_):
        return (self.R.sorted_lookups if sorted_ else self.R.unsorted_lookups)(self.f, keys)

    def delete(self, keys):
        self.R.supercluster_deletes(self.f, keys)

    def insert(self, keys):
        self.R.insert(self.f, keys)

    def table(self):
        return self.f.table()

    def close(self):
        del self.f


class _Oracle:
    def __init__(self, q, r):
        self.q, self.r, self.t = q, r, O.sqf_new(q, r)

    def build(self, how, keys, nodup):
        assert O.sqf_bulk_build(self.t, self.q, self.r, keys, nodup) == 0

    def lookups(self, keys, sorted_):
        return O.sqf_lookup(self.t, self.q, self.r, keys)

    def delete(self, keys):
        O.sqf_delete(self.t, self.q, self.r, keys)

    def insert(self, keys):
        O.sqf_insert(self.t, self.q, self.r, keys)

    def table(self):
        return self.t

    def close(self):
        pass


BACKENDS = {"ref": _Ref, "gqf": _Gqf, "oracle": _Oracle}


def run_case(case, backend: str, record=None):
    """Every step of one case on one backend: for each bulk build (3 builds x
    NoDup/Dup) a fresh filter; after the build the table and both lookup
    kinds; then deletes, table, inserts, table, lookups.  Returns
    {step: sha256}; ``record(step, array)`` sees each array as well."""
    name, q, r, keys, look, dels, ins = case
    d = {}

    def put(step, a):
        d[step] = sha(a)
        if record is not None:
            record(step, a)

    for how in BUILDS:
        for nodup in (True, False):
            tag = "%s_%s" % (how, "nodup" if nodup else "dup")
            f = BACKENDS[backend](q, r)
            try:
                f.build(how, keys, nodup)
                put(tag + "/build", f.table())
                put(tag + "/lookup_unsorted", f.lookups(look, False))
                put(tag + "/lookup_sorted", f.lookups(look, True))
                f.delete(dels)
                put(tag + "/delete", f.table())
                f.insert(ins)
                put(tag + "/insert", f.table())
                put(tag + "/lookup_after", f.lookups(look, False))
            finally:
                f.close()
    return d


def main():
    out = sys.argv[1] if len(sys.argv) > 1 else OUT
    g = {"generated_by": "tests/golden/make_golden_refgpu.py: the reference's quotientFilter.cu "
                         "kernels (oracle/_ref/ref_sqf_gpu.cubin) on a GPU",
         "cases": {}}
    for case in cases():
        g["cases"][case[0]] = run_case(case, "ref")
        print(case[0], "done", flush=True)
    with open(out, "w") as fh:
        json.dump(g, fh, indent=1, sort_keys=True)
    print("wrote", out)


if __name__ == "__main__":
    main()
