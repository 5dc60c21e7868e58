"""Generates tests/golden/golden.json from the reference's own CPU code.

Run in a checkout where the reference sources exist: it compiles them with
oracle/build_ref.sh (into oracle/_ref/, git-ignored) and records
  * MT19937 draws (mt19937ar.cpp) and Normal_APHash values (RSQF.cpp),
  * SQF CPU_version (quotientFilter.cpp) logical slot arrays after
    sequential insertItem, with its shipped FNV hash and with the GPU's
    Normal_APHash, plus mayContain results for a mixed lookup batch,
  * RSQF CPU_version (RSQF.cpp) packed blocks and return slots after
    inserting a batch in ascending fingerprint order, plus lookups -- as
    shipped (RBITS 5) and compiled with RBITS 8,
as SHA-256 digests (and a few raw arrays for small cases), so the oracle
can be pinned where the reference checkout is absent.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def mixed(keys, n, seed, ref):
    """n lookups: first n//2 inserted keys then n - n//2 further draws,
    interleaved (no shuffle needed for a digest)."""
    neg = ref.mt_keys(seed, n - n // 2, skip=keys.size)
    return np.concatenate([keys[: n // 2], neg]).astype(np.uint32)


def main():
    if not oracle.build_ref():
        raise SystemExit("reference checkout not found; nothing generated")
    ref = oracle.Ref()
    g = {"generated_by": "tests/golden/make_golden.py from the reference CPU_version sources"}

    g["mt19937"] = {
        str(s): {"first8": [int(x) for x in ref.mt_keys(s, 8)],
                 "skip10000_4": [int(x) for x in ref.mt_keys(s, 4, skip=10000)]}
        for s in (1, 2, 3, 4, 5)
    }
    keys = ref.mt_keys(11, 64)
    g["aphash"] = [[int(k), sz, int(ref.rsqf.ref_aphash(int(k), sz))]
                   for k, sz in zip(keys, [1 << b for b in range(5, 32)] * 3)]

    sqf_cases = []
    for (q, r, n, seed) in [(15, 5, 19661, 1), (15, 5, 19660, 1), (12, 5, 3686, 4),
                            (16, 5, 58982, 2), (14, 13, 13107, 3), (10, 5, 900, 5)]:
        k = ref.mt_keys(seed, n)
        look = mixed(k, n, seed, ref)
        case = {"q": q, "r": r, "n": n, "seed": seed}
        for name, gpu_hash in (("aphash", True), ("fnv", False)):
            words = ref.sqf_build_insert(q, r, k, gpu_hash=gpu_hash)
            slots = oracle.sqfcpu_slots(words, q, r)
            res = ref.sqf_insert_then_lookup(q, r, k, look, gpu_hash=gpu_hash).astype(np.uint32)
            case[name] = {
                "slots_sha256": sha(slots.astype(np.uint32)),
                "lookup_sha256": sha(res),
                "not_found_of_inserted": int((res[: n // 2] == oracle.NOT_FOUND).sum()),
                "false_positives": int((res[n // 2:] != oracle.NOT_FOUND).sum()),
            }
            if n <= 1000:
                case[name]["slots"] = [int(x) for x in slots]
        sqf_cases.append(case)
    g["sqf_cpu_version"] = sqf_cases

    def rsqf_cases(R, rbits, cases):
        out = []
        bb = int(R.ref_rsqf_block_bytes())
        for (q, n, batch, seed) in cases:
            k = ref.mt_keys(seed, n)
            fps = np.array([R.ref_aphash(int(x), 1 << (q + rbits)) for x in k], np.uint32)
            order = np.argsort(fps, kind="stable")
            f = R.ref_rsqf_new(q)
            try:
                rets = np.array([R.ref_rsqf_insert(f, int(x)) for x in k[order]], np.int32)
                nb = int(R.ref_rsqf_num_blocks(q)) + 1
                blocks = np.ctypeslib.as_array(C.cast(R.ref_rsqf_blocks(f), C.POINTER(C.c_uint8)),
                                               shape=(nb * bb,)).copy()
                bk = ref.mt_keys(seed, batch, skip=n)
                bf = np.array([R.ref_aphash(int(x), 1 << (q + rbits)) for x in bk], np.uint32)
                bo = np.argsort(bf, kind="stable")
                brets = np.array([R.ref_rsqf_insert(f, int(x)) for x in bk[bo]], np.int32)
                blocks2 = np.ctypeslib.as_array(C.cast(R.ref_rsqf_blocks(f), C.POINTER(C.c_uint8)),
                                                shape=(nb * bb,)).copy()
                look = mixed(k, min(n, 4096), seed, ref)
                lres = np.array([R.ref_rsqf_lookup(f, int(x)) for x in look], np.int32)
            finally:
                R.ref_rsqf_free(f)
            out.append({
                "q": q, "n": n, "batch": batch, "seed": seed, "rbits": rbits, "block_bytes": bb,
                "build_blocks_sha256": sha(blocks), "build_rets_sha256": sha(rets),
                "batch_blocks_sha256": sha(blocks2), "batch_rets_sha256": sha(brets),
                "lookup_n": int(look.size), "lookup_sha256": sha(lres),
            })
        return out

    g["rsqf_cpu_version"] = rsqf_cases(ref.rsqf, 5, [(12, 3686, 256, 3), (14, 14745, 1024, 3), (10, 972, 64, 6)])
    # RSQF.h with RBITS 8 (oracle/ref_rsqf8_pre.h): 81-byte blocks
    g["rsqf8_cpu_version"] = rsqf_cases(ref.rsqf8, 8, [(12, 3686, 256, 3), (14, 14745, 1024, 3), (10, 972, 64, 6),
                                                       (16, 58982, 2048, 7)])
    with open(OUT, "w") as fh:
        json.dump(g, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
