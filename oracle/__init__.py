"""CPU oracle for the quotient-filter hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the checker (or the timed CPU
baseline).  The product path (``gpuquotientfilters_gb300``) never imports it.

``liboracle.so`` is built from ``qf_oracle.c`` (a restatement of the
reference algorithms, each function citing the reference file:line).  When
the reference checkout is present, ``build_ref.sh`` also compiles the
reference's own CPU code into ``_ref/`` so tests can pin the restatement to it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
NOT_FOUND = 0xFFFFFFFF
APHASH, FNV = 0, 1

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile qf_oracle.c into liboracle.so (gcc, no GPU needed)."""
    src = os.path.join(HERE, "qf_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "qf_oracle.h"))
    ):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(
            ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-o", tmp, src]
        )
        os.replace(tmp, LIB)
    return LIB


def reference_dir() -> str:
    """The reference checkout the recipes read: $GQF_REFERENCE_DIR, else the
    folder this build was set up with."""
    return os.environ.get("GQF_REFERENCE_DIR", "/root/reference")


def build_ref(ref: str | None = None) -> bool:
    """Compile the reference CPU code into _ref/ if the checkout exists."""
    ref = ref or reference_dir()
    if not os.path.isdir(ref):
        return False
    env = dict(os.environ, REF=ref)
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")], env=env,
                          stdout=subprocess.DEVNULL)
    return True


def build_ref_gpu(ref: str | None = None) -> bool:
    """Compile the reference's standard-filter GPU source into
    _ref/ref_sqf_gpu.cubin (device code only) if the checkout exists."""
    ref = ref or reference_dir()
    if not os.path.isdir(ref):
        return False
    cubin = os.path.join(REF_DIR, "ref_sqf_gpu.cubin")
    srcs = [os.path.join(HERE, "build_ref_gpu.sh"), os.path.join(HERE, "ref_gpu_shim", "pre.cuh")]
    if os.path.exists(cubin) and os.path.getmtime(cubin) >= max(map(os.path.getmtime, srcs)):
        return True
    env = dict(os.environ, REF=ref)
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref_gpu.sh")], env=env,
                          stdout=subprocess.DEVNULL)
    return True


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        u32, u64, i32 = C.c_uint32, C.c_uint64, C.c_int32
        sz = C.c_size_t
        sig = {
            "or_mt_fill": (None, [u32, u64, _u32p, u64]),
            "or_aphash": (u32, [u32, u32]),
            "or_fnv": (u32, [u32, u32]),
            "or_hash_keys": (None, [_u32p, u64, u32, u32, C.c_int, _u32p]),
            "or_sqf_table_bytes": (sz, [u32, u32]),
            "or_sqf_num_slots": (u32, [u32]),
            "or_sqf_get": (u32, [_u8p, u32, u32, u32]),
            "or_sqf_insert_keys": (C.c_int, [_u8p, u32, u32, _u32p, u64, C.c_int]),
            "or_sqf_lookup_keys": (None, [_u8p, u32, u32, _u32p, u64, C.c_int, _u32p]),
            "or_sqf_delete_keys": (C.c_int, [_u8p, u32, u32, _u32p, u64, C.c_int]),
            "or_sqf_layout_sorted": (C.c_int, [_u8p, u32, u32, _u32p, u64]),
            "or_sqf_bulk_build": (C.c_int, [_u8p, u32, u32, _u32p, u64, C.c_int, C.c_int]),
            "or_sqf_extract": (u64, [_u8p, u32, u32, _u32p]),
            "or_sqf_insert_via_merge": (C.c_int, [_u8p, u32, u32, _u32p, u64, C.c_int]),
            "or_sqf_merge_two": (C.c_int, [_u8p, _u8p, u32, u32, C.c_int]),
            "or_sqfcpu_table_words": (sz, [u32, u32]),
            "or_rsqf_block_bytes": (sz, [u32]),
            "or_rsqf_num_blocks": (u32, [u32]),
            "or_rsqf_insert_fp": (i32, [_u8p, u32, u32, u32]),
            "or_rsqf_lookup_fp": (i32, [_u8p, u32, u32, u32]),
            "or_rsqf_insert_keys_sorted": (None, [_u8p, u32, u32, _u32p, u64, _i32p]),
            "or_rsqf_lookup_keys": (None, [_u8p, u32, u32, _u32p, u64, _i32p]),
            "or_rsqf_layout_sorted": (C.c_int, [_u8p, u32, u32, _u32p, u64]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


# ---------------------------------------------------------------- helpers
def mt_keys(seed: int, n: int, skip: int = 0) -> np.ndarray:
    """n draws of genrand_int32 after init_genrand(seed), skipping `skip`."""
    out = np.empty(n, np.uint32)
    lib().or_mt_fill(seed, skip, out, n)
    return out


def aphash(keys: np.ndarray, q: int, r: int) -> np.ndarray:
    keys = np.ascontiguousarray(keys, np.uint32)
    out = np.empty_like(keys)
    lib().or_hash_keys(keys, keys.size, q, r, APHASH, out)
    return out


def sqf_num_slots(q: int) -> int:
    return int(lib().or_sqf_num_slots(q))


def sqf_table_bytes(q: int, r: int) -> int:
    return int(lib().or_sqf_table_bytes(q, r))


def sqf_new(q: int, r: int) -> np.ndarray:
    return np.zeros(sqf_table_bytes(q, r), np.uint8)


def sqf_slots(t: np.ndarray, q: int, r: int) -> np.ndarray:
    """Logical slot values getElement(i) for i < (1<<q)*1.1."""
    ns = sqf_num_slots(q)
    bpe = (r + 3) // 8
    if bpe == 1:
        return t[:ns].astype(np.uint32)
    b = t[: ns * 2].reshape(ns, 2).astype(np.uint32)
    return (b[:, 0] << 8) | b[:, 1]


def sqf_bulk_build(t, q, r, keys, nodup=True, hash_kind=APHASH) -> int:
    keys = np.ascontiguousarray(keys, np.uint32)
    return lib().or_sqf_bulk_build(t, q, r, keys, keys.size, int(nodup), hash_kind)


def sqf_insert(t, q, r, keys, hash_kind=APHASH) -> int:
    keys = np.ascontiguousarray(keys, np.uint32)
    return lib().or_sqf_insert_keys(t, q, r, keys, keys.size, hash_kind)


def sqf_lookup(t, q, r, keys, hash_kind=APHASH) -> np.ndarray:
    keys = np.ascontiguousarray(keys, np.uint32)
    out = np.empty(keys.size, np.uint32)
    lib().or_sqf_lookup_keys(t, q, r, keys, keys.size, hash_kind, out)
    return out


def sqf_delete(t, q, r, keys, hash_kind=APHASH) -> int:
    keys = np.ascontiguousarray(keys, np.uint32)
    return lib().or_sqf_delete_keys(t, q, r, keys, keys.size, hash_kind)


def sqf_layout_sorted(t, q, r, fps) -> int:
    fps = np.ascontiguousarray(fps, np.uint32)
    return lib().or_sqf_layout_sorted(t, q, r, fps, fps.size)


def sqf_extract(t, q, r) -> np.ndarray:
    out = np.empty(sqf_num_slots(q) + 1, np.uint32)
    n = lib().or_sqf_extract(t, q, r, out)
    return out[:n].copy()


def sqf_insert_via_merge(t, q, r, keys, nodup) -> int:
    keys = np.ascontiguousarray(keys, np.uint32)
    return lib().or_sqf_insert_via_merge(t, q, r, keys, keys.size, int(nodup))


def sqf_merge_two(t1, t2, q, r, nodup) -> int:
    return lib().or_sqf_merge_two(t1, t2, q, r, int(nodup))


def rsqf_num_blocks(q: int) -> int:
    return int(lib().or_rsqf_num_blocks(q))


def rsqf_new(q: int, rbits: int = 5) -> np.ndarray:
    """Block array with one zeroed guard block after the logical blocks."""
    return np.zeros((rsqf_num_blocks(q) + 1) * lib().or_rsqf_block_bytes(rbits), np.uint8)


def rsqf_insert_sorted(blocks, q, keys, rbits=5) -> np.ndarray:
    keys = np.ascontiguousarray(keys, np.uint32)
    ret = np.empty(keys.size, np.int32)
    lib().or_rsqf_insert_keys_sorted(blocks, q, rbits, keys, keys.size, ret)
    return ret


def rsqf_lookup(blocks, q, keys, rbits=5) -> np.ndarray:
    keys = np.ascontiguousarray(keys, np.uint32)
    out = np.empty(keys.size, np.int32)
    lib().or_rsqf_lookup_keys(blocks, q, rbits, keys, keys.size, out)
    return out


def rsqf_layout_sorted(blocks, q, fps, rbits=5) -> int:
    fps = np.ascontiguousarray(fps, np.uint32)
    return lib().or_rsqf_layout_sorted(blocks, q, rbits, fps, fps.size)


# ------------------------------------------------------- reference (_ref)
class Ref:
    """ctypes view of the reference CPU code compiled by build_ref.sh."""

    def __init__(self):
        self.fnv = C.CDLL(os.path.join(REF_DIR, "libref_sqf_fnv.so"))
        self.ap = C.CDLL(os.path.join(REF_DIR, "libref_sqf_ap.so"))
        self.rsqf = C.CDLL(os.path.join(REF_DIR, "libref_rsqf.so"))
        # the same RSQF compiled with RBITS 8, when built
        p8 = os.path.join(REF_DIR, "libref_rsqf8.so")
        self.rsqf8 = C.CDLL(p8) if os.path.exists(p8) else None
        for L in (self.fnv, self.ap):
            L.ref_sqf_new.restype = C.c_void_p
            L.ref_sqf_new.argtypes = [C.c_uint, C.c_uint]
            L.ref_sqf_free.argtypes = [C.c_void_p]
            L.ref_sqf_insert_keys.argtypes = [C.c_void_p, _u32p, C.c_uint64]
            L.ref_sqf_lookup_keys.argtypes = [C.c_void_p, _u32p, C.c_uint64, _i32p]
            L.ref_sqf_hash.restype = C.c_uint32
            L.ref_sqf_hash.argtypes = [C.c_uint32, C.c_uint32]
            L.ref_sqf_table.restype = C.c_void_p
            L.ref_sqf_table.argtypes = [C.c_void_p]
            L.ref_sqf_words.restype = C.c_size_t
            L.ref_sqf_words.argtypes = [C.c_uint, C.c_uint]
        for R in (self.rsqf, self.rsqf8):
            if R is None:
                continue
            R.ref_rsqf_new.restype = C.c_void_p
            R.ref_rsqf_new.argtypes = [C.c_uint]
            R.ref_rsqf_free.argtypes = [C.c_void_p]
            R.ref_rsqf_insert.restype = C.c_int32
            R.ref_rsqf_insert.argtypes = [C.c_void_p, C.c_uint32]
            R.ref_rsqf_lookup.restype = C.c_int32
            R.ref_rsqf_lookup.argtypes = [C.c_void_p, C.c_uint32]
            R.ref_rsqf_blocks.restype = C.c_void_p
            R.ref_rsqf_blocks.argtypes = [C.c_void_p]
            R.ref_rsqf_block_bytes.restype = C.c_size_t
            R.ref_rsqf_num_blocks.restype = C.c_size_t
            R.ref_rsqf_num_blocks.argtypes = [C.c_uint]
            R.ref_aphash.restype = C.c_uint32
            R.ref_aphash.argtypes = [C.c_uint32, C.c_uint32]
            R.ref_mt_fill.argtypes = [C.c_uint32, C.c_uint64, _u32p, C.c_uint64]

    @staticmethod
    def available() -> bool:
        return all(
            os.path.exists(os.path.join(REF_DIR, n))
            for n in ("libref_sqf_fnv.so", "libref_sqf_ap.so", "libref_rsqf.so")
        )

    def mt_keys(self, seed, n, skip=0):
        out = np.empty(n, np.uint32)
        self.rsqf.ref_mt_fill(seed, skip, out, n)
        return out

    def sqf_build_insert(self, q, r, keys, gpu_hash=True):
        """Sequential insertItem of keys; returns logical slot values."""
        L = self.ap if gpu_hash else self.fnv
        f = L.ref_sqf_new(q, r)
        try:
            keys = np.ascontiguousarray(keys, np.uint32)
            L.ref_sqf_insert_keys(f, keys, keys.size)
            words = L.ref_sqf_words(q, r)
            tab = np.ctypeslib.as_array(
                C.cast(L.ref_sqf_table(f), C.POINTER(C.c_uint32)), shape=(words,)
            ).copy()
            return tab
        finally:
            L.ref_sqf_free(f)

    def sqf_insert_then_lookup(self, q, r, keys, lookups, gpu_hash=True):
        L = self.ap if gpu_hash else self.fnv
        f = L.ref_sqf_new(q, r)
        try:
            keys = np.ascontiguousarray(keys, np.uint32)
            lookups = np.ascontiguousarray(lookups, np.uint32)
            L.ref_sqf_insert_keys(f, keys, keys.size)
            out = np.empty(lookups.size, np.int32)
            L.ref_sqf_lookup_keys(f, lookups, lookups.size, out)
            return out
        finally:
            L.ref_sqf_free(f)


def sqfcpu_slots(words: np.ndarray, q: int, r: int) -> np.ndarray:
    """Logical slots of the CPU_version's bit-packed table (MSB first)."""
    ns = sqf_num_slots(q)
    w = r + 3
    idx = np.arange(ns, dtype=np.uint64)
    bit = idx * w
    word = (bit // 32).astype(np.int64)
    pos = (bit % 32).astype(np.uint64)
    ext = np.concatenate([words.astype(np.uint64), np.zeros(2, np.uint64)])
    two = (ext[word] << np.uint64(32)) | ext[word + 1]
    return ((two >> (np.uint64(64) - pos - np.uint64(w))) & np.uint64((1 << w) - 1)).astype(np.uint32)
