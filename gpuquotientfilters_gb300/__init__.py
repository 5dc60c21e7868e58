"""GB300 quotient-filter engine: Python mirror of the reference host API.

The functions below carry the names, argument meaning and return value
(elapsed milliseconds) of owensgroup/GPUQuotientFilters'
``quotientFilter.cuh`` and ``RSQF.cuh``; they call the C ABI of
``libgqf.so`` (declared in ``include/gqf.h``) through ctypes.  Device
buffers are passed as CUDA tensors (or raw integer device pointers); torch
only provides the memory and streams.

Where the reference prints and carries on (or aborts), these raise
``GQFError`` with the library's status.  There is no CPU fallback: if
``libgqf.so`` cannot be loaded, importing a compute entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgqf.so")
NOT_FOUND = 0xFFFFFFFF
RBITS = 5
SLOTS_PER_BLOCK = 64

(GQF_OK, GQF_ERR_ARG, GQF_ERR_FULL, GQF_ERR_CUDA, GQF_ERR_TIMEOUT, GQF_ERR_NOMEM, GQF_ERR_MISMATCH,
 GQF_ERR_LIMIT, GQF_ERR_FORMAT, GQF_ERR_IO) = range(10)


class GQFError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__("%s: %s (status %d)" % (what, _lib().gqf_status_string(status).decode(), status))


class quotient_filter(C.Structure):
    """struct quotient_filter (quotientFilter.cuh:25-31)."""
    _fields_ = [("qbits", C.c_uint), ("rbits", C.c_uint), ("bytesPerElement", C.c_uint),
                ("table", C.c_void_p)]


class gqf_sqf_job(C.Structure):
    """One filter of a batch (include/gqf.h): bulk build from n_build keys,
    then n_lookup unsorted lookups."""
    _fields_ = [("filter", quotient_filter), ("n_build", C.c_int), ("d_build_keys", C.c_void_p),
                ("n_lookup", C.c_int), ("d_lookup_keys", C.c_void_p), ("d_results", C.c_void_p)]


class gqf_batch_tuning(C.Structure):
    _fields_ = [("bucket_bits", C.c_int), ("scatter_chunk", C.c_int), ("cta_threads", C.c_int),
                ("items_per_thread", C.c_int)]


class gqf_server_config(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_streams", C.c_int), ("max_op_keys", C.c_int),
                ("coalesce", C.c_int)]


class gqf_completion(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int), ("submit_us", C.c_double), ("start_us", C.c_double),
                ("done_us", C.c_double)]


class countingQuotientFilterGPU(C.Structure):
    """struct countingQuotientFilterGPU (RSQF.cuh:32-37)."""
    _fields_ = [("qbits", C.c_uint), ("numBlocks", C.c_uint), ("blocks", C.c_void_p)]


_L = None


def build(force: bool = False) -> str:
    """Compiles libgqf.so in-tree for sm_103a (see buildlib.py)."""
    from . import buildlib
    return buildlib.build(force=force)


def _lib():
    global _L
    if _L is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libgqf.so is not built: run gpuquotientfilters_gb300.build()")
        L = C.CDLL(LIB_PATH)
        vp, u32, i32, f32p = C.c_void_p, C.c_uint32, C.c_int, C.POINTER(C.c_float)
        qfp = C.POINTER(quotient_filter)
        cqfp = C.POINTER(countingQuotientFilterGPU)
        sig = {
            "gqf_sqf_table_bytes": (C.c_size_t, [C.c_uint, C.c_uint]),
            "gqf_sqf_num_slots": (C.c_uint, [C.c_uint]),
            "gqf_aphash": (C.c_uint, [C.c_uint, C.c_uint]),
            "gqf_rsqf_num_blocks": (C.c_size_t, [C.c_uint]),
            "gqf_mt19937_fill": (None, [u32, C.c_uint64, vp, C.c_uint64]),
            "gqf_status_string": (C.c_char_p, [i32]),
            "gqf_stream_status": (i32, [vp]),
            "gqf_sqf_init": (i32, [qfp, C.c_uint, C.c_uint]),
            "gqf_sqf_free": (i32, [qfp]),
            "gqf_sqf_bulk_build": (i32, [qfp, i32, vp, i32, vp, f32p]),
            "gqf_sqf_lookup_unsorted": (i32, [qfp, i32, vp, vp, vp, f32p]),
            "gqf_sqf_lookup_sorted": (i32, [qfp, i32, vp, vp, vp, f32p]),
            "gqf_sqf_insert": (i32, [qfp, i32, vp, vp, f32p]),
            "gqf_sqf_delete": (i32, [qfp, i32, vp, vp, f32p]),
            "gqf_sqf_insert_via_merge": (i32, [qfp, vp, i32, vp, i32, i32, vp, f32p]),
            "gqf_sqf_merge": (i32, [qfp, qfp, i32, vp, f32p]),
            "gqf_sqf_bulk_build_noalloc": (i32, [qfp, i32, vp, i32, vp]),
            "gqf_kernel_launches": (C.c_ulonglong, []),
            "gqf_rsqf_init": (i32, [cqfp, C.c_uint]),
            "gqf_rsqf_free": (i32, [cqfp]),
            "gqf_rsqf_insert": (i32, [cqfp, i32, vp, vp, vp, f32p]),
            "gqf_rsqf_lookup_sorted": (i32, [cqfp, i32, vp, vp, vp, f32p]),
            "gqf_rsqf_lookup_unsorted": (i32, [cqfp, i32, vp, vp, vp, f32p]),
            "gqf_rsqf8_num_blocks": (C.c_size_t, [C.c_uint]),
            "gqf_rsqf8_init": (i32, [cqfp, C.c_uint]),
            "gqf_rsqf8_free": (i32, [cqfp]),
            "gqf_rsqf8_insert": (i32, [cqfp, i32, vp, vp, vp, f32p]),
            "gqf_rsqf8_lookup_sorted": (i32, [cqfp, i32, vp, vp, vp, f32p]),
            "gqf_rsqf8_lookup_unsorted": (i32, [cqfp, i32, vp, vp, vp, f32p]),
            "gqf_batch_create": (i32, [C.POINTER(C.c_void_p), C.POINTER(gqf_sqf_job), i32, i32,
                                       C.POINTER(gqf_batch_tuning)]),
            "gqf_batch_run": (i32, [C.c_void_p, i32, vp, f32p]),
            "gqf_batch_tuning_of": (i32, [C.c_void_p, C.POINTER(gqf_batch_tuning)]),
            "gqf_batch_destroy": (i32, [C.c_void_p]),
            "gqf_workspace_reserve": (i32, [vp, C.c_size_t, C.POINTER(C.c_size_t)]),
            "gqf_workspace_release": (i32, [vp]),
            "gqf_sqf_update_workspace_bytes": (C.c_size_t, [C.c_uint, C.c_uint, i32]),
            "gqf_server_create": (i32, [C.POINTER(C.c_void_p), qfp, i32, C.POINTER(gqf_server_config)]),
            "gqf_server_submit": (i32, [C.c_void_p, i32, i32, vp, i32, vp, C.POINTER(C.c_uint64)]),
            "gqf_server_poll": (i32, [C.c_void_p, C.POINTER(gqf_completion), i32, C.POINTER(C.c_int)]),
            "gqf_server_drain": (i32, [C.c_void_p]),
            "gqf_server_info": (i32, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_size_t)]),
            "gqf_server_destroy": (i32, [C.c_void_p]),
            "gqf_sqf_image_bytes": (C.c_size_t, [qfp]),
            "gqf_rsqf_image_bytes": (C.c_size_t, [cqfp]),
            "gqf_sqf_save": (i32, [qfp, vp, C.c_size_t, vp]),
            "gqf_rsqf_save": (i32, [cqfp, vp, C.c_size_t, vp]),
            "gqf_sqf_load": (i32, [qfp, vp, C.c_size_t]),
            "gqf_rsqf_load": (i32, [cqfp, vp, C.c_size_t]),
            "gqf_sqf_save_file": (i32, [qfp, C.c_char_p]),
            "gqf_rsqf_save_file": (i32, [cqfp, C.c_char_p]),
            "gqf_sqf_load_file": (i32, [qfp, C.c_char_p]),
            "gqf_rsqf_load_file": (i32, [cqfp, C.c_char_p]),
            "gqf_debug_lookback_probe": (i32, [vp, C.c_uint, C.c_uint, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _L = L
    return _L


def lib():
    """The loaded libgqf.so (ctypes.CDLL)."""
    return _lib()


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    return int(x.data_ptr())


def _stream_ptr(stream) -> int:
    if stream is None:
        return 0
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)


def _check(st: int, what: str):
    if st != GQF_OK:
        raise GQFError(st, what)


def _timed(fn, *args, stream=None, sync=True):
    """Calls a C ABI op.  sync=True: the call waits for the op and returns
    its device time in ms (a device-side error is its status).  sync=False:
    the op is only queued on `stream` and None is returned; a deferred
    device-side error shows in gqf_stream_status / stream_status()."""
    if not sync:
        _check(fn(*args, _stream_ptr(stream), None), fn.__name__)
        return None
    ms = C.c_float(0.0)
    st = fn(*args, _stream_ptr(stream), C.byref(ms))
    _check(st, fn.__name__)
    return ms.value


def stream_status(stream=None) -> None:
    """Waits for `stream` and raises GQFError if an op queued on it with
    sync=False hit a device-side error (gqf_stream_status)."""
    _check(_lib().gqf_stream_status(_stream_ptr(stream)), "gqf_stream_status")


# ------------------------------------------------------------- host helpers
def calcNumSlotsGPU(q: int, r: int) -> int:
    """Table bytes (quotientFilter.cu:37-42)."""
    return int(_lib().gqf_sqf_table_bytes(q, r))


def num_slots(q: int) -> int:
    return int(_lib().gqf_sqf_num_slots(q))


def Normal_APHash(value: int, tableSize: int) -> int:
    return int(_lib().gqf_aphash(value, tableSize))


Normal_APHashGPU = Normal_APHash


def calcNumBlocksGPU(q: int) -> int:
    return int(_lib().gqf_rsqf_num_blocks(q))


def mt19937(seed: int, n: int, skip: int = 0):
    """n draws of genrand_int32 after init_genrand(seed) (numpy uint32)."""
    import numpy as np
    out = np.empty(n, np.uint32)
    _lib().gqf_mt19937_fill(seed, skip, out.ctypes.data, n)
    return out


# --------------------------------------------------- standard quotient filter
def initFilterGPU(q: int, r: int) -> quotient_filter:
    qf = quotient_filter()
    _check(_lib().gqf_sqf_init(C.byref(qf), q, r), "initFilterGPU")
    return qf


def freeFilterGPU(qf: quotient_filter) -> None:
    _check(_lib().gqf_sqf_free(C.byref(qf)), "freeFilterGPU")


def bulkBuildSegmentedLayouts(qf, numValues, d_insertValues, NoDuplicates, stream=None, sync=True):
    return _timed(_lib().gqf_sqf_bulk_build, C.byref(qf), int(numValues), _ptr(d_insertValues),
                  int(bool(NoDuplicates)), stream=stream, sync=sync)


# The reference's other two bulk builds produce the same (canonical) table.
bulkBuildParallelMerging = bulkBuildSegmentedLayouts
bulkBuildSequentialShifts = bulkBuildSegmentedLayouts


def launchUnsortedLookups(qf, numValues, d_lookupValues, d_returnValues, stream=None, sync=True):
    return _timed(_lib().gqf_sqf_lookup_unsorted, C.byref(qf), int(numValues), _ptr(d_lookupValues),
                  _ptr(d_returnValues), stream=stream, sync=sync)


def launchSortedLookups(qf, numValues, d_lookupValues, d_returnValues, stream=None, sync=True):
    return _timed(_lib().gqf_sqf_lookup_sorted, C.byref(qf), int(numValues), _ptr(d_lookupValues),
                  _ptr(d_returnValues), stream=stream, sync=sync)


def insert(qf, numValues, d_insertValues, stream=None, sync=True):
    return _timed(_lib().gqf_sqf_insert, C.byref(qf), int(numValues), _ptr(d_insertValues), stream=stream, sync=sync)


def superclusterDeletes(qf, numValues, d_deleteValues, stream=None, sync=True):
    return _timed(_lib().gqf_sqf_delete, C.byref(qf), int(numValues), _ptr(d_deleteValues), stream=stream, sync=sync)


def insertViaMerge(qf, d_insertedValues, numOldValues, d_newValues, numNewValues, NoDuplicates,
                   stream=None, sync=True):
    return _timed(_lib().gqf_sqf_insert_via_merge, C.byref(qf), _ptr(d_insertedValues), int(numOldValues),
                  _ptr(d_newValues), int(numNewValues), int(bool(NoDuplicates)), stream=stream, sync=sync)


def mergeTwoFilters(qf1, qf2, NoDuplicates, stream=None, sync=True):
    return _timed(_lib().gqf_sqf_merge, C.byref(qf1), C.byref(qf2), int(bool(NoDuplicates)), stream=stream, sync=sync)


def table_bytes(qf):
    """Host copy of the table (numpy uint8), for inspection and tests."""
    import numpy as np
    n = calcNumSlotsGPU(qf.qbits, qf.rbits)
    host = np.empty(n, np.uint8)
    _memcpy_d2h(host.ctypes.data, qf.table, n)
    return host


def _memcpy_d2h(dst: int, src: int, nbytes: int):
    st = _cudart().cudaMemcpy(C.c_void_p(dst), C.c_void_p(src), C.c_size_t(nbytes), 2)
    if st != 0:
        raise RuntimeError("cudaMemcpy failed: %d" % st)


def _memcpy_h2d(dst: int, src: int, nbytes: int):
    st = _cudart().cudaMemcpy(C.c_void_p(dst), C.c_void_p(src), C.c_size_t(nbytes), 1)
    if st != 0:
        raise RuntimeError("cudaMemcpy failed: %d" % st)


_CUDART = None


def _cudart():
    global _CUDART
    if _CUDART is None:
        import glob
        import torch  # noqa: F401  (loads the CUDA runtime torch ships)
        cands = []
        for d in [os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")]:
            cands += sorted(glob.glob(os.path.join(d, "libcudart.so*")))
        L = None
        for c in cands + ["libcudart.so", "libcudart.so.13", "libcudart.so.12"]:
            try:
                L = C.CDLL(c)
                break
            except OSError:
                continue
        if L is None:
            raise OSError("libcudart not found")
        L.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        L.cudaMemcpy.restype = C.c_int
        _CUDART = L
    return _CUDART


def printQuotientFilterGPU(qf) -> None:
    """printQuotientFilterGPU (quotientFilter.cu:383-405): metadata row then
    remainder row, ten slots per line."""
    t = table_bytes(qf)
    bpe = qf.bytesPerElement
    n = num_slots(qf.qbits)
    print("Printing metadata and remainders:")
    for i in range(n // 10):
        els = []
        for j in range(10):
            k = (10 * i + j) * bpe
            e = 0
            for b in range(bpe):
                e = (e << 8) | int(t[k + b])
            els.append(e)
        print("".join("%u \t" % (e & 7) for e in els))
        print("".join("%u \t" % (e >> 3) for e in els))
        print(" --------------------------------------------------------------------- ")
    print()


# ----------------------------------------- rank-and-select quotient filter
# rbits: the remainder width the reference fixes at compile time (RBITS,
# RSQF.cuh:21): 5 as shipped, or 8 (the gqf_rsqf8_* entry points).  A
# filter remembers the width it was made with.
def _rsqf(cqf, name):
    return getattr(_lib(), ("gqf_rsqf8_" if getattr(cqf, "_rbits", 5) == 8 else "gqf_rsqf_") + name)


def initCQFGPU(q: int, rbits: int = RBITS) -> countingQuotientFilterGPU:
    if rbits not in (5, 8):
        raise GQFError(GQF_ERR_ARG, "initCQFGPU: remainder width must be 5 or 8")
    cqf = countingQuotientFilterGPU()
    cqf._rbits = rbits
    _check(_rsqf(cqf, "init")(C.byref(cqf), q), "initCQFGPU")
    return cqf


def freeCQFGPU(cqf) -> None:
    _check(_rsqf(cqf, "free")(C.byref(cqf)), "freeCQFGPU")


def insertGPU(cqf, numValues, d_insertValues, d_returnValues, stream=None, sync=True):
    return _timed(_rsqf(cqf, "insert"), C.byref(cqf), int(numValues), _ptr(d_insertValues),
                  _ptr(d_returnValues), stream=stream, sync=sync)


def launchLookups(cqf, numValues, d_lookupValues, d_slotValuesArray, stream=None, sync=True):
    return _timed(_rsqf(cqf, "lookup_sorted"), C.byref(cqf), int(numValues), _ptr(d_lookupValues),
                  _ptr(d_slotValuesArray), stream=stream, sync=sync)


def launchUnsortedLookupsRSQF(cqf, numValues, d_lookupValues, d_slotValuesArray, stream=None, sync=True):
    return _timed(_rsqf(cqf, "lookup_unsorted"), C.byref(cqf), int(numValues), _ptr(d_lookupValues),
                  _ptr(d_slotValuesArray), stream=stream, sync=sync)


def rsqf_blocks_bytes(cqf):
    """Host copy of the packed blocks (numpy uint8), guard block included."""
    import numpy as np
    n = (cqf.numBlocks + 1) * (17 + 8 * getattr(cqf, "_rbits", 5))
    host = np.empty(n, np.uint8)
    _memcpy_d2h(host.ctypes.data, cqf.blocks, n)
    return host


# ------------------------------------------------------------ serialization
def saveFilter(qf, path: str) -> None:
    """Writes the SQF image (64-byte header + slot table) to `path`."""
    _check(_lib().gqf_sqf_save_file(C.byref(qf), os.fsencode(path)), "gqf_sqf_save_file")


def loadFilter(path: str) -> quotient_filter:
    """A new SQF holding the image at `path` (free with freeFilterGPU)."""
    qf = quotient_filter()
    _check(_lib().gqf_sqf_load_file(C.byref(qf), os.fsencode(path)), "gqf_sqf_load_file")
    return qf


def saveCQF(cqf, path: str) -> None:
    """Writes the RSQF image (64-byte header + packed blocks) to `path`."""
    _check(_lib().gqf_rsqf_save_file(C.byref(cqf), os.fsencode(path)), "gqf_rsqf_save_file")


def loadCQF(path: str) -> countingQuotientFilterGPU:
    """A new RSQF holding the image at `path` (free with freeCQFGPU)."""
    cqf = countingQuotientFilterGPU()
    _check(_lib().gqf_rsqf_load_file(C.byref(cqf), os.fsencode(path)), "gqf_rsqf_load_file")
    return cqf


def filter_image(qf) -> bytes:
    """The SQF image in memory."""
    n = int(_lib().gqf_sqf_image_bytes(C.byref(qf)))
    buf = C.create_string_buffer(n)
    _check(_lib().gqf_sqf_save(C.byref(qf), buf, n, None), "gqf_sqf_save")
    return buf.raw


def filter_from_image(img: bytes) -> quotient_filter:
    qf = quotient_filter()
    _check(_lib().gqf_sqf_load(C.byref(qf), img, len(img)), "gqf_sqf_load")
    return qf


# ------------------------------------------------------------ batched filters
BATCH_DIRECT, BATCH_GRAPH, BATCH_PERSISTENT = 0, 1, 2


class Batch:
    """Many filters built and queried together (gqf_batch_* in
    include/gqf.h): by one launch per pipeline kernel, replayed from a
    captured CUDA graph, or by one persistent cooperative kernel.

    jobs: sequence of (filter, build_keys or None, lookup_keys or None,
    results or None); tensors or raw device pointers with lengths taken from
    the tensors (pass (ptr, n) tuples for raw pointers)."""

    def __init__(self, jobs, no_duplicates=True, bucket_bits=0, scatter_chunk=0, cta_threads=0,
                 items_per_thread=0):
        def ptr_len(x):
            if x is None:
                return 0, 0
            if isinstance(x, tuple):
                return int(x[0]), int(x[1])
            return int(x.data_ptr()), int(x.numel())
        arr = (gqf_sqf_job * len(jobs))()
        self._keep = list(jobs)
        for i, (qf, bk, lk, res) in enumerate(jobs):
            bp, bn = ptr_len(bk)
            lp, ln = ptr_len(lk)
            rp, _ = ptr_len(res)
            arr[i] = gqf_sqf_job(qf, bn, bp, ln, lp, rp)
        tune = gqf_batch_tuning(int(bucket_bits), int(scatter_chunk), int(cta_threads), int(items_per_thread))
        h = C.c_void_p()
        _check(_lib().gqf_batch_create(C.byref(h), arr, len(jobs), int(bool(no_duplicates)), C.byref(tune)),
               "gqf_batch_create")
        self._h = h

    def run(self, use_graph=True, stream=None, persistent=False) -> float:
        """Runs the batch once and returns its device time in ms."""
        mode = BATCH_PERSISTENT if persistent else (BATCH_GRAPH if use_graph else BATCH_DIRECT)
        ms = C.c_float(0.0)
        _check(_lib().gqf_batch_run(self._h, mode, _stream_ptr(stream), C.byref(ms)), "gqf_batch_run")
        return ms.value

    def tuning(self):
        t = gqf_batch_tuning()
        _check(_lib().gqf_batch_tuning_of(self._h, C.byref(t)), "gqf_batch_tuning_of")
        return {"bucket_bits": t.bucket_bits, "scatter_chunk": t.scatter_chunk, "cta_threads": t.cta_threads,
                "items_per_thread": t.items_per_thread}

    def close(self):
        if getattr(self, "_h", None):
            _lib().gqf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------- served filters
SERVE_LOOKUP, SERVE_INSERT, SERVE_DELETE = 0, 1, 2


class Server:
    """Request loop with continuous batching over resident filters
    (gqf_server_* in include/gqf.h).  submit() takes host buffers (pinned
    torch tensors or numpy arrays) and keeps them alive until the request
    completes; results of a lookup land in its results buffer."""

    def __init__(self, filters, hbm_budget=0, max_streams=0, max_op_keys=0, coalesce=True):
        arr = (quotient_filter * len(filters))(*filters)
        cfg = gqf_server_config(int(hbm_budget), int(max_streams), int(max_op_keys), int(bool(coalesce)))
        h = C.c_void_p()
        _check(_lib().gqf_server_create(C.byref(h), arr, len(filters), C.byref(cfg)), "gqf_server_create")
        self._h = h
        self._live = {}

    @staticmethod
    def _host_ptr(x):
        if x is None:
            return 0
        if hasattr(x, "data_ptr"):
            return int(x.data_ptr())
        return int(x.ctypes.data)

    def submit(self, filt: int, op: int, keys, results=None) -> int:
        rid = C.c_uint64()
        n = int(keys.numel() if hasattr(keys, "numel") else keys.size)
        _check(_lib().gqf_server_submit(self._h, int(filt), int(op), self._host_ptr(keys), n,
                                        self._host_ptr(results), C.byref(rid)), "gqf_server_submit")
        self._live[rid.value] = (keys, results)
        return rid.value

    def poll(self, max_items=4096):
        buf = (gqf_completion * max_items)()
        cnt = C.c_int()
        _check(_lib().gqf_server_poll(self._h, buf, max_items, C.byref(cnt)), "gqf_server_poll")
        out = []
        for i in range(cnt.value):
            c = buf[i]
            self._live.pop(c.id, None)
            out.append({"id": c.id, "status": c.status, "submit_us": c.submit_us, "start_us": c.start_us,
                        "done_us": c.done_us})
        return out

    def drain(self):
        _check(_lib().gqf_server_drain(self._h), "gqf_server_drain")

    def info(self):
        ns, hb = C.c_int(), C.c_size_t()
        _check(_lib().gqf_server_info(self._h, C.byref(ns), C.byref(hb)), "gqf_server_info")
        return {"streams": ns.value, "hbm_bytes": hb.value}

    def close(self):
        if getattr(self, "_h", None):
            _lib().gqf_server_destroy(self._h)
            self._h = None
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
