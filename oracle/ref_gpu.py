"""The reference's own standard-filter GPU kernels, run from a cubin --
TEST INFRASTRUCTURE ONLY.

``build_ref_gpu.sh`` compiles the reference's
``standardQuotientFilter/GPU_version/quotientFilter.cu`` unmodified into
``_ref/ref_sqf_gpu.cubin`` (device code only).  This module loads that cubin
through the CUDA driver API (in the current torch context) and runs the
reference's kernels in the order its host entry points launch them, with the
same launch shapes.  The host-side steps between the kernels -- Thrust
sort / unique / scans and CUB scans / flagged selects, whose results are
fully determined by their inputs -- are restated with torch ops; each
function cites the reference lines it follows.

Only tests may import this module, and only as a checker of the product
(``gpuquotientfilters_gb300``), which never imports it.

Memory layout of a table here: the ``T`` table bytes, then 4096 bytes of
padding; the first element past the last slot (slot index ``2^q * 1.1``) is
a guard element with only the occupied bit set.  The reference's delete
counts runs with loops of the form
``do b++ while(!isOccupied(b))`` (quotientFilter.cu:1150-1153, 1180-1182)
that, after deleting from the last run of the table, walk past its end
until they meet an occupied bit; the guard ends that walk at the first byte
past the table, where the next loop test (the element after the cluster is
not shifted) stops the delete.  Every other read past the table meets a zero
(empty) byte.  Keys equal to 0xFFFFFFFF are refused: the reference's insert
and delete rounds never retire them (quotientFilter.cu:431-433).
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_sqf_gpu.cubin")
NOT_FOUND = 0xFFFFFFFF
PAD = 4096
GUARD = 0x04  # occupied bit only: not empty, not shifted, not a continuation

# Itanium-ABI names of the reference kernels (quotientFilter.cu), as the
# cubin exports them.
_KERNELS = {
    "hashInputs": "_Z10hashInputsi15quotient_filterPjS0_",
    "lookUp": "_Z6lookUpi15quotient_filterPjS0_",
    "hashAndLookUp": "_Z13hashAndLookUpi15quotient_filterPjS0_",
    "locateInsertSuperclusters": "_Z25locateInsertSuperclustersi15quotient_filterPj",
    "superclusterBidding": "_Z19superclusterBiddingi15quotient_filterPjS0_PbS0_",
    "insertItemGPU": "_Z13insertItemGPUi15quotient_filterPjS0_S0_Pb",
    "quotienting": "_Z11quotientingijjPjS_",
    "findSegmentHeads": "_Z16findSegmentHeadsiPjS_",
    "calcOffsets": "_Z11calcOffsetsiPjS_PiS0_S0_",
    "shiftElements": "_Z13shiftElementsiPiS_PjS_S0_",
    "setMetadata": "_Z11setMetadataiPjS_S_",
    "writeRemainders": "_Z15writeRemaindersi15quotient_filterPjS0_",
    "setOccupiedBits": "_Z15setOccupiedBitsi15quotient_filterPj",
    "segmentStartLocations": "_Z21segmentStartLocationsiPjS_",
    "shiftSegments": "_Z13shiftSegmentsiPjS_iPb",
    "locateDeleteSuperclusters": "_Z25locateDeleteSuperclustersi15quotient_filterPj",
    "deleteItemGPU": "_Z13deleteItemGPUi15quotient_filterPjS0_Pb",
    "findSegmentStarts": "_Z17findSegmentStartsijPjS_",
    "layout": "_Z6layoutijPjS_PiS0_Pbi",
    "segmentedQFWrite": "_Z16segmentedQFWritei15quotient_filterPjS0_S0_Pii",
}


class _QF(C.Structure):
    """``struct quotient_filter`` (quotientFilter.cuh:25-31), passed by value."""
    _fields_ = [("qbits", C.c_uint), ("rbits", C.c_uint),
                ("bytesPerElement", C.c_uint), ("table", C.c_void_p)]


def available() -> bool:
    return os.path.exists(CUBIN)


_mod = None
_fns: dict = {}
_cu = None


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("CUDA driver call %s failed: %d" % (what, rc))


def _load():
    global _mod, _cu
    if _mod is not None:
        return
    import torch
    if not available():
        raise FileNotFoundError(CUBIN + " is missing (oracle/build_ref_gpu.sh builds it)")
    torch.cuda.init()
    torch.zeros(1, device="cuda")  # makes torch's primary context current
    _cu = C.CDLL("libcuda.so.1")
    _cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
    _cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
    _cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                   C.c_uint, C.c_uint, C.c_uint, C.c_void_p,
                                   C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
    mod = C.c_void_p()
    _check(_cu.cuModuleLoad(C.byref(mod), CUBIN.encode()), "cuModuleLoad")
    for k, name in _KERNELS.items():
        f = C.c_void_p()
        _check(_cu.cuModuleGetFunction(C.byref(f), mod, name.encode()), "cuModuleGetFunction " + k)
        _fns[k] = f
    _mod = mod


def _grid(n: int, threads: int):
    """The reference's 2-D grid: dim3((numBlocks + 31) / 32, 32)."""
    nb = (n + threads - 1) // threads
    return ((nb + 31) // 32, 32)


def _launch(name: str, n_cover: int, threads: int, *args):
    """Launch kernel ``name`` on torch's current stream with the reference's
    grid for ``n_cover`` items of ``threads`` per block."""
    import torch
    if n_cover <= 0:
        return
    gx, gy = _grid(n_cover, threads)
    holders = []
    for a in args:
        if isinstance(a, _QF):
            holders.append(a)
        elif isinstance(a, torch.Tensor):
            holders.append(C.c_void_p(a.data_ptr()))
        elif isinstance(a, bool):
            holders.append(C.c_bool(a))
        else:
            holders.append(C.c_int(int(a)))
    params = (C.c_void_p * len(holders))(*[C.cast(C.pointer(h), C.c_void_p) for h in holders])
    stream = torch.cuda.current_stream().cuda_stream
    _check(_cu.cuLaunchKernel(_fns[name], gx, gy, 1, threads, 1, 1, 0, C.c_void_p(stream),
                              params, None), "cuLaunchKernel " + name)


class RefFilter:
    """A standard quotient filter driven by the reference's kernels."""

    def __init__(self, q: int, r: int):
        import torch
        _load()
        assert q + r <= 32 and (r + 3) % 8 == 0
        self.q, self.r = q, r
        self.bpe = (r + 3) // 8
        self.slots = int((1 << q) * 1.1)  # filterSize (quotientFilter.cu:535)
        self.T = int((1 << q) * (r + 3) // 8 * 1.1)  # calcNumSlotsGPU (:37-42), bytes
        # the guard is the element at slot index `slots` (big-endian, like
        # every element); with 2-byte slots its high (zero) byte can be the
        # table's last byte, which no slot index reaches
        self.guard_off = self.slots * self.bpe
        self.buf = torch.zeros(max(self.T, self.guard_off + self.bpe) + PAD,
                               dtype=torch.uint8, device="cuda")
        self.buf[self.guard_off + self.bpe - 1] = GUARD
        self.qf = _QF(q, r, self.bpe, self.buf.data_ptr())

    def table(self) -> np.ndarray:
        import torch
        torch.cuda.synchronize()
        tail = self.buf[self.guard_off:].cpu().numpy()
        want = np.zeros_like(tail)
        want[self.bpe - 1] = GUARD
        assert (tail == want).all(), "reference kernels wrote past the table"
        return self.buf[: self.T].cpu().numpy()


def device_keys(a):
    """Keys as a CUDA int32 tensor holding the uint32 bits (host arrays are
    copied in; CUDA tensors pass through)."""
    import torch
    if isinstance(a, torch.Tensor):
        return a.contiguous()
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return torch.from_numpy(a.view(np.int32)).cuda()


def _u32(a):
    t = device_keys(a)
    if bool((t == -1).any()):
        raise ValueError("key 0xFFFFFFFF never leaves the reference's insert/delete queue")
    return t


def _as_u64(t):
    import torch
    return t.to(torch.int64) & 0xFFFFFFFF


def _fingerprints_sorted(f: RefFilter, d_keys, nodup: bool):
    """hashInputs, thrust::sort and (NoDup) thrust::unique
    (quotientFilter.cu:1470-1482)."""
    import torch
    n = d_keys.numel()
    fps = torch.zeros(n, dtype=torch.int32, device="cuda")
    _launch("hashInputs", n, 128, n, f.qf, d_keys, fps)
    s = torch.sort(_as_u64(fps)).values
    if nodup:
        s = torch.unique_consecutive(s)
    return s.to(torch.int32).contiguous()


def _quotienting(f: RefFilter, quotients):
    """quotienting kernel (quotientFilter.cu:1485-1490): the fingerprint
    array becomes quotients; remainders are written beside it."""
    import torch
    n = quotients.numel()
    rem = torch.zeros(n, dtype=torch.int32, device="cuda")
    _launch("quotienting", n, 768, n, f.q, f.r, quotients, rem)
    return rem


def bulk_build_segmented_layouts(f: RefFilter, keys, nodup: bool) -> None:
    """bulkBuildSegmentedLayouts (quotientFilter.cu:1446-1559)."""
    import torch
    d_keys = _u32(keys)
    quot = _fingerprints_sorted(f, d_keys, nodup)
    n = quot.numel()
    rem = _quotienting(f, quot)
    q = f.q
    nseg = (1 << q) // q + 1
    seg_starts = torch.zeros(nseg, dtype=torch.int32, device="cuda")
    _launch("findSegmentStarts", n, 256, n, q, quot, seg_starts)
    shifts = torch.zeros(nseg, dtype=torch.int32, device="cuda")
    overflows = torch.zeros(nseg, dtype=torch.int32, device="cuda")
    changed = torch.zeros(1, dtype=torch.bool, device="cuda")
    for _ in range(nseg + 2):  # the reference loops until nothing changes (:1516-1530)
        shifts.copy_(overflows)
        _launch("layout", nseg, 256, nseg, q, quot, seg_starts, shifts, overflows, changed, n)
        done = not bool(changed.item())
        changed.zero_()
        if done:
            break
    else:
        raise RuntimeError("reference layout did not converge")
    _launch("segmentedQFWrite", nseg, 128, nseg, f.qf, quot, rem, seg_starts, shifts, n)
    _launch("setOccupiedBits", n, 512, n, f.qf, quot)


def _initial_locations(quot):
    """thrust::exclusive_scan_by_key over an array of ones, plus the
    quotient (quotientFilter.cu:791-795, 985-989): each item's location is
    its quotient plus its rank among the items of that quotient."""
    import torch
    n = quot.numel()
    q64 = _as_u64(quot)
    idx = torch.arange(n, device="cuda", dtype=torch.int64)
    head = torch.ones(n, dtype=torch.bool, device="cuda")
    head[1:] = q64[1:] != q64[:-1]
    first = torch.where(head, idx, torch.zeros_like(idx))
    first = torch.cummax(first, 0).values
    return (q64 + (idx - first)).to(torch.int32).contiguous()


def _segment_labels(f: RefFilter, quot):
    """findSegmentHeads + thrust::inclusive_scan (quotientFilter.cu:811-820)."""
    import torch
    n = quot.numel()
    starts = torch.zeros(n, dtype=torch.int32, device="cuda")
    _launch("findSegmentHeads", n, 768, n, quot, starts)
    return torch.cumsum(starts.to(torch.int64), 0).to(torch.int32).contiguous()


def _write_filter(f: RefFilter, quot, rem, loc):
    """setMetadata, writeRemainders, setOccupiedBits (quotientFilter.cu:850-863)."""
    n = quot.numel()
    _launch("setMetadata", n, 1024, n, rem, quot, loc)
    _launch("writeRemainders", n, 1024, n, f.qf, rem, loc)
    _launch("setOccupiedBits", n, 512, n, f.qf, quot)


def bulk_build_sequential_shifts(f: RefFilter, keys, nodup: bool) -> None:
    """bulkBuildSequentialShifts (quotientFilter.cu:930-1058)."""
    import torch
    d_keys = _u32(keys)
    quot = _fingerprints_sorted(f, d_keys, nodup)
    n = quot.numel()
    rem = _quotienting(f, quot)
    loc = _initial_locations(quot)
    labels = _segment_labels(f, quot)
    nseg = int(labels[-1].item()) + 1
    seg_loc = torch.zeros(nseg, dtype=torch.int32, device="cuda")
    # launched with the grid of findSegmentHeads (768-item blocks) and 1024
    # threads per block (quotientFilter.cu:1020-1022)
    gx_items = ((n + 767) // 768) * 1024
    _launch("segmentStartLocations", gx_items, 1024, n, labels, seg_loc)
    changed = torch.zeros(1, dtype=torch.bool, device="cuda")
    for _ in range(n + 2):  # the reference loops until no segment moves (:1029-1036)
        _launch("shiftSegments", nseg, 192, nseg, seg_loc, loc, n, changed)
        done = not bool(changed.item())
        changed.zero_()
        if done:
            break
    else:
        raise RuntimeError("reference shiftSegments did not converge")
    _write_filter(f, quot, rem, loc)


def bulk_build_parallel_merging(f: RefFilter, keys, nodup: bool) -> None:
    """bulkBuildParallelMerging (quotientFilter.cu:737-878)."""
    import torch
    d_keys = _u32(keys)
    quot = _fingerprints_sorted(f, d_keys, nodup)
    n = quot.numel()
    rem = _quotienting(f, quot)
    loc = _initial_locations(quot)
    labels = _segment_labels(f, quot)
    nseg = int(labels[-1].item()) + 1
    # (int) ceil(log2((float)numSegments)) in single precision (:824)
    nloops = int(math.ceil(float(np.log2(np.float32(nseg)))))
    offsets = torch.zeros(nseg, dtype=torch.int32, device="cuda")
    carry = torch.zeros(nseg, dtype=torch.int32, device="cuda")
    credits = torch.zeros(n, dtype=torch.int32, device="cuda")
    for _ in range(nloops):
        offsets.zero_()
        carry.zero_()
        _launch("calcOffsets", n, 256, n, loc, labels, offsets, credits, carry)
        _launch("shiftElements", n, 768, n, offsets, credits, loc, carry, labels)
    _write_filter(f, quot, rem, loc)


def _rounds(f: RefFilter, keys, locate: str, apply: str, apply_threads: int,
            with_locations: bool) -> int:
    """The supercluster rounds shared by insert (quotientFilter.cu:533-634)
    and superclusterDeletes (:1202-1297): label superclusters, let every
    queued item bid for its supercluster, apply the winners, drop them from
    the queue (cub::DeviceSelect::Flagged), until the queue is empty."""
    import torch
    fs = f.slots
    max_sc = f.T + 1
    winners = torch.full((max_sc,), -1, dtype=torch.int32, device="cuda")
    locations = torch.zeros(max_sc, dtype=torch.int32, device="cuda")
    queue = _u32(keys)
    flags = torch.zeros(max(queue.numel(), 1), dtype=torch.bool, device="cuda")
    ind = torch.zeros(fs, dtype=torch.int32, device="cuda")
    rounds = 0
    left = queue.numel()
    while left > 0:
        rounds += 1
        if rounds > len(keys) + 2:
            raise RuntimeError("reference rounds did not drain the queue")
        _launch(locate, fs, 1024, fs, f.qf, ind)
        labels = torch.cumsum(ind.to(torch.int64), 0).to(torch.int32).contiguous()
        nsc = int(labels[fs - 1].item()) + 1
        _launch("superclusterBidding", left, 128, left, f.qf, queue, labels, flags, winners)
        if with_locations:
            _launch(apply, nsc, apply_threads, nsc, f.qf, queue, winners, locations, flags)
        else:
            _launch(apply, nsc, apply_threads, nsc, f.qf, queue, winners, flags)
        queue = queue[flags[:left]].contiguous()
        left = queue.numel()
    return rounds


def insert(f: RefFilter, keys) -> int:
    """insert (quotientFilter.cu:533-634); returns the number of rounds."""
    return _rounds(f, keys, "locateInsertSuperclusters", "insertItemGPU", 256, True)


def supercluster_deletes(f: RefFilter, keys) -> int:
    """superclusterDeletes (quotientFilter.cu:1202-1297); returns the
    number of rounds."""
    return _rounds(f, keys, "locateDeleteSuperclusters", "deleteItemGPU", 1024, False)


def _host(t, keys):
    """Results as a host uint32 array for host keys, else the CUDA tensor."""
    import torch
    if isinstance(keys, torch.Tensor):
        return t
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint32)


def unsorted_lookups(f: RefFilter, keys):
    """launchUnsortedLookups (quotientFilter.cu:359-381)."""
    import torch
    d = device_keys(keys)
    out = torch.zeros(d.numel(), dtype=torch.int32, device="cuda")
    _launch("hashAndLookUp", d.numel(), 1024, d.numel(), f.qf, d, out)
    return _host(out, keys)


def sorted_lookups(f: RefFilter, keys):
    """launchSortedLookups (quotientFilter.cu:272-318): hash, sort by hash
    with the input index, look up, sort the results back by index."""
    import torch
    d = device_keys(keys)
    n = d.numel()
    h = torch.zeros(n, dtype=torch.int32, device="cuda")
    _launch("hashInputs", n, 128, n, f.qf, d, h)
    order = torch.sort(_as_u64(h), stable=True).indices
    hs = h[order].contiguous()
    res = torch.zeros(n, dtype=torch.int32, device="cuda")
    _launch("lookUp", n, 1024, n, f.qf, hs, res)
    out = torch.empty_like(res)
    out[order] = res
    return _host(out, keys)
