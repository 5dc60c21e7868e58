"""CPU check of the one-byte-slot query walks that the lookup kernels run.

The byte-lane walk (sqf_query_b1 in gpuquotientfilters_gb300/csrc/sqf_lookup.cuh)
and the bit-plane mirror (mirror_record / mirror_query in sqf_mirror.cuh) are
host+device code; here they are compiled for the host by nvcc and run over
tables made by the oracle, and their results must equal the oracle's lookups
(the reference's hashAndLookUp, quotientFilter.cu:320-357) on every query, at
fills up to 1.0, with and without duplicate fingerprints, after deletes, near
the table's ends, and where the pending-run count saturates."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "drivers", "swar_query_host.cu")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = shutil.which("nvcc")
    if not nvcc:
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("swq") / "swar_query_host")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe, SRC],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def run_driver(exe, tmp_path, t, q, r, fps, mirror=False):
    tf, ff, of = tmp_path / "t.bin", tmp_path / "f.bin", tmp_path / "o.bin"
    t.tofile(tf)
    np.ascontiguousarray(fps, np.uint32).tofile(ff)
    env = dict(os.environ)
    if mirror:
        env["SWAR_MIRROR"] = "1"
    p = subprocess.run([exe, str(tf), str(ff), str(q), str(r), str(O.sqf_num_slots(q)), str(of)],
                       capture_output=True, text=True, env=env)
    assert p.returncode == 0, p.stderr
    return np.fromfile(of, np.uint32)


@pytest.mark.parametrize("q,fill,nodup", [(12, 0.5, True), (14, 0.8, True), (14, 0.95, True),
                                          (13, 0.9, False), (10, 1.0, True)])
def test_walk_matches_oracle(driver, tmp_path, q, fill, nodup):
    r = 5
    n = int((1 << q) * fill)
    keys = O.mt_keys(11 + q, n)
    if not nodup:
        keys = np.concatenate([keys, keys[: n // 4]])  # repeated fingerprints
    t = O.sqf_new(q, r)
    O.sqf_bulk_build(t, q, r, keys, nodup)
    look = np.concatenate([keys, O.mt_keys(1000 + q, n)])
    want = O.sqf_lookup(t, q, r, look)
    got = run_driver(driver, tmp_path, t, q, r, O.aphash(look, q, r))
    assert np.array_equal(got, want)
    # the bit-plane mirror's two-record window, the walk where it is undecided
    got = run_driver(driver, tmp_path, t, q, r, O.aphash(look, q, r), mirror=True)
    assert np.array_equal(got, want)
    # every fingerprint of the quotient space near the table's start and end
    allq = np.arange(1 << (q + r), dtype=np.uint32)
    edge = np.concatenate([allq[: 64 << r], allq[-(64 << r):]])
    want_edge = _oracle_fp_lookup(t, q, r, edge)
    assert np.array_equal(run_driver(driver, tmp_path, t, q, r, edge), want_edge)
    assert np.array_equal(run_driver(driver, tmp_path, t, q, r, edge, mirror=True), want_edge)


def _oracle_fp_lookup(t, q, r, fps):
    """Oracle lookups by fingerprint: find keys hashing to each fp is not
    possible, so restate the reference walk on the slot bytes directly."""
    ns = O.sqf_num_slots(q)
    s = t[:ns].astype(np.int64)
    out = np.empty(len(fps), np.uint32)
    for i, fp in enumerate(fps.tolist()):
        fq, fr = (fp >> r) & ((1 << q) - 1), fp & ((1 << r) - 1)
        out[i] = 0xFFFFFFFF
        if not (s[fq] >> 2) & 1:
            continue
        b = fq
        while b > 0 and (s[b] & 1):
            b -= 1
        p = b
        while b != fq:  # findRunStartGPU, quotientFilter.cu:172-196
            p += 1
            while p < ns and (s[p] >> 1) & 1:
                p += 1
            b += 1
            while b < ns and not (s[b] >> 2) & 1:
                b += 1
        while True:
            rem = s[p] >> 3
            if rem == fr:
                out[i] = p
                break
            if rem > fr:
                break
            p += 1
            if p >= ns or not (s[p] >> 1) & 1:
                break
    return out


def test_walk_after_deletes(driver, tmp_path):
    q, r = 13, 5
    n = int((1 << q) * 0.85)
    keys = O.mt_keys(77, n)
    t = O.sqf_new(q, r)
    O.sqf_bulk_build(t, q, r, keys, True)
    O.sqf_delete(t, q, r, keys[: n // 3])
    look = np.concatenate([keys, O.mt_keys(78, n // 2)])
    want = O.sqf_lookup(t, q, r, look)
    assert np.array_equal(run_driver(driver, tmp_path, t, q, r, O.aphash(look, q, r)), want)
    assert np.array_equal(run_driver(driver, tmp_path, t, q, r, O.aphash(look, q, r), mirror=True), want)


def test_mirror_saturated_pending_count(driver, tmp_path):
    """A cluster with more than 254 runs pending: the mirror records carry
    P = 255 there and those queries fall back to the full walk."""
    q, r = 12, 5
    fps = [(5 << r) | (i * 32 // 300) for i in range(300)]      # one run of 300 at quotient 5
    fps += [(qq << r) | 7 for qq in range(6, 306)]             # 300 runs pushed behind it
    fps += [(qq << r) | 3 for qq in range(1000, 1040, 3)]      # a separate sparse region
    fps = np.array(sorted(fps), np.uint32)
    t = O.sqf_new(q, r)
    assert O.sqf_layout_sorted(t, q, r, fps) == 0
    ns = O.sqf_num_slots(q)
    probe = np.concatenate([fps, np.arange(0, 1 << (q + r), 7, dtype=np.uint32)])
    want = _oracle_fp_lookup(t, q, r, probe)
    assert (want[: fps.size] != 0xFFFFFFFF).all()
    assert np.array_equal(run_driver(driver, tmp_path, t, q, r, probe, mirror=True), want)
    assert ns > 700


@pytest.mark.parametrize("q,fill,nodup", [(11, 0.8, True), (13, 0.95, False), (10, 1.0, True)])
def test_mirror_build_transposition(driver, tmp_path, q, fill, nodup):
    """The mirror build kernel's per-thread transposition (8x8 bit transposes,
    a 4x4 byte transpose, funnel shifts into 31-slot groups), compiled for the
    host, gives every group record exactly as mirror_record does, including
    the groups past the table's end."""
    r = 5
    n = int((1 << q) * fill)
    keys = O.mt_keys(300 + q, n)
    if not nodup:
        keys = np.concatenate([keys, keys[: n // 5]])
    t = O.sqf_new(q, r)
    O.sqf_bulk_build(t, q, r, keys, nodup)
    tf, ff, of = tmp_path / "t.bin", tmp_path / "f.bin", tmp_path / "o.bin"
    t.tofile(tf)
    np.zeros(1, np.uint32).tofile(ff)
    env = dict(os.environ, SWAR_MIRROR_GROUPS="1")
    p = subprocess.run([driver, str(tf), str(ff), str(q), str(r), str(O.sqf_num_slots(q)), str(of)],
                       capture_output=True, text=True, env=env)
    assert p.returncode == 0, p.stderr
    assert "differing 0" in p.stderr
