"""Deletes are cluster-local, restated in Python over whole tables and
checked against the oracle (no GPU).

A cluster is a maximal stretch of non-empty slots; its first slot holds an
unshifted run start, so the lookup's pending-run count is 0 there and the
cluster can be decoded on its own: its run starts, in slot order, belong to
its occupied quotients in order.  Deleting elements only shrinks clusters.
So a batch of deletes can be applied cluster by cluster: drop the deleted
elements of each touched cluster, lay the rest out canonically from the
cluster's first slot (pos = max(quotient, previous pos + 1)), rewrite the
cluster's old span, and leave every other slot as it is.  The result must
be the oracle's delete (the reference's superclusterDeletes semantics: one
stored copy per occurrence in the batch, keys not stored delete nothing),
byte for byte, with no write outside a touched cluster's old span."""
import numpy as np
import pytest

import oracle as O


def clusters(s):
    """(first slot, end slot) of every cluster of slot array s."""
    ne = (s & 7) != 0
    out, i, n = [], 0, s.size
    while i < n:
        if ne[i]:
            j = i
            while j < n and ne[j]:
                j += 1
            out.append((i, j))
            i = j
        else:
            i += 1
    return out


def decode(s, cs, ce):
    """Elements of the cluster [cs, ce) in slot order: [quotient, remainder]."""
    occ = [x for x in range(cs, ce) if (s[x] >> 2) & 1]
    els, k = [], -1
    for x in range(cs, ce):
        if not (s[x] >> 1) & 1:  # a run start
            k += 1
        els.append([occ[k], int(s[x]) >> 3])
    assert k == len(occ) - 1, "every occupied quotient of a cluster has one run in it"
    return els


def layout(els, cs, ce):
    """Slot bytes of the span [cs, ce) holding els canonically from cs."""
    out = np.zeros(ce - cs, np.int64)
    prev, last_q = cs - 1, -1
    for q, rem in els:
        pos = max(q, prev + 1)
        assert pos < ce, "a delete only shrinks a cluster"
        out[pos - cs] |= (rem << 3) | (2 if q == last_q else 0) | (1 if pos != q else 0)
        prev, last_q = pos, q
    for q, _ in els:
        out[q - cs] |= 4
    return out


def cluster_delete(t, q, r, fps):
    ns = O.sqf_num_slots(q)
    s = t[:ns].astype(np.int64)
    spans = clusters(s)
    starts = [a for a, _ in spans]
    touched = {}
    for fp in (int(x) for x in fps):
        fq, fr = fp >> r, fp & ((1 << r) - 1)
        if not (s[fq] >> 2) & 1:
            continue  # quotient not occupied: nothing stored
        k = int(np.searchsorted(starts, fq, side="right")) - 1
        cs, ce = spans[k]
        els = touched.setdefault(cs, (ce, decode(s, cs, ce)))[1]
        for i, (eq, er) in enumerate(els):
            if eq == fq and er == fr:
                del els[i]  # one stored copy per occurrence in the batch
                break
    out = s.copy()
    for cs, (ce, els) in touched.items():
        out[cs:ce] = layout(els, cs, ce)
    res = t.copy()
    res[:ns] = out.astype(np.uint8)
    return res, touched


@pytest.mark.parametrize("q,fill,nodup,frac", [(12, 0.8, True, 0.05), (13, 0.9, True, 0.2), (12, 0.8, False, 0.1),
                                               (11, 1.0, True, 0.5), (10, 0.6, False, 1.0)])
def test_cluster_local_delete_equals_oracle(q, fill, nodup, frac):
    r = 5
    n = int((1 << q) * fill)
    keys = O.mt_keys(500 + q, n)
    if not nodup:
        keys = np.concatenate([keys, keys[: n // 4]])  # repeated fingerprints
    t = O.sqf_new(q, r)
    assert O.sqf_bulk_build(t, q, r, keys, nodup) == 0
    m = int(n * frac)
    # present keys (some twice), and keys never stored
    dels = np.concatenate([keys[:m], keys[: m // 10], O.mt_keys(900 + q, m // 4, skip=n)]).astype(np.uint32)
    want = t.copy()
    O.sqf_delete(want, q, r, dels)
    got, touched = cluster_delete(t, q, r, O.aphash(dels, q, r))
    assert np.array_equal(got, want)
    # the untouched clusters keep their bytes; the touched ones are a minority at small batches
    ns = O.sqf_num_slots(q)
    if frac <= 0.05:
        assert sum(ce - cs for cs, (ce, _) in touched.items()) < 0.5 * ns
