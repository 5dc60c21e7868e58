"""The in-place insert's merge rule, restated in Python over a whole table
and checked against the oracle (no GPU).

k_bucket_insert_merge places the table's stored elements and the new
fingerprints without decoding runs: walking the old slots in order with c =
the first free slot, a stored element at old slot s goes to max(s, c) (an
insert only moves elements right, so its home quotient is never needed) and a
new fingerprint of quotient q goes to max(q, c), in front of the old slot it
is inserted before.  This test restates that rule for one bucket spanning the
table and compares the result, byte for byte, with the oracle's sequential
insert (the reference's insertItemGPU semantics: a stored fingerprint is not
stored again, a repeated one goes in once)."""
import numpy as np
import pytest

import oracle as O


def merge_insert(t, q, r, fps):
    ns = O.sqf_num_slots(q)
    old = t[:ns].astype(np.int64)
    occ = (old >> 2) & 1
    rs = np.flatnonzero((old & 7 != 0) & ((old >> 1) & 1 == 0))  # run starts, in quotient order
    occq = np.flatnonzero(occ)                                     # occupied quotients
    run_of_q = {int(x): int(p) for x, p in zip(occq, rs)}          # one run per occupied quotient
    items = []                                                     # (insertion point, fp, head)
    for fp in sorted(set(int(x) for x in fps)):
        fq, fr = fp >> r, fp & ((1 << r) - 1)
        if fq in run_of_q:
            p = t_ = run_of_q[fq]
            while True:
                rem = int(old[t_]) >> 3
                if rem >= fr:
                    break
                t_ += 1
                if not (old[t_] & 7 and old[t_] & 2):
                    break
            if t_ < ns and old[t_] & 7 and (t_ == p or old[t_] & 2) and int(old[t_]) >> 3 == fr:
                continue  # already stored
            items.append((t_, fp, t_ == p))
        else:
            later = [p for x, p in run_of_q.items() if x > fq]
            ip = min(later) if later else int(np.flatnonzero(old & 7).max()) + 1 if (old & 7).any() else 0
            items.append((ip, fp, True))
    items.sort()
    # the first kept fingerprint of a quotient at the front heads its run
    seen = set()
    fixed = []
    for ip, fp, head in items:
        fq = fp >> r
        fixed.append((ip, fp, head and fq not in seen))
        seen.add(fq)
    displaced = {ip for ip, fp, head in fixed if head and (fp >> r) in run_of_q}
    out = np.zeros(ns, np.int64)
    newocc = occ.copy()
    c, k = 0, 0
    for s in range(ns + 1):
        while k < len(fixed) and fixed[k][0] == s:
            _, fp, head = fixed[k]
            fq, fr = fp >> r, fp & ((1 << r) - 1)
            pos = max(fq, c)
            out[pos] = (fr << 3) | (0 if head else 2) | (1 if pos != fq else 0)
            newocc[fq] = 1
            c = pos + 1
            k += 1
        if s < ns and old[s] & 7:
            e = int(old[s]) | (2 if s in displaced else 0)
            pos = max(s, c)
            out[pos] = (e & ~4) | (1 if pos != s else 0)
            c = pos + 1
    out |= newocc << 2
    res = t.copy()
    res[:ns] = out.astype(np.uint8)
    return res


@pytest.mark.parametrize("q,fill,nins,seed", [(10, 0.5, 120, 1), (11, 0.8, 300, 2), (12, 0.9, 200, 3),
                                              (10, 0.0, 400, 4)])
def test_merge_rule_matches_oracle_insert(q, fill, nins, seed):
    r = 5
    n = int(fill * (1 << q))
    keys = O.mt_keys(seed, n)
    t = O.sqf_new(q, r)
    if n:
        O.sqf_bulk_build(t, q, r, keys, True)
    new = np.concatenate([O.mt_keys(seed + 50, nins), keys[: min(n, 20)], O.mt_keys(seed + 50, 10)])
    want = t.copy()
    O.sqf_insert(want, q, r, new)
    got = merge_insert(t, q, r, O.aphash(new, q, r))
    assert np.array_equal(got, want)
