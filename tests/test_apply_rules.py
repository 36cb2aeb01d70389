"""The device batch application's rules (k_apply in ddp_gb300/csrc/dynamic.cu),
restated in Python and checked against the oracle's merge (no GPU).

The graph sits in the dynamic layout: rows with [begin, end) and a capacity
inside one arc array, dead arcs marked -1.  Ops are grouped by tail row (and
inserts also by head row); each group runs in batch order on its leader, the
leaders in any order (shuffled here).  Deletes and weight changes act on the
first live u->v arc and on the first live reverse arc with the same tail and
weight; an arc hit more than once is classified once from its pre-batch and
final weight; inserts are appended after all deletes, a row that outgrows
its capacity first moves to the array's tail (capacity doubled, at least 4,
until the inserts fit).  A first pass refuses the whole batch when the moves
do not fit.  After each batch the compacted rows equal the oracle's merged
CSR (DA_dyn_cpu.cu removeDelEdges + mergeDiff semantics), every slot index
stays inside the arrays, and the repair records match the arcs' net change.
"""
import random

import numpy as np
import pytest

UPD_INS, UPD_TREE, UPD_LIGHTER = 1, 2, 3


class Layout:
    """Rows with slack (capacity = used + max(2, used / 4)) and a reserve."""

    def __init__(self, n, off, col, w, reserve):
        self.n = n
        self.beg, self.end, self.cap = [0] * n, [0] * n, [0] * n
        arcs = []
        for u in range(n):
            row = [(int(col[j]), int(w[j])) for j in range(off[u], off[u + 1])]
            c = len(row) + max(2, len(row) // 4)
            self.beg[u] = len(arcs)
            self.end[u] = len(arcs) + len(row)
            self.cap[u] = c
            arcs += row + [(-1, 0)] * (c - len(row))
        self.tail = len(arcs)
        self.arc = arcs + [(-1, 0)] * reserve

    def compact(self):
        off, col, w = [0], [], []
        for u in range(self.n):
            for j in range(self.beg[u], self.end[u]):
                if self.arc[j][0] >= 0:
                    col.append(self.arc[j][0])
                    w.append(self.arc[j][1])
            off.append(len(col))
        return np.array(off, np.int64), np.array(col, np.int64), np.array(w, np.int64)


def grown_cap(used, cap, add):
    if used + add <= cap:
        return cap
    c = max(4, 2 * cap)
    while c < used + add:
        c *= 2
    return c


def apply_batch(F, R, ops, rng):
    """F, R: forward and reverse layouts; ops: [(flag, u, v, w)].  Returns
    (applied, records)."""
    n = F.n
    valid = [i for i, (f, u, v, w) in enumerate(ops) if 0 <= f <= 2 and 0 <= u < n and 0 <= v < n]
    ka = sorted(valid, key=lambda i: (ops[i][1], i))
    kb = sorted((i for i in valid if ops[i][0] == 1), key=lambda i: (ops[i][2], i))

    def groups(k, col):
        g = {}
        for i in k:
            g.setdefault(ops[i][col], []).append(i)
        return g

    ga, gb = groups(ka, 1), groups(kb, 2)
    # room
    need = [0, 0]
    for side, (L, grp) in enumerate(((F, ga), (R, gb))):
        for r, items in grp.items():
            add = sum(ops[i][0] == 1 for i in items)
            c = grown_cap(L.end[r] - L.beg[r], L.cap[r], add)
            if c > L.cap[r]:
                need[side] += c
    if F.tail + need[0] > len(F.arc) or R.tail + need[1] > len(R.arc):
        return False, []
    recs = []
    hit, w0 = {}, {}
    leaders = list(ga.items())
    rng.shuffle(leaders)
    for a, items in leaders:
        for i in items:
            f, _, b, w = ops[i]
            if f == 1:
                continue
            jf = next((j for j in range(F.beg[a], F.end[a]) if F.arc[j][0] == b), -1)
            if jf < 0:
                continue
            wold = F.arc[jf][1]
            hit[i], w0[i] = jf, wold
            jr = next((j for j in range(R.beg[b], R.end[b]) if R.arc[j] == (a, wold)), -1)
            if f == 0:
                F.arc[jf] = (-1, F.arc[jf][1])
                if jr >= 0:
                    R.arc[jr] = (-1, R.arc[jr][1])
            else:
                F.arc[jf] = (b, w)
                if jr >= 0:
                    R.arc[jr] = (a, w)
        seen = set()
        for i in items:
            if i not in hit or hit[i] in seen:
                continue
            seen.add(hit[i])
            fin = F.arc[hit[i]]
            if fin[0] < 0 or fin[1] > w0[i]:
                recs.append((UPD_TREE, a, ops[i][2], 0))
            elif fin[1] < w0[i]:
                recs.append((UPD_LIGHTER, a, ops[i][2], fin[1]))
    jobs = [(0, r, it) for r, it in ga.items()] + [(1, r, it) for r, it in gb.items()]
    rng.shuffle(jobs)
    for side, r, items in jobs:
        L = R if side else F
        add = sum(ops[i][0] == 1 for i in items)
        if not add:
            continue
        c = grown_cap(L.end[r] - L.beg[r], L.cap[r], add)
        if c > L.cap[r]:
            base = L.tail
            L.tail += c
            assert L.tail <= len(L.arc)
            used = L.end[r] - L.beg[r]
            L.arc[base:base + used] = L.arc[L.beg[r]:L.end[r]]
            L.beg[r], L.end[r], L.cap[r] = base, base + used, c
        e = L.end[r]
        for i in items:
            f, u, v, w = ops[i]
            if f != 1:
                continue
            assert e < L.beg[r] + L.cap[r]
            L.arc[e] = (u, w) if side else (v, w)
            e += 1
            if not side:
                recs.append((UPD_INS, u, v, w))
        L.end[r] = e
    return True, recs


def _graph(rng, n, e, wmax, par):
    u = rng.integers(0, n, e)
    v = rng.integers(0, n, e)
    if par:  # parallel arcs, some with equal weights
        u = np.concatenate([u, u[: e // 5]])
        v = np.concatenate([v, v[: e // 5]])
    w = rng.integers(1, wmax + 1, len(u))
    if par:
        w[e: e + e // 10] = w[: e // 10]
    order = np.lexsort((v, u))
    u, v, w = u[order], v[order], w[order]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, u + 1, 1)
    return np.cumsum(off), v, w


def _reverse(n, off, col, w):
    src = np.repeat(np.arange(n), np.diff(off))
    order = np.argsort(col, kind="stable")
    roff = np.zeros(n + 1, np.int64)
    np.add.at(roff, col + 1, 1)
    return np.cumsum(roff), src[order], w[order]


@pytest.mark.parametrize("seed,par,reserve", [(1, False, 64), (2, True, 64), (3, True, 4096), (4, False, 8)])
def test_apply_rules_match_oracle_merge(oracle, seed, par, reserve):
    rng = np.random.default_rng(seed)
    prng = random.Random(seed)
    n, e = 300, 900
    off, col, w = _graph(rng, n, e, 50, par)
    F = Layout(n, off, col, w, reserve)
    roff, rcol, rw = _reverse(n, off, col, w)
    R = Layout(n, roff, rcol, rw, reserve)
    cur = (off, col, w)
    refused = 0
    for b in range(30):
        ops = []
        k = int(rng.integers(1, 120))
        co, cc, cw = cur
        for _ in range(k):
            f = int(rng.integers(0, 3))
            if f != 1 and len(cc) and rng.random() < 0.8:  # hit an existing arc
                j = int(rng.integers(0, len(cc)))
                uu = int(np.searchsorted(co, j, side="right") - 1)
                vv = int(cc[j])
            else:
                uu, vv = int(rng.integers(0, n)), int(rng.integers(0, n))
            if f == 1 and rng.random() < 0.3:
                uu = int(rng.integers(0, 5))  # a few hub rows outgrow their capacity
            ops.append((f, uu, vv, int(rng.integers(1, 60))))
        if rng.random() < 0.3 and ops:  # the same arc twice (lighter, then heavier)
            f0, uu, vv, _ = ops[0]
            ops += [(2, uu, vv, 1), (2, uu, vv, 500)]
        ops.append((1, -1, 3, 5))   # out of range: ignored
        ops.append((7, 1, 2, 5))    # unknown flag: ignored
        before = cur
        ok, recs = apply_batch(F, R, ops, prng)
        if not ok:
            refused += 1
            # the host path lays the arrays out again with a larger reserve
            fo, fc, fw = F.compact()
            F = Layout(n, fo, fc, fw, 4096)
            ro, rc, rwt = R.compact()
            R = Layout(n, ro, rc, rwt, 4096)
            ok, recs = apply_batch(F, R, ops, prng)
            assert ok
        fl = np.array([o[0] for o in ops], np.int32)
        uu = np.array([o[1] for o in ops], np.int32)
        vv = np.array([o[2] for o in ops], np.int32)
        ww = np.array([o[3] for o in ops], np.uint32)
        noff, ncol, nw, _ = oracle.apply_batch(n, before[0][:-1].astype(np.int32), before[1].astype(np.int32),
                                               before[2].astype(np.uint32), fl, uu, vv, ww)
        got = F.compact()
        assert np.array_equal(got[0][:-1], noff) and np.array_equal(got[1], ncol) and np.array_equal(got[2], nw), b
        # the reverse rows hold the same arcs (as a multiset per head)
        rr = R.compact()
        want_r = _reverse(n, np.append(noff, len(ncol)), ncol, nw)
        for x in range(n):
            a = sorted(zip(rr[1][rr[0][x]:rr[0][x + 1]].tolist(), rr[2][rr[0][x]:rr[0][x + 1]].tolist()))
            bb = sorted(zip(want_r[1][want_r[0][x]:want_r[0][x + 1]].tolist(),
                            want_r[2][want_r[0][x]:want_r[0][x + 1]].tolist()))
            assert a == bb, (b, x)
        # repair records: one per insert, one per arc whose weight changed or that died
        assert sum(r[0] == UPD_INS for r in recs) == int(((fl == 1) & (uu >= 0) & (uu < n) & (vv >= 0)
                                                            & (vv < n)).sum())
        for kind, a, bb, wt in recs:
            if kind == UPD_LIGHTER:
                assert wt in nw[noff[a]:(noff[a + 1] if a + 1 < n else len(ncol))][
                    ncol[noff[a]:(noff[a + 1] if a + 1 < n else len(ncol))] == bb]
        cur = (np.append(noff, len(ncol)).astype(np.int64), ncol.astype(np.int64), nw.astype(np.int64))
    if reserve == 8:
        assert refused > 0  # the room check ran
