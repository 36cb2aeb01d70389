"""The bidirectional engine's rules, restated sequentially in Python and
checked against Dijkstra (no GPU): buckets of width delta on g with one
threshold per direction, advanced only while that direction's open set is
not much larger than the other's, entries popped in random order (standing
in for the warps' interleaving), the meeting offer g(u) + w + g_other(v) kept with the arc's
forward-side tail, relaxations and far entries at or above mu dropped, the
stop rule (smallest open forward key + smallest open reverse key >= mu, or
an empty direction), and the path rebuilt from the meeting tail.  This is
the logic of ddp_gb300/csrc/engine_bidir.cuh; the GPU tests check the
kernel itself against the oracle."""
import heapq
import random

import numpy as np
import pytest

INF = 2147483647


def _csr(n, u, v, w):
    order = np.lexsort((v, u))
    u, v, w = u[order], v[order], w[order]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, u + 1, 1)
    return np.cumsum(off), v.astype(np.int64), w.astype(np.int64)


def _dijkstra(n, off, col, w, s, t):
    d = [INF] * n
    d[s] = 0
    h = [(0, s)]
    while h:
        g, u = heapq.heappop(h)
        if g > d[u]:
            continue
        if u == t:
            return g
        for k in range(off[u], off[u + 1]):
            ng = g + int(w[k])
            if ng < d[col[k]]:
                d[col[k]] = ng
                heapq.heappush(h, (ng, int(col[k])))
    return INF


def bidir(n, fw, rv, s, t, delta, rng, ring_cap=1 << 30, pot=None):
    """fw, rv = (off, col, w) of the graph and of its reverse.  A split
    moves at most ring_cap entries to the bucket; the rest stay in far.
    pot = (pt, ps): consistent lower bounds of d(v, t) and d(s, v); keys are
    then 2g + pt - ps (forward) and 2g + ps - pt (reverse), the stop rule
    a + b >= 2 mu, and a label g is pruned when g + the other side's bound
    reaches mu.  Without pot, keys are g."""
    if s == t:
        return 0, [s]
    if pot is None:
        def key(g, v, dr):
            return g
        bound = lambda m: m
        other = lambda v, dr: 0
        dk = delta
    else:
        pt, ps = pot

        def key(g, v, dr):
            return 2 * g + (int(ps[v]) - int(pt[v]) if dr else int(pt[v]) - int(ps[v]))
        bound = lambda m: 2 * m
        other = lambda v, dr: int(ps[v]) if dr else int(pt[v])
        dk = 2 * delta
    lab = [[INF] * n, [INF] * n]
    par = [[-1] * n, [-1] * n]
    lab[0][s] = 0
    lab[1][t] = 0
    mu, mux = INF, -1
    near = [(s, 0, key(0, s, 0)), (t, 1, key(0, t, 1))]
    far = []
    Td = [key(0, s, 0) + dk, key(0, t, 1) + dk]   # per-direction thresholds of the current bucket
    lo = [0, 0]           # jump target of a direction whose advance moved nothing
    expand = True
    while True:
        if expand:
            while near:
                u, dr, kk = near.pop(rng.randrange(len(near)))
                g = lab[dr][u]
                if g >= INF or key(g, u, dr) != kk or kk >= bound(mu):
                    continue
                off, col, w = fw if dr == 0 else rv
                for k in range(off[u], off[u + 1]):
                    v, ng = int(col[k]), g + int(w[k])
                    if ng >= min(mu, INF) or ng + other(v, dr) >= mu:
                        continue
                    go = lab[1 - dr][v]
                    if go < INF and ng + go < mu:
                        mu, mux = ng + go, (u if dr == 0 else v)
                    if ng < lab[dr][v]:
                        lab[dr][v] = ng
                        par[dr][v] = u
                        nk = key(ng, v, dr)
                        (near if nk < Td[dr] else far).append((v, dr, nk))
        # balance: advance a direction while its open set is not much larger
        opn = [sum(1 for e in far if e[1] == d) for d in (0, 1)]
        adv = [opn[0] <= 2 * opn[1] + 64, opn[1] <= 2 * opn[0] + 64]
        Ts = [max(Td[d], lo[d]) + dk if adv[d] else Td[d] for d in (0, 1)]
        moved, kept, mins, nmoved = [], [], [INF, INF], [0, 0]
        for (v, dr, g) in far:   # g: the entry's key
            if g >= bound(mu):
                continue
            if g < Ts[dr] and len(moved) < ring_cap:
                moved.append((v, dr, g))
                nmoved[dr] += 1
            else:
                kept.append((v, dr, g))
            mins[dr] = min(mins[dr], g)
        far = kept
        a, b = mins
        if a == INF or b == INF or a + b >= bound(mu):
            break
        lo = [mins[d] if adv[d] and nmoved[d] == 0 else 0 for d in (0, 1)]
        Td = Ts
        near = moved
        expand = bool(moved)
    if mu >= INF:
        return INF, []
    x = mux
    off, col, w = fw
    y = next(int(col[k]) for k in range(off[x], off[x + 1])
             if lab[1][col[k]] < INF and lab[0][x] + int(w[k]) + lab[1][col[k]] == mu)
    left = [x]
    while left[-1] != s:
        left.append(par[0][left[-1]])
    right = [y]
    while right[-1] != t:
        right.append(par[1][right[-1]])
    return mu, left[::-1] + right


def _path_weight(fw, p):
    off, col, w = fw
    tot = 0
    for a, b in zip(p[:-1], p[1:]):
        ws = [int(w[k]) for k in range(off[a], off[a + 1]) if col[k] == b]
        assert ws, (a, b)
        tot += min(ws)
    return tot


@pytest.mark.parametrize("seed,n,e,wmax,zero", [(1, 300, 1200, 100, False), (2, 500, 900, 5, True),
                                                (3, 2000, 16000, 100, False), (4, 800, 900, 3, True)])
@pytest.mark.parametrize("delta,ring_cap", [(1, 1 << 30), (7, 1 << 30), (60, 1 << 30), (60, 5)])
def test_bidir_rules_match_dijkstra(seed, n, e, wmax, zero, delta, ring_cap):
    r = np.random.default_rng(seed)
    u = r.integers(0, n, e)
    v = r.integers(0, n, e)
    keep = u != v
    u, v = u[keep], v[keep]
    w = r.integers(0 if zero else 1, wmax + 1, len(u))
    fw = _csr(n, u, v, w)
    rv = _csr(n, v, u, w)
    rng = random.Random(seed * 100 + delta)
    for q in range(40):
        s, t = int(r.integers(0, n)), int(r.integers(0, n))
        want = _dijkstra(n, *fw, s, t)
        got, path = bidir(n, fw, rv, s, t, delta, rng, ring_cap)
        assert got == want, (s, t)
        if want < INF:
            assert path[0] == s and path[-1] == t
            assert _path_weight(fw, path) == want


def test_bidir_rules_grid():
    # 4-connected 30 x 30 grid with walls, unit weights (long, narrow searches)
    R = C = 30
    r = np.random.default_rng(9)
    wall = r.random(R * C) < 0.25
    us, vs = [], []
    for i in range(R):
        for j in range(C):
            a = i * C + j
            if wall[a]:
                continue
            for di, dj in ((1, 0), (-1, 0), (0, 1), (0, -1)):
                ii, jj = i + di, j + dj
                if 0 <= ii < R and 0 <= jj < C and not wall[ii * C + jj]:
                    us.append(a)
                    vs.append(ii * C + jj)
    u, v = np.array(us), np.array(vs)
    w = np.ones(len(u), np.int64)
    fw = _csr(R * C, u, v, w)
    rv = _csr(R * C, v, u, w)
    rng = random.Random(3)
    open_cells = np.flatnonzero(~wall)
    for q in range(60):
        s, t = (int(x) for x in r.choice(open_cells, 2))
        want = _dijkstra(R * C, *fw, s, t)
        got, path = bidir(R * C, fw, rv, s, t, 2, rng)
        assert got == want
        if want < INF:
            assert _path_weight(fw, path) == want


@pytest.mark.parametrize("seed,delta", [(11, 3), (12, 40), (13, 400)])
def test_bidir_rules_euclidean_potentials(seed, delta):
    """Points in a square joined to near neighbours, w = ceil(length); the
    potentials floor(rho |v - t|) and floor(rho |s - v|) with rho <= w /
    length on every arc are consistent, so the keyed rules stay exact."""
    r = np.random.default_rng(seed)
    n = 700
    xy = r.integers(0, 10000, (n, 2))
    us, vs, ws = [], [], []
    for a in range(n):
        d2 = ((xy - xy[a]) ** 2).sum(1)
        for b in np.argsort(d2)[1:6]:
            ln = float(np.sqrt(d2[b]))
            us += [a, b]
            vs += [b, a]
            ws += [int(np.ceil(ln)) + int(r.integers(0, 50))] * 2
    u, v, w = np.array(us), np.array(vs), np.array(ws, np.int64)
    fw = _csr(n, u, v, w)
    rv = _csr(n, v, u, w)
    ln = np.sqrt(((xy[u] - xy[v]) ** 2).sum(1))
    rho = float((w / np.maximum(ln, 1e-9)).min()) * (1 - 1e-9)
    rng = random.Random(seed)
    for q in range(40):
        s, t = (int(x) for x in r.integers(0, n, 2))
        pt = np.floor(rho * np.sqrt(((xy - xy[t]) ** 2).sum(1))).astype(np.int64)
        ps = np.floor(rho * np.sqrt(((xy - xy[s]) ** 2).sum(1))).astype(np.int64)
        want = _dijkstra(n, *fw, s, t)
        got, path = bidir(n, fw, rv, s, t, delta, rng, pot=(pt, ps))
        assert got == want, (s, t)
        if want < INF:
            assert path[0] == s and path[-1] == t and _path_weight(fw, path) == want
