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


def bidir(n, fw, rv, s, t, delta, rng, ring_cap=1 << 30):
    """fw, rv = (off, col, w) of the graph and of its reverse.  A split
    moves at most ring_cap entries to the bucket; the rest stay in far."""
    if s == t:
        return 0, [s]
    lab = [[INF] * n, [INF] * n]
    par = [[-1] * n, [-1] * n]
    lab[0][s] = 0
    lab[1][t] = 0
    mu, mux = INF, -1
    near = [(s, 0, 0), (t, 1, 0)]
    far = []
    Td = [delta, delta]   # per-direction thresholds of the current bucket
    lo = [0, 0]           # jump target of a direction whose advance moved nothing
    expand = True
    while True:
        if expand:
            while near:
                u, dr, g = near.pop(rng.randrange(len(near)))
                if lab[dr][u] != g or g >= mu:
                    continue
                off, col, w = fw if dr == 0 else rv
                for k in range(off[u], off[u + 1]):
                    v, ng = int(col[k]), g + int(w[k])
                    if ng >= min(mu, INF):
                        continue
                    go = lab[1 - dr][v]
                    if go < INF and ng + go < mu:
                        mu, mux = ng + go, (u if dr == 0 else v)
                    if ng < lab[dr][v]:
                        lab[dr][v] = ng
                        par[dr][v] = u
                        (near if ng < Td[dr] else far).append((v, dr, ng))
        # balance: advance a direction while its open set is not much larger
        opn = [sum(1 for e in far if e[1] == d) for d in (0, 1)]
        adv = [opn[0] <= 2 * opn[1] + 64, opn[1] <= 2 * opn[0] + 64]
        Ts = [max(Td[d], lo[d]) + delta if adv[d] else Td[d] for d in (0, 1)]
        moved, kept, mins, nmoved = [], [], [INF, INF], [0, 0]
        for (v, dr, g) in far:
            if g >= mu:
                continue
            if g < Ts[dr] and len(moved) < ring_cap:
                moved.append((v, dr, g))
                nmoved[dr] += 1
            else:
                kept.append((v, dr, g))
            mins[dr] = min(mins[dr], g)
        far = kept
        a, b = mins
        if a == INF or b == INF or a + b >= mu:
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
