"""The dynamic search's rules, restated sequentially in Python and checked
against Dijkstra after every update batch (no GPU).

A keep-mode threshold search (every generated node stays open, far entries
carry g and their f is re-derived at each split) runs once; then each batch
is applied and repaired the way k_dyn does it (ddp_gb300/csrc/dynamic.cu):
A. inserted arcs lower the hop heuristic, propagated over reverse arcs;
B. a deleted or heavier arc that is its head's parent arc invalidates the
   head's subtree; C. invalidated nodes are re-seeded from valid
   in-neighbours (reads first, then writes); D. inserted and lighter arcs
   relax their heads; E. the search resumes from the far pile.  The resumed
search has the cold tier of run_search (ddp_gb300/csrc/engine.cuh): its first
split sets live entries with g at or above the previous cost aside
unexamined, later splits scan the rest until min(f(t), threshold) passes
that bound, then one split takes the cold entries back; they rejoin the pile
when the search ends.  Entries are examined in random order (standing in for
the warps' interleaving).  The GPU tests check the kernels themselves against
the oracle."""
import heapq
import random

import numpy as np
import pytest

INF = 1 << 40


class Graph:
    def __init__(self, n):
        self.n = n
        self.rows = [[] for _ in range(n)]  # [v, w, alive]

    def arcs(self, u):
        return ((a[0], a[1]) for a in self.rows[u] if a[2])

    def rev(self):
        r = [[] for _ in range(self.n)]
        for u in range(self.n):
            for v, w in self.arcs(u):
                r[v].append((u, w))
        return r

    def wmin(self):
        return min((w for u in range(self.n) for _, w in self.arcs(u)), default=1)


def dijkstra(G, s, t):
    d = [INF] * G.n
    d[s] = 0
    h = [(0, s)]
    while h:
        g, u = heapq.heappop(h)
        if g > d[u]:
            continue
        if u == t:
            return g
        for v, w in G.arcs(u):
            if g + w < d[v]:
                d[v] = g + w
                heapq.heappush(h, (g + w, v))
    return INF


def bfs_hops(G, t):
    r = G.rev()
    hops = [INF] * G.n
    hops[t] = 0
    q = [t]
    for x in q:
        for p, _ in r[x]:
            if hops[p] == INF:
                hops[p] = hops[x] + 1
                q.append(p)
    return hops


class DynSearch:
    def __init__(self, G, s, t, delta, heur, cold, rng):
        self.G, self.s, self.t, self.delta, self.heur, self.use_cold, self.rng = G, s, t, delta, heur, cold, rng
        self.g = [INF] * G.n
        self.par = [-1] * G.n
        self.hops = bfs_hops(G, t) if heur else None
        self.far = []
        self.cost = INF
        self.search(resume=False)

    def h(self, v):
        if not self.heur:
            return 0
        return INF if self.hops[v] == INF else self.hops[v] * self.G.wmin()

    def search(self, resume):
        g, par, t = self.g, self.par, self.t
        cold, ncold_x = [], INF
        if resume and self.use_cold and self.cost < INF:
            ncold_x = self.cost
        cold_pass = ncold_x < INF
        if resume:
            near, T, Tsplit, splitting = [], 0, 0, True
        else:
            g[self.s], par[self.s] = 0, -1
            near, T, splitting = [(self.s, 0)], self.h(self.s) + self.delta, False
        far = self.far
        while True:
            ft = g[t] + self.h(t) if g[t] < INF else INF
            if not splitting:
                # drain the bucket: entries with f < T expand, others stay open
                while near:
                    u, gu = near.pop(self.rng.randrange(len(near)))
                    if g[u] != gu:
                        continue
                    for v, w in self.G.arcs(u):
                        ng = gu + w
                        if ng < g[v]:
                            g[v], par[v] = ng, u
                            f = ng + self.h(v)
                            (near if f < T else far).append((v, ng))
                splitting, Tsplit = True, T + self.delta
                continue
            # split: cold tier made on the first split of a resumed search
            merge = bool(cold) and min(ft, Tsplit) > ncold_x
            scan = far + (cold if merge else [])
            if merge:
                cold, ncold_x = [], INF
            self.rng.shuffle(scan)
            moved, kept, m = [], [], INF
            for v, gv in scan:
                if g[v] != gv:
                    continue  # stale
                if cold_pass and gv >= ncold_x:
                    cold.append((v, gv))  # f >= g >= the bound: h not read
                    continue
                f = gv + self.h(v)
                if f < ft and f < Tsplit:
                    moved.append((v, gv))
                elif f < INF:
                    kept.append((v, gv))
                    m = min(m, f)
            cold_pass = False
            far = kept
            mall = min(m, ncold_x) if cold else m
            if moved:
                near, T, splitting = moved, Tsplit, False
            elif (not far and not cold) or mall >= ft:
                break
            else:
                Tsplit = mall + self.delta
        self.far = far + cold  # the cold tier rejoins the pile
        self.cost = g[t] + self.h(t) if g[t] < INF else INF

    def update(self, batch):
        """batch: [(flag, u, v, w)], flag 1 insert, 0 delete, 2 set weight;
        the reference's semantics (deletes and weight changes first, on the
        first live u->v arc)."""
        G, g, par = self.G, self.g, self.par
        tree, lighter, ins = [], [], []
        for fl, u, v, w in batch:
            if fl == 1:
                continue
            a = next((a for a in G.rows[u] if a[2] and a[0] == v), None)
            if a is None:
                continue
            if fl == 0:
                a[2] = False
                tree.append((u, v))
            else:
                old, a[1] = a[1], w
                if w > old:
                    tree.append((u, v))
                elif w < old:
                    lighter.append((u, v, w))
        for fl, u, v, w in batch:
            if fl == 1:
                G.rows[u].append([v, w, True])
                ins.append((u, v, w))
        # A. hop repair over inserted arcs
        if self.heur:
            r = G.rev()
            q = []
            for u, v, _ in ins:
                if self.hops[v] < INF and self.hops[v] + 1 < self.hops[u]:
                    self.hops[u] = self.hops[v] + 1
                    q.append(u)
            for x in q:
                for p, _ in r[x]:
                    if self.hops[x] + 1 < self.hops[p]:
                        self.hops[p] = self.hops[x] + 1
                        q.append(p)
        # B. invalidate subtrees under removed / heavier tree arcs
        inv = []
        for u, v in tree:
            if g[v] < INF and par[v] == u:
                g[v], par[v] = INF, -1
                inv.append(v)
        for x in inv:
            for y, _ in G.arcs(x):
                if g[y] < INF and par[y] == x:
                    g[y], par[y] = INF, -1
                    inv.append(y)
        # C. re-seed from valid in-neighbours (reads first, then writes)
        r = G.rev()
        best = []
        for x in inv:
            c = min(((g[p] + w, p) for p, w in r[x] if g[p] < INF), default=(INF, -1))
            best.append(c)
        for x, (c, p) in zip(inv, best):
            if c < INF:
                g[x], par[x] = c, p
                self.far.append((x, c))
        # D. relax heads of inserted / lighter arcs
        for u, v, w in ins + lighter:
            if g[u] < INF and g[u] + w < g[v]:
                g[v], par[v] = g[u] + w, u
                self.far.append((v, g[v]))
        self.search(resume=True)


def _random_graph(n, deg, wmax, seed):
    rng = np.random.default_rng(seed)
    G = Graph(n)
    perm = rng.permutation(n)
    for a, b in zip(perm[:-1], perm[1:]):
        G.rows[int(a)].append([int(b), int(rng.integers(1, wmax + 1)), True])
    for _ in range(n * (deg - 1)):
        u, v = int(rng.integers(0, n)), int(rng.integers(0, n))
        if u != v:
            G.rows[u].append([v, int(rng.integers(1, wmax + 1)), True])
    return G, int(perm[0]), int(perm[-1])


def _path_weight(G, par, s, t):
    tot, v, steps = 0, t, 0
    while v != s:
        u = par[v]
        assert u >= 0 and steps <= G.n
        tot += min(w for x, w in G.arcs(u) if x == v)
        v, steps = u, steps + 1
    return tot


@pytest.mark.parametrize("heur", [False, True])
@pytest.mark.parametrize("cold", [False, True])
@pytest.mark.parametrize("delta", [1, 25, 400])
def test_dynamic_rules_match_dijkstra(heur, cold, delta):
    seed = 7 + 3 * delta + (11 if heur else 0)
    G, s, t = _random_graph(400, 4, 100, seed)
    rng = np.random.default_rng(seed + 1)
    D = DynSearch(G, s, t, delta, heur, cold, random.Random(seed))
    assert D.cost == dijkstra(G, s, t)
    for b in range(25):
        batch = []
        live = [(u, a[0]) for u in range(G.n) for a in G.rows[u] if a[2]]
        for _ in range(12):
            u, v = live[int(rng.integers(0, len(live)))]
            batch.append((0, u, v, 0))
        for _ in range(6):
            u, v = live[int(rng.integers(0, len(live)))]
            batch.append((2, u, v, int(rng.integers(1, 200))))
        for _ in range(12):
            u, v = int(rng.integers(0, G.n)), int(rng.integers(0, G.n))
            if u != v:
                batch.append((1, u, v, int(rng.integers(1, 100))))
        if b % 5 == 4 and D.par[t] >= 0:
            batch.append((0, D.par[t], t, 0))  # an arc of the current path
        D.update(batch)
        want = dijkstra(G, s, t)
        assert D.cost == want, (b, D.cost, want)
        if want < INF:
            assert _path_weight(G, D.par, s, t) == want, b
