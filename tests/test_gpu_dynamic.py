"""Dynamic A* (ddp_dyn) against the oracle: after every update batch the
cost equals a from-scratch A* on the updated graph (the reference's own
check, DA_star/genCSRwholegraph.cpp + GA_v2.cu on graph_cg.txt), the path is
valid on that graph, and the device graph equals the oracle's merged CSR
(DA_dyn_cpu.cu removeDelEdges + mergeDiff semantics) row by row."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scratch_cost(O, off_ref, col, w, s, t, heuristic=True):
    n = len(off_ref)
    h = np.maximum(O.bfs_heuristic(n, off_ref, col, w, t), 0) if heuristic else np.zeros(n, np.int32)
    found, cost, _, _, _ = O.astar(n, off_ref, col, w, h, s, t)
    return cost if found else 2147483647


def _run(d, O, g, batches, s, t, hkind=None, check_csr_every=1, **opts):
    """g: CSR with a sentinel last node; batches: list of (flag,u,v,w)."""
    hkind = d.H_BFS_HOPS if hkind is None else hkind
    dg = d.DeviceGraph.from_csr(g)
    dyn = d.DynamicSearch(dg, s, t, hkind, **opts)
    search_ctas, update_ctas = dyn.grid
    assert search_ctas >= 1 and update_ctas >= 1
    if opts.get("group", 0) > 0:
        assert update_ctas == opts["group"]  # far below the co-resident limit here
    else:
        assert update_ctas == search_ctas  # default: the initial search's grid
    off, col, w = g.off[:-1].copy(), g.col.copy(), g.w.copy()
    assert dyn.cost == _scratch_cost(O, off, col, w, s, t)
    for bi, (fl, uu, vv, ww) in enumerate(batches):
        cost = dyn.update(fl, uu, vv, ww)
        off, col, w, _ = O.apply_batch(len(off), off, col, w, fl, uu, vv, ww)
        want = _scratch_cost(O, off, col, w, s, t)
        assert cost == want, f"batch {bi}: {cost} != {want} ({dyn.stats()})"
        full_off = np.concatenate([off, [len(col)]]).astype(np.int32)
        if want != d.INF:
            ok, why = O.check_path(full_off, col, w, dyn.path(), s, t, cost)
            assert ok, f"batch {bi}: {why}"
        if bi % check_csr_every == 0:
            r = dg.read_csr()
            assert np.array_equal(r.off, full_off) and np.array_equal(r.col, col) and np.array_equal(r.w, w), bi
    dyn.close()
    return dg


def _split(fl, u, v, w, per):
    return [(fl[i:i + per], u[i:i + per], v[i:i + per], w[i:i + per]) for i in range(0, len(fl), per)]


@pytest.mark.parametrize("group", [0, 1, 8])
def test_dynamic_random_batches(gpu, oracle, group):
    """The 1M-node update workload's shape at 1/50 scale (20k nodes, avg
    out-degree 10): inserts of new arcs and deletes of existing non-chain
    arcs, weights in [1,1000].  Update batches on the initial search's grid
    (the default), on the one-CTA kernel and on a cooperative grid of 8
    CTAs."""
    d = gpu
    base = d.gen_random_chain(20000, 10, 1, 1000, 303)
    fl, u, v, w = d.gen_updates(base, 25, 200, 100, 1, 1000, 304)
    g = base.with_sentinel()
    s, t = int(base.perm[0]), int(base.perm[-1])
    _run(d, oracle, g, _split(fl, u, v, w, 200), s, t, group=group)


def test_dynamic_deletes_on_the_path(gpu, oracle):
    """Deleting arcs of the current shortest path exercises subtree
    invalidation and re-seeding; re-inserting them restores the cost."""
    d = gpu
    base = d.gen_random_chain(5000, 6, 1, 100, 11)
    g = base.with_sentinel()
    s, t = int(base.perm[0]), int(base.perm[-1])
    dg = d.DeviceGraph.from_csr(g)
    dyn = d.DynamicSearch(dg, s, t)
    off, col, w = g.off[:-1].copy(), g.col.copy(), g.w.copy()
    removed = []
    for rnd in range(6):
        p = dyn.path()
        assert len(p) >= 2
        a, b = int(p[len(p) // 2 - 1]), int(p[len(p) // 2])
        row = slice(off[a], off[a + 1] if a + 1 < len(off) else len(col))
        ws = w[row][col[row] == b]
        removed.append((a, b, int(ws[0])))
        fl, uu, vv, ww = [0], [a], [b], [0]
        cost = dyn.update(fl, uu, vv, ww)
        off, col, w, nd = oracle.apply_batch(len(off), off, col, w, fl, uu, vv, ww)
        assert nd == 1
        assert cost == _scratch_cost(oracle, off, col, w, s, t), rnd
        assert dyn.stats()["invalidated"] >= 1
    fl = [1] * len(removed)
    uu = [x[0] for x in removed]
    vv = [x[1] for x in removed]
    ww = [x[2] for x in removed]
    cost = dyn.update(fl, uu, vv, ww)
    off, col, w, _ = oracle.apply_batch(len(off), off, col, w, fl, uu, vv, ww)
    assert cost == _scratch_cost(oracle, off, col, w, s, t)
    dyn.close()


def test_dynamic_weight_changes_and_unreachable(gpu, oracle):
    d = gpu
    base = d.gen_random_chain(3000, 4, 1, 50, 21)
    g = base.with_sentinel()
    s, t = int(base.perm[0]), int(base.perm[-1])
    dg = d.DeviceGraph.from_csr(g)
    dyn = d.DynamicSearch(dg, s, t)
    off, col, w = g.off[:-1].copy(), g.col.copy(), g.w.copy()
    rng = np.random.default_rng(2)
    for rnd in range(8):
        p = dyn.path()
        k = int(rng.integers(0, len(p) - 1))
        a, b = int(p[k]), int(p[k + 1])
        nw = int(rng.integers(1, 200))
        fl, uu, vv, ww = [2, 2], [a, int(p[0])], [b, int(p[1])], [nw, 1]
        cost = dyn.update(fl, uu, vv, ww)
        off, col, w, _ = oracle.apply_batch(len(off), off, col, w, fl, uu, vv, ww)
        assert cost == _scratch_cost(oracle, off, col, w, s, t), rnd
    # cut every arc into t: unreachable, then one arc back
    n = len(off)
    ends = np.append(off[1:], len(col))
    src = np.repeat(np.arange(n), ends - off)
    into = np.flatnonzero((col == t))
    fl = [0] * len(into)
    uu = src[into].tolist()
    vv = [t] * len(into)
    cost = dyn.update(fl, uu, vv, [0] * len(into))
    off, col, w, _ = oracle.apply_batch(len(off), off, col, w, fl, uu, vv, [0] * len(into))
    assert cost == d.INF == _scratch_cost(oracle, off, col, w, s, t)
    assert len(dyn.path()) == 0
    cost = dyn.update([1], [s], [t], [777])
    off, col, w, _ = oracle.apply_batch(len(off), off, col, w, [1], [s], [t], [777])
    assert cost == _scratch_cost(oracle, off, col, w, s, t) <= 777
    dyn.close()


@pytest.mark.parametrize("heur", ["hops", "zero"])
def test_dynamic_same_arc_twice_in_one_batch(gpu, oracle, heur):
    """One batch changes a tree arc's weight twice: lighter, then heavier
    than before (the arc's final weight is what the repair may use), and
    heavier, then lighter than before; also a delete plus a weight change of
    the same pair (the change then hits the next live parallel arc, if any).
    Every cost equals a from-scratch oracle search on the updated graph."""
    d = gpu
    base = d.gen_random_chain(4000, 4, 20, 60, 77)
    g = base.with_sentinel()
    s, t = int(base.perm[0]), int(base.perm[-1])
    dg = d.DeviceGraph.from_csr(g)
    hk = d.H_BFS_HOPS if heur == "hops" else d.H_ZERO
    dyn = d.DynamicSearch(dg, s, t, hk)
    off, col, w = g.off[:-1].copy(), g.col.copy(), g.w.copy()
    rng = np.random.default_rng(5)
    for rnd in range(9):
        p = dyn.path()
        assert len(p) >= 2
        k = int(rng.integers(0, len(p) - 1))
        a, b = int(p[k]), int(p[k + 1])
        ends = np.append(off[1:], len(col))
        row = np.arange(off[a], ends[a])
        w0 = int(w[row[col[row] == b][0]])
        if rnd % 3 == 0:
            fl, ww = [2, 2], [1, w0 + 400]           # lighter, then heavier than before
        elif rnd % 3 == 1:
            fl, ww = [2, 2], [w0 + 400, max(1, w0 - 7)]  # heavier, then lighter than before
        else:
            fl, ww = [0, 2], [0, 1]                  # delete, then change the next parallel arc
        cost = dyn.update(fl, [a, a], [b, b], ww)
        off, col, w, _ = oracle.apply_batch(len(off), off, col, w, fl, [a, a], [b, b], ww)
        want = _scratch_cost(oracle, off, col, w, s, t)
        assert cost == want, (rnd, fl, ww, dyn.stats())
        if want != d.INF:
            full_off = np.concatenate([off, [len(col)]]).astype(np.int32)
            ok, why = oracle.check_path(full_off, col, w, dyn.path(), s, t, cost)
            assert ok, why
    dyn.close()


def test_dynamic_row_growth_and_relayout(gpu, oracle):
    """Many inserts into a few rows: rows move to the end of the arc array
    and the array is laid out again when it fills; the CSR stays exact."""
    d = gpu
    base = d.gen_random_chain(2000, 3, 1, 30, 5)
    g = base.with_sentinel()
    s, t = int(base.perm[0]), int(base.perm[-1])
    rng = np.random.default_rng(9)
    batches = []
    for b in range(6):
        m = 3000
        uu = rng.choice([s, int(base.perm[5]), int(base.perm[9])], m).astype(np.int32)
        vv = rng.integers(0, base.n, m).astype(np.int32)
        keep = uu != vv
        uu, vv = uu[keep], vv[keep]
        batches.append((np.ones(len(uu), np.int32), uu, vv, rng.integers(5, 60, len(uu)).astype(np.uint32)))
    _run(d, oracle, g, batches, s, t)


def test_dynamic_zero_heuristic_and_recreate(gpu, oracle):
    d = gpu
    base = d.gen_random_chain(8000, 8, 1, 1000, 77)
    fl, u, v, w = d.gen_updates(base, 6, 100, 50, 1, 1000, 78)
    g = base.with_sentinel()
    s, t = int(base.perm[3]), int(base.perm[-2])
    dg = _run(d, oracle, g, _split(fl, u, v, w, 100), s, t, hkind=d.H_ZERO, check_csr_every=3)
    # a second dynamic search on the same (already updated) graph
    r = dg.read_csr()
    dyn = d.DynamicSearch(dg, t, s)
    h = np.maximum(oracle.bfs_heuristic(r.n, r.off[:-1], r.col, r.w, s), 0)
    f, c, _, _, _ = oracle.astar(r.n, r.off[:-1], r.col, r.w, h, t, s)
    assert dyn.cost == (c if f else d.INF)
    # the static single-query engine sees the updated graph too
    hh = dg.heuristic(s, d.H_BFS_HOPS)
    assert dg.solve(t, s, hh).cost == dyn.cost
    dyn.close()


def test_dynamic_maze_obstacle_moves(gpu, oracle):
    """The maze workload of maze/create_maze.cpp:137-251: obstacles move
    every batch (cells open and close), dynamic costs equal from scratch."""
    d = gpu
    rows, cols = 96, 96
    wall = d.maze_walls(rows, cols, 0.3, 21)
    g = d.grid_from_walls(rows, cols, wall).with_sentinel()
    prot = np.zeros(rows * cols, np.uint8)
    prot[0] = prot[-1] = 1
    counts, fl, u, v, w = d.gen_maze_moves(rows, cols, wall, 10, 40, 22, prot)
    batches, pos = [], 0
    for c in counts:
        batches.append((fl[pos:pos + c], u[pos:pos + c], v[pos:pos + c], w[pos:pos + c]))
        pos += c
    _run(d, oracle, g, batches, 0, rows * cols - 1, check_csr_every=3)


def test_k_paths_match_successive_oracle(gpu, oracle):
    """ddp_kpaths (the reference's k-short method: delete the last arc of
    each path, re-solve) against the oracle doing the same deletions; wide
    weights make ties unlikely, so paths compare exactly."""
    d = gpu
    base = d.gen_random_chain(3000, 4, 1, 1_000_000, 31)
    g = base.with_sentinel()
    s, t = int(base.perm[0]), int(base.perm[-1])
    dg = d.DeviceGraph.from_csr(g)
    res = d.k_paths(dg, s, t, 6, d.H_BFS_HOPS, restore=True)
    assert len(res) >= 2
    off, col, w = g.off[:-1].copy(), g.col.copy(), g.w.copy()
    zeros = np.zeros(g.n, np.int32)
    for cost, path in res:
        f, c, p, _, _ = oracle.astar(len(off), off, col, w, zeros, s, t)
        p = list(p)
        if p and p[0] == t:
            p = p[::-1]
        assert f and c == cost and p == list(path)
        off, col, w, _ = oracle.apply_batch(len(off), off, col, w, [0], [int(path[-2])], [int(path[-1])], [0])
    # restore=True put the deleted arcs back: the first answer again
    assert dg.solve(s, t, dg.heuristic(t, d.H_BFS_HOPS)).cost == res[0][0]
    costs = [c for c, _ in res]
    assert costs == sorted(costs)
