"""The bidirectional batch engine (DDP_H_BIDIR): every cost against the
oracle and every path validated, on random digraphs, graphs with zero-weight
arcs, grids, unreachable targets, source == target, the dynamic layout after
updates, the CUDA-graph replay of the device path, and serving (alone equals
mixed, answers on the graph version each request ran on)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INF = 2147483647


def _oracle_costs(O, g, S, T):
    gs = g.with_sentinel()
    cost, _, _, done = O.astar_many(gs.n, gs.off[:-1], gs.col, gs.w, S, T, hkind=0, mode=O.HEAP_POSMAP,
                                    threads=os.cpu_count() or 1, budget_s=1e9)
    assert done == len(S)
    return cost


def _check(O, be, g, S, T, cost, want, plen=None):
    assert np.array_equal(cost, want), np.flatnonzero(cost != want)[:8]
    for i in range(len(S)):
        p = be.path(i)
        if want[i] == INF:
            assert len(p) == 0, i
            continue
        if plen is not None:
            assert len(p) == plen[i]
        ok, why = O.check_path(g.off, g.col, g.w, p, int(S[i]), int(T[i]), int(want[i]))
        assert ok, f"query {i} ({S[i]} -> {T[i]}): {why}"


def _pairs(n, k, seed):
    rng = np.random.default_rng(seed)
    S = rng.integers(0, n, k).astype(np.int32)
    T = rng.integers(0, n, k).astype(np.int32)
    T[:3] = S[:3]
    return S, T


@pytest.mark.parametrize("n,deg,wmax,seed", [(30000, 8, 100, 11), (20000, 3, 1000, 12), (5001, 2, 5, 13)])
def test_bidir_random_graphs(gpu, oracle, n, deg, wmax, seed):
    d = gpu
    g = d.gen_random_chain(n, deg, 1, wmax, seed)
    dg = d.DeviceGraph.from_csr(g)
    S, T = _pairs(g.n, 300, seed)
    want = _oracle_costs(oracle, g, S, T)
    be = d.BatchEngine(dg, d.H_BIDIR)
    for _ in range(2):  # the second batch reuses the reset slots
        cost, plen = be.solve(S, T)
        _check(oracle, be, g, S, T, cost, want, plen)
    be.close()
    dg.close()


def test_bidir_zero_weights_and_unreachable(gpu, oracle):
    """Zero-weight arcs (ties) and nodes that cannot reach each other: a
    chain-free random graph leaves some pairs disconnected."""
    d = gpu
    rng = np.random.default_rng(5)
    n, e = 4000, 10000
    u = rng.integers(0, n, e)
    v = rng.integers(0, n, e)
    keep = u != v
    u, v = u[keep], v[keep]
    w = rng.integers(0, 4, len(u)).astype(np.uint32)  # a quarter of the arcs weigh 0
    order = np.lexsort((v, u))
    u, v, w = u[order], v[order], w[order]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, u + 1, 1)
    off = np.cumsum(off).astype(np.int32)
    g = d.CSR(n, off, v.astype(np.int32), w)
    dg = d.DeviceGraph.from_csr(g)
    S, T = _pairs(n, 400, 6)
    want = _oracle_costs(oracle, g, S, T)
    assert (want == INF).any() and ((want > 0) & (want < INF)).sum() > 50
    be = d.BatchEngine(dg, d.H_BIDIR, grid=32)
    cost, plen = be.solve(S, T)
    _check(oracle, be, g, S, T, cost, want, plen)
    be.close()
    dg.close()


def test_bidir_maze_long_paths(gpu, oracle):
    d = gpu
    m = d.gen_maze(200, 300, 0.25, 21)
    dg = d.DeviceGraph.from_csr(m)
    S, T = _pairs(m.n, 64, 22)
    S[10], T[10] = 0, m.n - 1
    want = _oracle_costs(oracle, m, S, T)
    be = d.BatchEngine(dg, d.H_BIDIR)
    cost, plen = be.solve(S, T)
    _check(oracle, be, m, S, T, cost, want, plen)
    be.close()
    dg.close()


def test_bidir_device_replay_and_dynamic_layout(gpu, oracle):
    torch = pytest.importorskip("torch")
    d = gpu
    g = d.gen_random_chain(20000, 6, 1, 100, 31)
    dg = d.DeviceGraph.from_csr(g)
    S, T = _pairs(g.n, 256, 32)
    dev = torch.device("cuda", 0)
    dS = torch.from_numpy(S).to(dev)
    dT = torch.from_numpy(T).to(dev)
    dcost = torch.empty(len(S), dtype=torch.int32, device=dev)
    be = d.BatchEngine(dg, d.H_BIDIR)
    want = _oracle_costs(oracle, g, S, T)
    for _ in range(3):
        dcost.fill_(-7)
        be.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), 0)
        be.sync()
        _check(oracle, be, g, S, T, dcost.cpu().numpy(), want)
    # updates switch the graph to rows with explicit ends and dead arcs
    rng = np.random.default_rng(33)
    src = np.repeat(np.arange(g.n, dtype=np.int32), np.diff(g.off))
    dj = rng.choice(g.e, 2000, replace=False)
    ins_u = rng.integers(0, g.n, 1500).astype(np.int32)
    ins_v = rng.integers(0, g.n, 1500).astype(np.int32)
    ok = ins_u != ins_v
    fl = np.concatenate([np.zeros(len(dj), np.int32), np.ones(ok.sum(), np.int32)])
    uu = np.concatenate([src[dj], ins_u[ok]])
    vv = np.concatenate([g.col[dj], ins_v[ok]])
    ww = np.concatenate([g.w[dj], rng.integers(1, 10, ok.sum()).astype(np.uint32)])
    dyn = d.DynamicSearch(dg, int(S[5]), int(T[5]), d.H_ZERO)
    dyn.update(fl, uu, vv, ww)
    dyn.close()
    g2 = dg.read_csr()
    want2 = _oracle_costs(oracle, g2, S, T)
    assert not np.array_equal(want, want2)
    for _ in range(2):
        dcost.fill_(-7)
        be.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), 0)
        be.sync()
        _check(oracle, be, g2, S, T, dcost.cpu().numpy(), want2)
    be.close()
    dg.close()


def test_bidir_serving_alone_equals_mixed(gpu, oracle):
    d = gpu
    g = d.gen_random_chain(20000, 6, 1, 100, 41)
    dg = d.DeviceGraph.from_csr(g)
    S, T = _pairs(g.n, 200, 42)
    want = _oracle_costs(oracle, g, S, T)
    srv = d.Server(dg, d.H_BIDIR, max_requests=1 << 14, grid=48)
    first = srv.submit(S, T)
    ids, costs, _, _ = srv.drain()
    got = np.empty(len(S), np.int32)
    got[ids - first] = costs
    assert np.array_equal(got, want)
    for i in range(0, len(S), 23):  # alone
        f1 = srv.submit(S[i:i + 1], T[i:i + 1])
        ids1, c1, _, _ = srv.drain()
        assert ids1[-1] == f1 and c1[-1] == want[i]
    srv.close()
    dg.close()


def test_bidir_serving_with_updates(gpu, oracle):
    """Weight changes, deletes and inserts between requests while searches
    run: each answer equals the oracle on the graph version it reports."""
    d = gpu
    g = d.gen_random_chain(20000, 6, 1, 100, 44)
    dg = d.DeviceGraph.from_csr(g)
    srv = d.Server(dg, d.H_BIDIR, max_requests=4096, versions=3, grid=32)
    rng = np.random.default_rng(45)
    off, col, w = g.off[:-1].copy(), g.col.copy(), g.w.copy()
    versions = [g]
    submitted = []
    for rnd in range(5):
        S = rng.integers(0, g.n, 40).astype(np.int32)
        T = rng.integers(0, g.n, 40).astype(np.int32)
        srv.submit(S, T)
        submitted += list(zip(S.tolist(), T.tolist()))
        src = np.repeat(np.arange(len(off)), np.diff(np.append(off, len(col))))
        live = np.flatnonzero(col >= 0)
        pick = rng.choice(live, 60, replace=False)
        fl, uu, vv, ww = [], [], [], []
        for j in pick[:40]:
            fl.append(2); uu.append(int(src[j])); vv.append(int(col[j]))
            ww.append(max(1, int(round(w[j] * rng.uniform(0.5, 2.0)))))
        for j in pick[40:50]:
            fl.append(0); uu.append(int(src[j])); vv.append(int(col[j])); ww.append(0)
        for j in pick[50:60]:
            fl.append(1); uu.append(int(col[j])); vv.append(int(src[j])); ww.append(int(rng.integers(1, 5)))
        srv.update(fl, uu, vv, ww)
        off, col, w, _ = oracle.apply_batch(len(off), off, col, w, fl, uu, vv, ww)
        versions.append(d.CSR(g.n, np.append(off, len(col)).astype(np.int32), col, w))
    ids, costs, lat, ver = srv.drain()
    assert len(ids) == len(submitted)
    for k in range(len(ids)):
        s_, t_ = submitted[int(ids[k])]
        gv = versions[int(ver[k])]
        want = _oracle_costs(oracle, gv, np.array([s_], np.int32), np.array([t_], np.int32))[0]
        assert costs[k] == want, (int(ids[k]), int(ver[k]))
    srv.close()
    dg.close()


@pytest.mark.parametrize("rows,cols,wall,seed", [(200, 300, 0.25, 51), (120, 120, 0.35, 52)])
def test_bidir_manhattan_potentials_maze(gpu, oracle, rows, cols, wall, seed):
    """Bidirectional A* with average Manhattan potentials on mazes: costs
    against the oracle, every path valid; the corner-to-corner query too."""
    d = gpu
    m = d.gen_maze(rows, cols, wall, seed)
    dg = d.DeviceGraph.from_csr(m)
    S, T = _pairs(m.n, 96, seed + 1)
    S[10], T[10] = 0, m.n - 1
    want = _oracle_costs(oracle, m, S, T)
    be = d.BatchEngine(dg, d.H_BIDIR_MANHATTAN)
    for _ in range(2):
        cost, plen = be.solve(S, T)
        _check(oracle, be, m, S, T, cost, want, plen)
    # the potentials only steer the search: it expands fewer nodes than the
    # plain bidirectional search on the long query
    st_pot = be.stats()[0][10, 0]
    bz = d.BatchEngine(dg, d.H_BIDIR)
    bz.solve(S, T)
    assert st_pot < bz.stats()[0][10, 0]
    bz.close()
    be.close()
    dg.close()


def _geo(d, n, seed):
    g = d.gen_geometric(n, 6, 1 << 20, 100000, seed)
    dg = d.DeviceGraph.from_csr(g)
    dg.set_euclid(d.euclid_rho_fp(g))
    return g, dg


def test_bidir_euclid_potentials_geometric(gpu, oracle):
    d = gpu
    g, dg = _geo(d, 30000, 61)
    S, T = _pairs(g.n, 200, 62)
    want = _oracle_costs(oracle, g, S, T)
    be = d.BatchEngine(dg, d.H_BIDIR_EUCLID)
    cost, plen = be.solve(S, T)
    _check(oracle, be, g, S, T, cost, want, plen)
    expanded_pot = be.stats()[0][:, 0].sum()
    bz = d.BatchEngine(dg, d.H_BIDIR)
    bz.solve(S, T)
    assert expanded_pot < bz.stats()[0][:, 0].sum()
    bz.close()
    be.close()
    dg.close()


def test_bidir_euclid_serving_with_updates(gpu, oracle):
    """Weight changes x[0.5, 2] (the Euclidean scale drops), deletes and
    inserts while searches run: each answer equals the oracle on the graph
    version it reports."""
    d = gpu
    g, dg = _geo(d, 20000, 71)
    srv = d.Server(dg, d.H_BIDIR_EUCLID, max_requests=4096, versions=3, grid=32)
    rng = np.random.default_rng(72)
    off, col, w = g.off[:-1].copy(), g.col.copy(), g.w.copy()
    versions = [g]
    submitted = []
    for rnd in range(4):
        S = rng.integers(0, g.n, 40).astype(np.int32)
        T = rng.integers(0, g.n, 40).astype(np.int32)
        srv.submit(S, T)
        submitted += list(zip(S.tolist(), T.tolist()))
        src = np.repeat(np.arange(len(off)), np.diff(np.append(off, len(col))))
        live = np.flatnonzero(col >= 0)
        pick = rng.choice(live, 60, replace=False)
        fl, uu, vv, ww = [], [], [], []
        for j in pick[:40]:
            fl.append(2); uu.append(int(src[j])); vv.append(int(col[j]))
            ww.append(max(1, int(round(w[j] * rng.uniform(0.5, 2.0)))))
        for j in pick[40:50]:
            fl.append(0); uu.append(int(src[j])); vv.append(int(col[j])); ww.append(0)
        for j in pick[50:60]:
            fl.append(1); uu.append(int(col[j])); vv.append(int(src[j])); ww.append(int(w[j]))
        srv.update(fl, uu, vv, ww)
        off, col, w, _ = oracle.apply_batch(len(off), off, col, w, fl, uu, vv, ww)
        versions.append(d.CSR(g.n, np.append(off, len(col)).astype(np.int32), col, w, xy=g.xy))
    ids, costs, lat, ver = srv.drain()
    assert len(ids) == len(submitted)
    for k in range(len(ids)):
        s_, t_ = submitted[int(ids[k])]
        gv = versions[int(ver[k])]
        want = _oracle_costs(oracle, gv, np.array([s_], np.int32), np.array([t_], np.int32))[0]
        assert costs[k] == want, (int(ids[k]), int(ver[k]))
    srv.close()
    dg.close()


@pytest.mark.parametrize("n,deg,wmax,seed", [(30000, 8, 100, 81), (6001, 2, 3, 82)])
def test_bidir_hashed_records(gpu, oracle, n, deg, wmax, seed):
    """DDP_OPT_HASH: each slot keeps its closed set in a hash table sized to
    the touched nodes; costs and paths as with one record per node, on the
    host path and the device path (two replays)."""
    torch = pytest.importorskip("torch")
    d = gpu
    g = d.gen_random_chain(n, deg, 1, wmax, seed)
    dg = d.DeviceGraph.from_csr(g)
    S, T = _pairs(g.n, 300, seed)
    want = _oracle_costs(oracle, g, S, T)
    be = d.BatchEngine(dg, d.H_BIDIR, flags=d.OPT_HASH)
    cost, plen = be.solve(S, T)
    _check(oracle, be, g, S, T, cost, want, plen)
    dev = torch.device("cuda", 0)
    dS, dT = torch.from_numpy(S).to(dev), torch.from_numpy(T).to(dev)
    dc = torch.empty(len(S), dtype=torch.int32, device=dev)
    for _ in range(2):
        dc.fill_(-7)
        be.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dc.data_ptr(), 0)
        be.sync()
        _check(oracle, be, g, S, T, dc.cpu().numpy(), want)
    be.close()
    dg.close()


def test_bidir_hashed_table_full(gpu, oracle):
    """Two disconnected 100k-node components: a query across them explores
    both (about 200k records, more than the 2^16-record table of a graph
    this size holds).  The device path reports -1 for it; the host path
    re-runs it and returns the oracle's answer; queries inside a component
    stay exact."""
    torch = pytest.importorskip("torch")
    d = gpu
    a = d.gen_random_chain(100000, 3, 1, 50, 91)
    b = d.gen_random_chain(100000, 3, 1, 50, 92)
    off = np.concatenate([a.off[:-1], b.off + a.e]).astype(np.int32)
    col = np.concatenate([a.col, b.col + a.n]).astype(np.int32)
    w = np.concatenate([a.w, b.w]).astype(np.uint32)
    g = d.CSR(a.n + b.n, off, col, w)
    dg = d.DeviceGraph.from_csr(g)
    S = np.array([5, 7, 100005, 11], np.int32)
    T = np.array([150000, 99999, 100100, 12], np.int32)  # query 0 crosses components
    want = _oracle_costs(oracle, g, S, T)
    assert want[0] == INF
    be = d.BatchEngine(dg, d.H_BIDIR, flags=d.OPT_HASH, grid=4)
    dev = torch.device("cuda", 0)
    dS, dT = torch.from_numpy(S).to(dev), torch.from_numpy(T).to(dev)
    dc = torch.empty(len(S), dtype=torch.int32, device=dev)
    be.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dc.data_ptr(), 0)
    be.sync()
    got = dc.cpu().numpy()
    assert got[0] == -1 and np.array_equal(got[1:], want[1:])
    cost, _ = be.solve(S, T)
    assert np.array_equal(cost, want)
    be.close()
    dg.close()
