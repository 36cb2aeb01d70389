"""GPU parity: the CUDA path (through the C-ABI) against the oracle.

Bar: costs bit-exact; every returned path starts at s, ends at t, uses live
arcs only and its summed weight (+ h(t)) equals the cost (ties may pick a
different equal-cost path)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_cost(O, g, h, s, t):
    """g has a sentinel; h >= 0 array or None."""
    hh = np.zeros(g.n, np.int32) if h is None else np.maximum(h, 0)
    found, cost, _, _, _ = O.astar(g.n, g.off[:-1], g.col, g.w, hh, s, t)
    return cost if found else 2147483647


def test_golden_cases_user_heuristic(gpu, oracle, golden):
    d = gpu
    for name, c in golden.items():
        if name == "lib_main":
            continue
        n = int(c["n"])
        off = np.concatenate([c["off"], [len(c["col"])]]).astype(np.int32)
        g = d.CSR(n, off, c["col"], c["w"])
        dg = d.DeviceGraph.from_csr(g)
        s, t = int(c["s"]), int(c["t"])
        h = dg.heuristic(t, d.H_USER, user_h=c["h"])
        r = dg.solve(s, t, h)
        if name == "last_row_quirk":
            # the reference drops the last arc of node n-1 (A_star_cpu.cpp:170);
            # the product reads the full row, so its cost can only be <=
            assert r.cost <= int(c["cost"])
            continue
        want = int(c["cost"]) if int(c["cost"]) >= 0 else d.INF
        assert r.cost == want, name
        if want != d.INF:
            ok, why = oracle.check_path(off, c["col"], c["w"], r.path, s, t, r.cost, int(c["h"][t]))
            assert ok, f"{name}: {why}"
        else:
            assert len(r.path) == 0
        dg.close()


def test_lib_mirror_on_golden(gpu, golden):
    d = gpu
    c = golden["kat8"]
    g = d.Graph.from_csr(d.CSR(8, np.concatenate([c["off"], [12]]).astype(np.int32), c["col"], c["w"]))
    gg = d.GPU_Graph(g)
    a = d.GPU_A_Star(d.GPU_Dynamic_Graph(gg), 0, 7, 1)
    assert a.get_path() == [-1]
    a.set_huiristics(np.zeros(8, np.int32))
    assert a.get_path() == golden["lib_main"]["path"].tolist() == [0, 2, 4, 6, 7]
    b = d.A_Star(d.Dynamic_Graph(g), 7, 0, 3)
    b.set_huiristics(np.zeros(8, np.int32))
    assert b.get_path() == [7, 0]


def test_bfs_heuristic_exact(gpu, oracle):
    d = gpu
    for seed, n, deg in [(1, 2000, 3), (2, 20000, 8), (3, 5000, 1)]:
        g = d.gen_random_chain(n, deg, 1, 100, seed)
        # cut the chain's reachability: remove all arcs into node perm[n//2]
        dg = d.DeviceGraph.from_csr(g)
        for t in (0, n // 3, n - 1):
            h = dg.heuristic(t, d.H_BFS_HOPS, want_values=True)
            ref = oracle.bfs_heuristic(g.n, g.off[:-1], g.col, g.w, t)
            assert np.array_equal(h.values, ref)
            h.close()


def test_single_query_random(gpu, oracle):
    d = gpu
    rng = np.random.default_rng(5)
    for seed in range(3):
        g = d.gen_random_chain(30000, 8, 1, 100, 40 + seed).with_sentinel()
        dg = d.DeviceGraph.from_csr(g)
        for _ in range(4):
            s, t = (int(x) for x in rng.integers(0, g.n - 1, 2))
            h = dg.heuristic(t, d.H_BFS_HOPS, want_values=True)
            for K, delta in [(0, 0), (1024, 0), (64, 1), (0, 500)]:
                r = dg.solve(s, t, h, K=K, delta=delta)
                assert r.cost == _oracle_cost(oracle, g, h.values, s, t)
                ok, why = oracle.check_path(g.off, g.col, g.w, r.path, s, t, r.cost)
                assert ok, why
            h.close()


@pytest.mark.parametrize("flags", [0, 2])  # 2 = OPT_ONE_CTA (latency mode of the one-CTA engine)
def test_zero_weights_and_edge_cases(gpu, oracle, flags):
    d = gpu
    g = d.gen_random_chain(4000, 5, 0, 3, 8).with_sentinel()   # many zero-weight arcs
    dg = d.DeviceGraph.from_csr(g)
    for s, t in [(1, 2), (5, 3999), (7, 7), (0, g.n - 1)]:
        r = dg.solve(s, t, flags=flags)
        assert r.cost == _oracle_cost(oracle, g, None, s, t)
        if s == t:
            assert r.path.tolist() == [s]
        elif r.cost == d.INF:
            assert len(r.path) == 0
        else:
            ok, why = oracle.check_path(g.off, g.col, g.w, r.path, s, t, r.cost)
            assert ok, why
    with pytest.raises(d.DdpError):
        dg.solve(-1, 3)
    with pytest.raises(d.DdpError):
        dg.solve(0, g.n)


def test_zero_weight_batches(gpu, oracle):
    """Zero-weight arcs through the batch slots (one-CTA engine, both
    relaxation modes: zero h runs the latency mode, BFS hops the throughput
    mode): exact costs and valid paths (no parent cycles on equal g)."""
    d = gpu
    g = d.gen_random_chain(6000, 6, 0, 2, 18).with_sentinel()
    dg = d.DeviceGraph.from_csr(g)
    rng = np.random.default_rng(4)
    S = rng.integers(0, g.n - 1, 64).astype(np.int32)
    T = rng.integers(0, g.n - 1, 64).astype(np.int32)
    want = np.array([_oracle_cost(oracle, g, None, int(s), int(t)) for s, t in zip(S, T)])
    for hk in (d.H_ZERO, d.H_BFS_HOPS):
        be = d.BatchEngine(dg, hk, group=1)
        cost, _ = be.solve(S, T)
        assert np.array_equal(cost, want), hk
        for i in range(64):
            if cost[i] != d.INF:
                ok, why = oracle.check_path(g.off, g.col, g.w, be.path(i), int(S[i]), int(T[i]), int(cost[i]))
                assert ok, (hk, i, why)


def test_dead_arcs_are_skipped(gpu, oracle):
    d = gpu
    g = d.gen_random_chain(3000, 6, 1, 50, 12).with_sentinel()
    col = g.col.copy()
    rng = np.random.default_rng(0)
    dead = rng.choice(len(col), len(col) // 5, replace=False)
    col[dead] = -1
    g2 = d.CSR(g.n, g.off, col, g.w)
    dg = d.DeviceGraph.from_csr(g2)
    # oracle on the compacted live graph
    live = col >= 0
    src = np.repeat(np.arange(g.n), np.diff(g.off))[live]
    off = np.zeros(g.n + 1, np.int32)
    np.add.at(off, src + 1, 1)
    off = np.cumsum(off).astype(np.int32)
    gl = d.CSR(g.n, off, col[live], g.w[live])
    for s, t in [(3, 2500), (100, 7), (2999, 0)]:
        r = dg.solve(s, t)
        assert r.cost == _oracle_cost(oracle, gl, None, s, t)
        if r.cost != d.INF:
            ok, why = oracle.check_path(gl.off, gl.col, gl.w, r.path, s, t, r.cost)
            assert ok, why


def test_maze_manhattan(gpu, oracle):
    d = gpu
    m = d.gen_maze(200, 300, 0.3, 4)
    dg = d.DeviceGraph.from_csr(m)
    t = m.n - 1
    h = dg.heuristic(t, d.H_MANHATTAN, want_values=True)
    r = dg.solve(0, t, h, K=256)
    mg = m.with_sentinel()
    hh = np.concatenate([h.values, [0]]).astype(np.int32)
    assert r.cost == _oracle_cost(oracle, mg, hh, 0, t)
    ok, why = oracle.check_path(m.off, m.col, m.w, r.path, 0, t, r.cost)
    assert ok, why


def test_batch_matches_oracle(gpu, oracle):
    d = gpu
    g = d.gen_random_chain(20000, 8, 1, 100, 77).with_sentinel()
    dg = d.DeviceGraph.from_csr(g)
    S, T, _ = d.gen_pairs(d.CSR(g.n, g.off, g.col, g.w), 96, 4, 400, 5)
    for hk in (d.H_BFS_HOPS, d.H_ZERO):
        be = d.BatchEngine(dg, hk, grid=40)
        cost, plen = be.solve(S, T)
        for i in range(len(S)):
            h = None
            if hk == d.H_BFS_HOPS:
                h = oracle.bfs_heuristic(g.n, g.off[:-1], g.col, g.w, int(T[i]))
            assert cost[i] == _oracle_cost(oracle, g, h, int(S[i]), int(T[i])), i
            p = be.path(i)
            assert len(p) == plen[i]
            ok, why = oracle.check_path(g.off, g.col, g.w, p, int(S[i]), int(T[i]), int(cost[i]))
            assert ok, f"{i}: {why}"
        st, t0, t1 = be.stats()
        assert (st[:, 0] > 0).all() and (t1 >= t0).all()
        be.close()


def test_batch_alone_equals_mixed(gpu):
    """Each query's result is the same alone and inside a batch."""
    d = gpu
    g = d.gen_random_chain(20000, 8, 1, 100, 78)
    dg = d.DeviceGraph.from_csr(g)
    S, T, _ = d.gen_pairs(g, 64, 4, 400, 6)
    be = d.BatchEngine(dg, d.H_BFS_HOPS, grid=24)
    mixed, _ = be.solve(S, T)
    for i in range(0, 64, 7):
        alone, _ = be.solve(S[i:i + 1], T[i:i + 1])
        assert alone[0] == mixed[i]
        h = dg.heuristic(int(T[i]), d.H_BFS_HOPS)
        assert dg.solve(int(S[i]), int(T[i]), h).cost == mixed[i]
        h.close()


def test_batch_maze_and_overflow_recovery(gpu, oracle):
    d = gpu
    m = d.gen_maze(120, 160, 0.25, 9)
    dg = d.DeviceGraph.from_csr(m)
    rng = np.random.default_rng(3)
    S = rng.integers(0, m.n, 24).astype(np.int32)
    T = rng.integers(0, m.n, 24).astype(np.int32)
    # tiny queues: every query overflows its slot and is re-run on the
    # single-query engine, results stay exact
    be = d.BatchEngine(dg, d.H_MANHATTAN, grid=8, queue_cap=64)
    cost, _ = be.solve(S, T)
    mg = m.with_sentinel()
    for i in range(len(S)):
        tx, ty = m.xy[T[i]]
        h = np.concatenate([np.abs(m.xy[:, 0] - tx) + np.abs(m.xy[:, 1] - ty), [0]]).astype(np.int32)
        assert cost[i] == _oracle_cost(oracle, mg, h, int(S[i]), int(T[i]))
        if cost[i] != d.INF:
            ok, why = oracle.check_path(m.off, m.col, m.w, be.path(i), int(S[i]), int(T[i]), int(cost[i]))
            assert ok, why
    be.close()


def test_explicit_small_queue_reports_overflow(gpu):
    d = gpu
    g = d.gen_random_chain(20000, 8, 1, 100, 3)
    dg = d.DeviceGraph.from_csr(g)
    with pytest.raises(d.DdpError) as ei:
        dg.solve(0, 12345, queue_cap=16)
    assert ei.value.code == 5  # DDP_ERR_QUEUE_OVERFLOW
    # the handle stays usable
    assert dg.solve(0, 12345).cost > 0


def test_config1_full_size(gpu, oracle):
    """The 100k-node single-query workload at full size: N=100,000, avg
    out-degree 8, w in [1,100], one seeded pair, h = reverse-BFS hops x
    min w, K = 1024."""
    d = gpu
    g = d.gen_random_chain(100000, 8, 1, 100, 2024)
    dg = d.DeviceGraph.from_csr(g)
    s, t = int(g.perm[0]), int(g.perm[-1])
    h = dg.heuristic(t, d.H_BFS_HOPS, want_values=True)
    r = dg.solve(s, t, h, K=1024)
    gs = g.with_sentinel()
    hh = np.concatenate([h.values, [0]])
    assert r.cost == _oracle_cost(oracle, gs, hh, s, t)
    ok, why = oracle.check_path(g.off, g.col, g.w, r.path, s, t, r.cost)
    assert ok, why


def test_capped_bfs_heuristic(gpu, oracle):
    """DDP_H_BFS_CAPPED: exact hops up to the cap, cap elsewhere; costs stay
    exact (single query and batch)."""
    d = gpu
    g = d.gen_random_chain(200000, 8, 1, 100, 91).with_sentinel()
    dg = d.DeviceGraph.from_csr(g)
    S, T, _ = d.gen_pairs(d.CSR(g.n, g.off, g.col, g.w), 24, 4, 400, 15)
    be = d.BatchEngine(dg, d.H_BFS_CAPPED, grid=24)
    cost, _ = be.solve(S, T)
    for i in range(len(S)):
        s, t = int(S[i]), int(T[i])
        href = oracle.bfs_heuristic(g.n, g.off[:-1], g.col, g.w, t)
        h = dg.heuristic(t, d.H_BFS_CAPPED, want_values=True)
        # capped values never exceed the exact hops (admissible)
        reach = href >= 0
        assert (h.values[reach] <= href[reach]).all()
        assert (h.values[reach] >= np.minimum(href[reach], h.values[reach].max())).all()
        want = _oracle_cost(oracle, g, href, s, t)
        assert dg.solve(s, t, h).cost == want
        assert cost[i] == want
        h.close()
    be.close()


@pytest.mark.parametrize("group", [2, 7])
def test_batch_multi_cta_groups(gpu, oracle, group):
    """Slots made of several cooperative CTAs give the same exact costs."""
    d = gpu
    g = d.gen_random_chain(50000, 8, 1, 100, 123).with_sentinel()
    dg = d.DeviceGraph.from_csr(g)
    S, T, _ = d.gen_pairs(d.CSR(g.n, g.off, g.col, g.w), 40, 4, 400, 8)
    be = d.BatchEngine(dg, d.H_BFS_CAPPED, group=group)
    assert be.info()["group"] == group
    cost, plen = be.solve(S, T)
    for i in range(len(S)):
        href = oracle.bfs_heuristic(g.n, g.off[:-1], g.col, g.w, int(T[i]))
        assert cost[i] == _oracle_cost(oracle, g, href, int(S[i]), int(T[i])), i
        ok, why = oracle.check_path(g.off, g.col, g.w, be.path(i), int(S[i]), int(T[i]), int(cost[i]))
        assert ok, why
    be.close()


def test_async_one_cta_engine(gpu, oracle):
    """The asynchronous single-CTA engine (ddp_solve with OPT_ONE_CTA, and
    one-CTA batch slots) matches the oracle, also when it alternates with the
    phase-synchronous engine on the same workspace."""
    d = gpu
    m = d.gen_maze(160, 200, 0.3, 12)
    dm = d.DeviceGraph.from_csr(m)
    t = m.n - 1
    h = dm.heuristic(t, d.H_MANHATTAN, want_values=True)
    mg = m.with_sentinel()
    hh = np.concatenate([h.values, [0]]).astype(np.int32)
    want = _oracle_cost(oracle, mg, hh, 0, t)
    for flags in (d.OPT_ONE_CTA, 0, d.OPT_ONE_CTA):
        r = dm.solve(0, t, h, flags=flags)
        assert r.cost == want
        ok, why = oracle.check_path(m.off, m.col, m.w, r.path, 0, t, r.cost)
        assert ok, why
    g = d.gen_random_chain(20000, 8, 1, 100, 404).with_sentinel()
    dg = d.DeviceGraph.from_csr(g)
    S, T, _ = d.gen_pairs(d.CSR(g.n, g.off, g.col, g.w), 48, 4, 400, 9)
    for hk in (d.H_BFS_CAPPED, d.H_ZERO):
        be = d.BatchEngine(dg, hk, group=1)
        cost, _ = be.solve(S, T)
        for i in range(len(S)):
            href = oracle.bfs_heuristic(g.n, g.off[:-1], g.col, g.w, int(T[i]))
            assert cost[i] == _oracle_cost(oracle, g, href, int(S[i]), int(T[i])), i
            ok, why = oracle.check_path(g.off, g.col, g.w, be.path(i), int(S[i]), int(T[i]), int(cost[i]))
            assert ok, why
        be.close()
    for s_, t_ in [(3, 15000), (19000, 7)]:
        hq = dg.heuristic(t_, d.H_BFS_HOPS)
        a = dg.solve(s_, t_, hq, flags=d.OPT_ONE_CTA)
        b = dg.solve(s_, t_, hq)
        assert a.cost == b.cost == _oracle_cost(oracle, g, oracle.bfs_heuristic(g.n, g.off[:-1], g.col, g.w, t_), s_, t_)
