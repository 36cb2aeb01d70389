"""Edge cases across the entry points: empty batches, single-node and
arc-less graphs, source == target, more landmarks than nodes, k-paths at
s == t, out-of-range queries in a batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_empty_and_degenerate_batches(gpu):
    d = gpu
    g = d.gen_random_chain(500, 4, 1, 20, 3)
    dg = d.DeviceGraph.from_csr(g)
    for hk in (d.H_ZERO, d.H_BFS_HOPS):
        be = d.BatchEngine(dg, hk, group=1)
        cost, plen = be.solve(np.zeros(0, np.int32), np.zeros(0, np.int32))
        assert len(cost) == 0 and len(plen) == 0
        cost, plen = be.solve([5, 7, 9], [5, 7, 9])  # s == t
        assert cost.tolist() == [0, 0, 0] and plen.tolist() == [1, 1, 1]
        assert be.path(1).tolist() == [7]
        be.close()


def test_single_node_and_arcless_graphs(gpu):
    d = gpu
    one = d.CSR(1, np.array([0, 0], np.int32), np.zeros(0, np.int32), np.zeros(0, np.uint32))
    dg = d.DeviceGraph.from_csr(one)
    r = dg.solve(0, 0)
    assert r.cost == 0 and r.path.tolist() == [0]
    bare = d.CSR(50, np.zeros(51, np.int32), np.zeros(0, np.int32), np.zeros(0, np.uint32))
    db = d.DeviceGraph.from_csr(bare)
    assert db.solve(3, 9).cost == d.INF
    assert db.solve(3, 9, flags=d.OPT_ONE_CTA).cost == d.INF
    cost, _ = d.BatchEngine(db, d.H_ZERO, group=1).solve([1, 2], [2, 2])
    assert cost.tolist() == [d.INF, 0]


def test_landmarks_on_a_tiny_graph(gpu, oracle):
    d = gpu
    g = d.gen_random_chain(6, 2, 1, 9, 5)
    dg = d.DeviceGraph.from_csr(g)
    dg.build_landmarks(8, seed=2)  # more landmarks than nodes: repeats are allowed
    gs = g.with_sentinel()
    for s in range(6):
        for t in range(6):
            f, c, _, _, _ = oracle.astar(gs.n, gs.off[:-1], gs.col, gs.w, np.zeros(gs.n, np.int32), s, t)
            assert dg.solve(s, t, dg.heuristic(t, d.H_LANDMARK)).cost == (c if f else d.INF)


def test_kpaths_at_source_equals_target(gpu):
    d = gpu
    g = d.gen_random_chain(300, 3, 1, 10, 6).with_sentinel()
    dg = d.DeviceGraph.from_csr(g)
    res = d.k_paths(dg, 4, 4, 3, d.H_ZERO)
    assert len(res) == 1 and res[0][0] == 0 and res[0][1].tolist() == [4]


def test_batch_rejects_nothing_but_reports_out_of_range(gpu):
    """Out-of-range endpoints inside a batch answer DDP_INF for that query
    alone; the other queries stay exact."""
    d = gpu
    g = d.gen_random_chain(400, 4, 1, 20, 9)
    dg = d.DeviceGraph.from_csr(g)
    ref = d.BatchEngine(dg, d.H_ZERO, group=1).solve([1, 2], [3, 4])[0]
    cost, _ = d.BatchEngine(dg, d.H_ZERO, group=1).solve([1, -5, 2, 0], [3, 4, 4, 10**6])
    assert cost.tolist() == [ref[0], d.INF, ref[1], d.INF]
