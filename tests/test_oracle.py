"""The oracle (CPU restatement of the reference) pinned against the
reference's own outputs: the hand-checkable 8-node graph and golden vectors
produced by the reference's compiled GA_star/A_star_cpu.cpp."""
import numpy as np
import pytest

KAT_OFF = [0, 2, 3, 5, 7, 9, 10, 11]
KAT_COL = [1, 2, 3, 3, 4, 4, 5, 5, 6, 7, 7, 0]
KAT_W = [4, 1, 2, 6, 3, 1, 2, 5, 1, 3, 1, 9]


def test_kat8(oracle):
    for mode in (oracle.HEAP_SCAN, oracle.HEAP_POSMAP):
        found, cost, path, _, _ = oracle.astar(8, KAT_OFF, KAT_COL, KAT_W, [0] * 8, 0, 7, mode=mode)
        assert found and cost == 6
        assert path.tolist() == [0, 2, 4, 6, 7]


def test_golden_vectors(oracle, golden):
    """Every golden case: both heap modes reproduce the reference binary's
    cost and exact path (same pops, same tie-breaks)."""
    assert len(golden) >= 10
    for name, c in golden.items():
        if name == "lib_main":
            continue
        n = int(c["n"])
        for mode in (oracle.HEAP_SCAN, oracle.HEAP_POSMAP):
            found, cost, path, _, _ = oracle.astar(n, c["off"], c["col"], c["w"], c["h"], int(c["s"]),
                                                   int(c["t"]), mode=mode)
            if int(c["cost"]) < 0:
                assert not found, name
                continue
            assert found and cost == int(c["cost"]), name
            assert path.tolist() == c["path"].tolist(), name


def test_lib_main_golden(golden):
    # LIB/main.cpp (CPU A_Star<unsigned,int>) on the 8-node graph
    assert golden["lib_main"]["path"].tolist() == [0, 2, 4, 6, 7]


def test_heap_modes_agree_on_random(oracle, ddp):
    for seed in range(4):
        g = ddp.gen_random_chain(3000, 6, 1, 100, 100 + seed).with_sentinel()
        h = np.maximum(oracle.bfs_heuristic(g.n, g.off[:-1], g.col, g.w, 2000 + seed), 0)
        a = oracle.astar(g.n, g.off[:-1], g.col, g.w, h, seed, 2000 + seed, mode=oracle.HEAP_SCAN)
        b = oracle.astar(g.n, g.off[:-1], g.col, g.w, h, seed, 2000 + seed, mode=oracle.HEAP_POSMAP)
        assert a[1] == b[1] and a[2].tolist() == b[2].tolist() and (a[3] == b[3]).all()


@pytest.mark.skipif(not __import__("os").path.exists(
    __import__("os").path.join(__import__("os").path.dirname(__file__), "..", "oracle", "_ref", "a_star_cpu")),
    reason="reference binary not built here")
def test_live_reference_binary(oracle, ddp):
    """Fresh seeded cases through the reference binary itself."""
    for seed in range(3):
        g = ddp.gen_random_chain(1000, 5, 1, 50, 500 + seed).with_sentinel()
        t = 900 - seed
        h = np.maximum(oracle.bfs_heuristic(g.n, g.off[:-1], g.col, g.w, t), 0)
        rc, rp = oracle.run_reference_astar(g.n, g.off[:-1], g.col, g.w, h, seed, t)
        f, c, p, _, _ = oracle.astar(g.n, g.off[:-1], g.col, g.w, h, seed, t)
        assert f and c == rc and p.tolist() == rp.tolist()


def _py_bfs(n, off, col, root):
    # independent BFS on the reverse graph
    rev = [[] for _ in range(n)]
    for u in range(n):
        for j in range(off[u], off[u + 1]):
            if col[j] >= 0:
                rev[col[j]].append(u)
    dist = [-1] * n
    dist[root] = 0
    q = [root]
    for u in q:
        for p in rev[u]:
            if dist[p] < 0:
                dist[p] = dist[u] + 1
                q.append(p)
    return dist


def test_bfs_restatement(oracle, ddp):
    g = ddp.gen_random_chain(800, 3, 1, 9, 31)
    roff, rcol, _ = oracle.reverse_csr(g.n, g.off[:-1], g.col, g.w)
    for root in (0, 17, 799):
        d = oracle.bfs_hops(g.n, roff, rcol, root)
        assert d.tolist() == _py_bfs(g.n, g.off, g.col, root)


def test_reverse_csr_matches_package(oracle, ddp):
    g = ddp.gen_random_chain(500, 4, 1, 20, 3)
    roff, rcol, rw = oracle.reverse_csr(g.n, g.off[:-1], g.col, g.w)
    r = g.reverse()
    assert roff.tolist() == r.off[:-1].tolist()
    assert rcol.tolist() == r.col.tolist() and rw.tolist() == r.w.tolist()


def test_apply_batch_semantics(oracle):
    # rows: 0:[1,2,1] 1:[2] 2:[]
    off = [0, 3, 4]
    col = [1, 2, 1, 2]
    w = [5, 6, 7, 8]
    # insert 0->2 (w 9), delete 0->1 (first live copy, w 5), delete 2->0 (absent),
    # set weight of 1->2 to 3
    flag = [1, 0, 0, 2]
    u = [0, 0, 2, 1]
    v = [2, 1, 0, 2]
    uw = [9, 0, 0, 3]
    noff, ncol, nw, nd = oracle.apply_batch(3, off, col, w, flag, u, v, uw)
    assert nd == 1
    assert noff.tolist() == [0, 3, 4]
    assert ncol.tolist() == [2, 1, 2, 2]
    assert nw.tolist() == [6, 7, 9, 3]
