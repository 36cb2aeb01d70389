"""Landmark (ALT) heuristic: the device-built distance table against scipy's
Dijkstra, h values against the ALT formula, and exact costs (single query
and batched) against the oracle, including graphs where many node pairs are
disconnected."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

UNR = 0x7FFFFFFF


def _scipy_dists(g, ids):
    sp = pytest.importorskip("scipy.sparse")
    cg = pytest.importorskip("scipy.sparse.csgraph")
    src = np.repeat(np.arange(g.n), np.diff(g.off))
    live = g.col >= 0
    # parallel arcs: keep the lightest (csr_matrix would add them)
    order = np.lexsort((g.w[live], g.col[live], src[live]))
    a, b, w = src[live][order], g.col[live][order], g.w[live][order].astype(np.float64)
    first = np.ones(len(a), bool)
    first[1:] = (a[1:] != a[:-1]) | (b[1:] != b[:-1])
    A = sp.csr_matrix((w[first], (a[first], b[first])), shape=(g.n, g.n))
    fw = cg.dijkstra(A, indices=ids)
    bw = cg.dijkstra(A.T.tocsr(), indices=ids)
    conv = lambda x: np.where(np.isfinite(x), np.round(x), UNR).astype(np.int64)
    return conv(fw), conv(bw)


def _scale(fw, bw, bits):
    """Smallest s with every finite floor(d / s) below the all-ones marker."""
    fin = np.concatenate([fw[fw != UNR], bw[bw != UNR]])
    top = (1 << bits) - 2
    return max(1, -(-int(fin.max()) // top)) if fin.size else 1


def _alt(fw, bw, t, s=1):
    """h(v) for target t from landmark distances (rows: landmarks) stored as
    q = floor(d / s): each term s (q_a - q_b) - (s - 1); -1 = cut."""
    n = fw.shape[1]
    h = np.zeros(n, np.int64)
    cut = np.zeros(n, bool)
    for F, B in zip(fw, bw):
        qF = np.where(F != UNR, F // s, UNR)
        qB = np.where(B != UNR, B // s, UNR)
        ok = (F[t] != UNR) & (F != UNR)
        h = np.where(ok, np.maximum(h, (qF[t] - qF) * s - (s - 1)), h)
        cut |= (F[t] == UNR) & (F != UNR)
        ok = (B != UNR) & (B[t] != UNR)
        h = np.where(ok, np.maximum(h, (qB - qB[t]) * s - (s - 1)), h)
        cut |= (B == UNR) & (B[t] != UNR)
    return np.where(cut, -1, h)


def _oracle(O, g, s, t):
    gs = g.with_sentinel()
    f, c, _, _, _ = O.astar(gs.n, gs.off[:-1], gs.col, gs.w, np.zeros(gs.n, np.int32), s, t)
    return c if f else 2147483647


@pytest.mark.parametrize("count,bits", [(4, 16), (16, 16), (32, 16), (8, 8), (32, 8), (64, 8)])
def test_landmark_table_and_values(gpu, count, bits):
    d = gpu
    # heavier arcs for 8-bit entries, so that the table needs a scale > 1
    g = d.gen_random_chain(3000, 4, 1, 50 if bits == 16 else 400, 71)
    dg = d.DeviceGraph.from_csr(g)
    ids = dg.build_landmarks(count, seed=3, bits=bits)
    assert len(set(ids.tolist())) == count
    fw, bw = _scipy_dists(g, ids)
    s = _scale(fw, bw, bits)
    if bits == 8:
        assert s > 1
    rng = np.random.default_rng(2)
    for t in rng.integers(0, g.n, 6):
        h = dg.heuristic(int(t), d.H_LANDMARK, want_values=True)
        assert np.array_equal(h.values.astype(np.int64), _alt(fw, bw, int(t), s))
        assert h.values[t] == 0


@pytest.mark.parametrize("bits", [16, 8])
def test_landmark_single_and_batch_exact(gpu, oracle, bits):
    d = gpu
    g = d.gen_random_chain(20000, 6, 1, 100, 72)
    dg = d.DeviceGraph.from_csr(g)
    dg.build_landmarks(8, seed=5, bits=bits)
    rng = np.random.default_rng(9)
    S = rng.integers(0, g.n, 48).astype(np.int32)
    T = rng.integers(0, g.n, 48).astype(np.int32)
    want = np.array([_oracle(oracle, g, int(s), int(t)) for s, t in zip(S, T)])
    for k in range(6):
        h = dg.heuristic(int(T[k]), d.H_LANDMARK)
        r = dg.solve(int(S[k]), int(T[k]), h)
        assert r.cost == want[k]
        ok, why = oracle.check_path(g.off, g.col, g.w, r.path, int(S[k]), int(T[k]), r.cost, 0)
        assert ok, why
    for group in (1, 4):
        be = d.BatchEngine(dg, d.H_LANDMARK, group=group)
        cost, _ = be.solve(S, T)
        assert np.array_equal(cost, want), group
        for i in range(0, 48, 11):
            ok, why = oracle.check_path(g.off, g.col, g.w, be.path(i), int(S[i]), int(T[i]), int(cost[i]), 0)
            assert ok, why


@pytest.mark.parametrize("bits", [16, 8])
def test_landmark_disconnected(gpu, oracle, bits):
    """Sparse random arcs (no chain): many pairs have no path; the cut rule
    must prune only nodes that cannot reach t."""
    d = gpu
    rng = np.random.default_rng(4)
    n, e = 4000, 5000
    a = rng.integers(0, n, e)
    b = rng.integers(0, n, e)
    keep = a != b
    a, b = a[keep], b[keep]
    order = np.argsort(a, kind="stable")
    a, b = a[order], b[order]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, a + 1, 1)
    off = np.cumsum(off).astype(np.int32)
    w = rng.integers(1, 30, len(b)).astype(np.uint32)
    g = d.CSR(n, off, b.astype(np.int32), w)
    dg = d.DeviceGraph.from_csr(g)
    dg.build_landmarks(8, seed=1, bits=bits)
    S = rng.integers(0, n, 64).astype(np.int32)
    T = rng.integers(0, n, 64).astype(np.int32)
    # plus pairs two arcs apart (reachable)
    u = np.flatnonzero(np.diff(off) > 0)[:200:25]
    mid = g.col[off[u]]
    far = np.array([g.col[off[m]] if off[m + 1] > off[m] else m for m in mid])
    S = np.concatenate([S, u]).astype(np.int32)
    T = np.concatenate([T, far]).astype(np.int32)
    want = np.array([_oracle(oracle, g, int(s), int(t)) for s, t in zip(S, T)])
    assert (want == d.INF).any() and (want != d.INF).any()
    cost, _ = d.BatchEngine(dg, d.H_LANDMARK, group=1).solve(S, T)
    assert np.array_equal(cost, want)


def test_landmark_table_goes_stale(gpu):
    d = gpu
    g = d.gen_random_chain(2000, 4, 1, 50, 73)
    dg = d.DeviceGraph.from_csr(g)
    dg.build_landmarks(4)
    dg.heuristic(5, d.H_LANDMARK).close()
    dyn = d.DynamicSearch(dg, 0, 5, d.H_ZERO)
    dyn.update([1], [0], [7], [1])
    with pytest.raises(d.DdpError):
        dg.heuristic(5, d.H_LANDMARK)
    dyn.close()
    dg.build_landmarks(4)  # rebuilt on the updated graph
    dg.heuristic(5, d.H_LANDMARK).close()


@pytest.mark.parametrize("bits", [16, 8])
def test_landmark_scaled_table_admissible(gpu, oracle, bits):
    """Weights up to 60,000 push distances past 16 (and 8) bits: the table
    stores floor(d / s); h must stay a lower bound of the true distance to t
    and costs stay exact."""
    d = gpu
    g = d.gen_random_chain(3000, 4, 20000, 60000, 74)
    dg = d.DeviceGraph.from_csr(g)
    ids = dg.build_landmarks(8, seed=4, bits=bits)
    lfw, _ = _scipy_dists(g, ids)
    assert lfw[lfw != UNR].max() > 65534  # the table needs a scale > 1
    rng = np.random.default_rng(6)
    for t in rng.integers(0, g.n, 4):
        h = dg.heuristic(int(t), d.H_LANDMARK, want_values=True).values.astype(np.int64)
        _, to_t = _scipy_dists(g, np.array([int(t)]))  # d(v, t) via the reverse graph
        dv = to_t[0]
        ok = dv != UNR
        assert (h[ok] <= dv[ok]).all() and (h[ok] >= 0).all()
        assert h[int(t)] == 0
    S = rng.integers(0, g.n, 24).astype(np.int32)
    T = rng.integers(0, g.n, 24).astype(np.int32)
    want = np.array([_oracle(oracle, g, int(s), int(t)) for s, t in zip(S, T)])
    cost, _ = d.BatchEngine(dg, d.H_LANDMARK, group=1).solve(S, T)
    assert np.array_equal(cost, want)


@pytest.mark.parametrize("n", [4003, 4002, 4001])
def test_slot_reuse_after_reset(gpu, oracle, n):
    """Few slots, many queries: every slot runs ~16 searches back to back, so
    each search starts from the reset of the previous one.  n % 4 != 0 puts
    the slots' state arrays off 32-byte boundaries, where the reset writes
    single words at the array ends and whole sectors inside."""
    d = gpu
    g = d.gen_random_chain(n, 5, 1, 60, 75)
    dg = d.DeviceGraph.from_csr(g)
    dg.build_landmarks(16, seed=2, bits=8)
    rng = np.random.default_rng(n)
    S = rng.integers(0, g.n, 64).astype(np.int32)
    T = rng.integers(0, g.n, 64).astype(np.int32)
    want = np.array([_oracle(oracle, g, int(s), int(t)) for s, t in zip(S, T)])
    be = d.BatchEngine(dg, d.H_LANDMARK, group=1, grid=4)
    for _ in range(2):
        cost, _ = be.solve(S, T)
        assert np.array_equal(cost, want)
    be.close()
