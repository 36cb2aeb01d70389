"""The device-pointer batch path (ddp_batch_solve_device), the call the
benchmark times.  Every cost of repeated CUDA-graph replays is checked
against the oracle and every path is validated; the replay is re-captured
when the graph's arrays or the landmark table change; a stale table is an
error; a query that outgrows its slot's queues reports cost -1."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INF = 2147483647


def _oracle_costs(O, g, S, T):
    """Reference A* (h = 0) on every pair; g without a sentinel (one is
    appended here, so the oracle's last-row quirk cannot drop an arc)."""
    gs = g.with_sentinel()
    cost, _, _, done = O.astar_many(gs.n, gs.off[:-1], gs.col, gs.w, S, T, hkind=0, mode=O.HEAP_POSMAP,
                                    threads=os.cpu_count() or 1, budget_s=1e9)
    assert done == len(S)
    return cost


def _pairs(n, k, seed):
    rng = np.random.default_rng(seed)
    S = rng.integers(0, n, k).astype(np.int32)
    T = rng.integers(0, n, k).astype(np.int32)
    T[:4] = S[:4]  # source == target
    return S, T


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.int32)).to(torch.device("cuda", 0))


def _check_all(d, O, be, g, S, T, dcost, dplen, want):
    cost = dcost.cpu().numpy()
    assert np.array_equal(cost, want), np.flatnonzero(cost != want)[:8]
    plen = dplen.cpu().numpy() if dplen is not None else None
    for i in range(len(S)):
        p = be.path(i)
        if want[i] == INF:
            assert len(p) == 0, i
            continue
        if plen is not None:
            assert len(p) == plen[i], i
        ok, why = O.check_path(g.off, g.col, g.w, p, int(S[i]), int(T[i]), int(cost[i]))
        assert ok, f"query {i}: {why}"


@pytest.mark.parametrize("kind", ["landmark8", "landmark16", "bfs_hops", "zero"])
def test_device_batch_replays_match_oracle(gpu, oracle, kind):
    torch = pytest.importorskip("torch")
    d = gpu
    g = d.gen_random_chain(30000, 8, 1, 100, 4242)
    dg = d.DeviceGraph.from_csr(g)
    hk = {"bfs_hops": d.H_BFS_HOPS, "zero": d.H_ZERO}.get(kind, d.H_LANDMARK)
    if hk == d.H_LANDMARK:
        dg.build_landmarks(16, seed=5, bits=int(kind[8:]))
    S, T = _pairs(g.n, 256, 17)
    want = _oracle_costs(oracle, g, S, T)
    be = d.BatchEngine(dg, hk, group=1)
    dS, dT = _dev(torch, S), _dev(torch, T)
    dcost = torch.full((len(S),), -7, dtype=torch.int32, device="cuda")
    dplen = torch.full((len(S),), -7, dtype=torch.int32, device="cuda")
    for rep in range(3):  # the first call captures, the next ones replay
        dcost.fill_(-7)
        be.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), dplen.data_ptr())
        be.sync()
        _check_all(d, oracle, be, g, S, T, dcost, dplen, want)
    # without a path-length array: paths are still readable
    dcost.fill_(-7)
    be.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), 0)
    be.sync()
    _check_all(d, oracle, be, g, S, T, dcost, None, want)
    be.close()
    dg.close()


def test_device_batch_recaptures_after_landmark_rebuild(gpu, oracle):
    torch = pytest.importorskip("torch")
    d = gpu
    g = d.gen_random_chain(20000, 6, 1, 100, 808)
    dg = d.DeviceGraph.from_csr(g)
    S, T = _pairs(g.n, 128, 23)
    want = _oracle_costs(oracle, g, S, T)
    dS, dT = _dev(torch, S), _dev(torch, T)
    dcost = torch.empty(len(S), dtype=torch.int32, device="cuda")
    dg.build_landmarks(8, seed=1, bits=16)
    be = d.BatchEngine(dg, d.H_LANDMARK, group=1)
    for count, bits, seed in ((8, 16, 1), (32, 8, 2), (16, 16, 3), (16, 16, 3)):
        if (count, bits, seed) != (8, 16, 1):
            dg.build_landmarks(count, seed=seed, bits=bits)  # the old table is freed
        for _ in range(2):
            dcost.fill_(-7)
            be.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), 0)
            be.sync()
            assert np.array_equal(dcost.cpu().numpy(), want), (count, bits)
    be.close()
    dg.close()


def test_device_batch_after_dynamic_update(gpu, oracle):
    """A dynamic update changes the graph's arrays (rows with explicit ends,
    moved rows): the zero-heuristic replay is re-captured and stays exact on
    the updated graph; the landmark engine refuses the stale table until it
    is rebuilt."""
    torch = pytest.importorskip("torch")
    d = gpu
    g = d.gen_random_chain(20000, 6, 1, 100, 909)
    dg = d.DeviceGraph.from_csr(g)
    dg.build_landmarks(16, seed=4, bits=8)
    S, T = _pairs(g.n, 128, 29)
    dS, dT = _dev(torch, S), _dev(torch, T)
    dcost = torch.empty(len(S), dtype=torch.int32, device="cuda")
    bz = d.BatchEngine(dg, d.H_ZERO, group=1)
    bl = d.BatchEngine(dg, d.H_LANDMARK, group=1)
    want0 = _oracle_costs(oracle, g, S, T)
    for be in (bz, bl):
        be.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), 0)
        be.sync()
        assert np.array_equal(dcost.cpu().numpy(), want0)
    # one batch: 3,000 cheap arcs out of a few sources (rows outgrow their
    # slack) and deletes of existing arcs
    rng = np.random.default_rng(31)
    src = np.repeat(np.arange(g.n, dtype=np.int32), np.diff(g.off))
    ins_u = np.repeat(S[4:10], 500).astype(np.int32)
    ins_v = rng.integers(0, g.n, len(ins_u)).astype(np.int32)
    ok = ins_u != ins_v
    ins_u, ins_v = ins_u[ok], ins_v[ok]
    dj = rng.choice(g.e, 300, replace=False)
    fl = np.concatenate([np.ones(len(ins_u), np.int32), np.zeros(len(dj), np.int32)])
    uu = np.concatenate([ins_u, src[dj]]).astype(np.int32)
    vv = np.concatenate([ins_v, g.col[dj]]).astype(np.int32)
    ww = np.concatenate([np.ones(len(ins_u), np.uint32), g.w[dj]]).astype(np.uint32)
    dyn = d.DynamicSearch(dg, int(S[10]), int(T[10]), d.H_ZERO)
    dyn.update(fl, uu, vv, ww)
    dyn.close()
    g2 = dg.read_csr()
    want1 = _oracle_costs(oracle, g2, S, T)
    assert not np.array_equal(want0, want1)  # the update changed some answers
    for _ in range(2):
        dcost.fill_(-7)
        bz.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), 0)
        bz.sync()
        assert np.array_equal(dcost.cpu().numpy(), want1)
    with pytest.raises(d.DdpError) as ei:
        bl.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), 0)
    assert ei.value.code == 1  # DDP_ERR_INVALID: stale landmark table
    dg.build_landmarks(16, seed=4, bits=8)
    dcost.fill_(-7)
    bl.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), 0)
    bl.sync()
    assert np.array_equal(dcost.cpu().numpy(), want1)
    for i in range(0, len(S), 9):
        if want1[i] != INF:
            ok, why = oracle.check_path(g2.off, g2.col, g2.w, bl.path(i), int(S[i]), int(T[i]), int(want1[i]))
            assert ok, why
    bz.close()
    bl.close()
    dg.close()


def test_device_batch_overflow_reports_minus_one(gpu, oracle):
    """Slots with tiny queues: the device path reports -1 for the queries
    that outgrew them and exact costs for the rest."""
    torch = pytest.importorskip("torch")
    d = gpu
    m = d.gen_maze(120, 160, 0.25, 9)
    dg = d.DeviceGraph.from_csr(m)
    rng = np.random.default_rng(3)
    S = rng.integers(0, m.n, 48).astype(np.int32)
    T = rng.integers(0, m.n, 48).astype(np.int32)
    T[:6] = np.minimum(S[:6] + 1, m.n - 1)  # some short queries fit
    want = _oracle_costs(oracle, m, S, T)
    be = d.BatchEngine(dg, d.H_MANHATTAN, grid=8, queue_cap=64)
    dS, dT = _dev(torch, S), _dev(torch, T)
    dcost = torch.empty(len(S), dtype=torch.int32, device="cuda")
    for _ in range(2):
        be.solve_device(len(S), dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), 0)
        be.sync()
        got = dcost.cpu().numpy()
        over = got == -1
        assert over.any()
        assert np.array_equal(got[~over], want[~over])
    be.close()
    dg.close()
