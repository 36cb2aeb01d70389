"""Serving (continuous batching with interleaved updates): every answer is
exact for the graph version it ran on, each request gives the same answer
alone and in the mix, and updates between requests are applied."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _geo(d, n, seed):
    g = d.gen_geometric(n, 6, 1 << 20, 1000, seed, 4)
    dg = d.DeviceGraph.from_csr(g)
    dg.set_euclid(d.euclid_rho_fp(g))
    return g, dg


def _oracle(O, g, s, t, rho_fp):
    n = g.n
    dx = g.xy[:, 0].astype(np.int64) - g.xy[t, 0]
    dy = g.xy[:, 1].astype(np.int64) - g.xy[t, 1]
    r = np.floor(np.sqrt((dx * dx + dy * dy).astype(np.float64))).astype(np.int64)
    # exact floor sqrt
    r -= (r * r > dx * dx + dy * dy)
    r += ((r + 1) * (r + 1) <= dx * dx + dy * dy)
    h = ((r * rho_fp) >> 16).astype(np.int32)
    gs = g.with_sentinel()
    hh = np.concatenate([h, [0]]).astype(np.int32)
    f, c, _, _, _ = O.astar(gs.n, gs.off[:-1], gs.col, gs.w, hh, s, t)
    return c if f else 2147483647


def test_serving_mix_equals_alone_and_oracle(gpu, oracle):
    d = gpu
    g, dg = _geo(d, 50_000, 31)
    rho = d.euclid_rho_fp(g)
    srv = d.Server(dg, d.H_EUCLID, max_requests=4096, grid=64)
    rng = np.random.default_rng(1)
    S = rng.integers(0, g.n, 300).astype(np.int32)
    T = rng.integers(0, g.n, 300).astype(np.int32)
    # arrivals in waves while earlier requests are still running
    for i in range(0, 300, 50):
        srv.submit(S[i:i + 50], T[i:i + 50])
        time.sleep(0.001)
    ids, costs, lat, ver = srv.drain()
    order = np.argsort(ids)
    ids, costs = ids[order], costs[order]
    assert ids.tolist() == list(range(300))
    for i in range(0, 300, 23):
        h = dg.heuristic(int(T[i]), d.H_EUCLID)
        alone = dg.solve(int(S[i]), int(T[i]), h).cost
        h.close()
        assert costs[i] == alone == _oracle(oracle, g, int(S[i]), int(T[i]), rho), i
    st = srv.stats()
    assert st["completed"] == 300 and st["slots"] >= 1
    srv.close()


@pytest.mark.parametrize("nver,rounds", [(8, 4), (2, 8)])
def test_serving_with_updates(gpu, oracle, nver, rounds):
    """Weight changes, deletes and inserts between requests while searches
    run (the graph ring is reused when rounds >= versions): each answer
    equals the oracle on the graph version it reports."""
    d = gpu
    g, dg = _geo(d, 20_000, 41)
    srv = d.Server(dg, d.H_EUCLID, max_requests=4096, versions=nver, grid=32)
    srv.record_paths(8192)
    rng = np.random.default_rng(5)
    versions = [(g.off.copy(), g.col.copy(), g.w.copy(), d.euclid_rho_fp(g))]
    off, col, w = g.off[:-1].copy(), g.col.copy(), g.w.copy()
    submitted = []
    for rnd in range(rounds):
        S = rng.integers(0, g.n, 40).astype(np.int32)
        T = rng.integers(0, g.n, 40).astype(np.int32)
        srv.submit(S, T)
        submitted += list(zip(S.tolist(), T.tolist()))
        # an update batch: 30 weight changes x[0.5,2], 5 deletes, 5 inserts between neighbours
        src = np.repeat(np.arange(len(off)), np.diff(np.append(off, len(col))))
        live = np.flatnonzero(col >= 0)
        pick = rng.choice(live, 40, replace=False)
        fl, uu, vv, ww = [], [], [], []
        for j in pick[:30]:
            fl.append(2); uu.append(int(src[j])); vv.append(int(col[j]))
            ww.append(max(1, int(round(w[j] * rng.uniform(0.5, 2.0)))))
        for j in pick[30:35]:
            fl.append(0); uu.append(int(src[j])); vv.append(int(col[j])); ww.append(0)
        for j in pick[35:40]:
            a, b = int(col[j]), int(src[j])
            fl.append(1); uu.append(a); vv.append(b); ww.append(int(w[j]))
        srv.update(fl, uu, vv, ww)
        off, col, w, _ = oracle.apply_batch(len(off), off, col, w, fl, uu, vv, ww)
        gg = d.CSR(g.n, np.append(off, len(col)).astype(np.int32), col, w, xy=g.xy)
        versions.append((gg.off, gg.col, gg.w, d.euclid_rho_fp(gg)))
    ids, costs, lat, ver = srv.drain()
    assert len(ids) == len(submitted)
    for k in range(0, len(ids), 7):
        i = int(ids[k])
        s_, t_ = submitted[i]
        vo, vc, vw, vrho = versions[int(ver[k])]
        # the server's scale is a lower bound of every version's own rho
        gv = d.CSR(g.n, vo, vc, vw, xy=g.xy)
        want = _oracle(oracle, gv, s_, t_, 0)  # h = 0: the cost does not depend on h
        assert costs[k] == want, (i, int(ver[k]))
        if want != d.INF:  # the path is one of that version's graph
            ok, why = oracle.check_path(vo, vc, vw, srv.path(i), s_, t_, int(costs[k]))
            assert ok, (i, int(ver[k]), why)
    assert srv.stats()["version"] == rounds
    srv.close()


def test_serving_through_relayouts(gpu, oracle):
    """Insert batches large enough to exhaust the arc reserve: the master
    graph is laid out again and the version buffers take full copies (on the
    service CTA when the kernel runs).  Requests around the batches stay
    exact for the version they report."""
    d = gpu
    g, dg = _geo(d, 5000, 43)
    srv = d.Server(dg, d.H_EUCLID, max_requests=8192, versions=3, grid=16)
    rng = np.random.default_rng(8)
    versions = [(g.off.copy(), g.col.copy(), g.w.copy())]
    off, col, w = g.off[:-1].copy(), g.col.copy(), g.w.copy()
    submitted = []
    for rnd in range(4):
        S = rng.integers(0, g.n, 60).astype(np.int32)
        T = rng.integers(0, g.n, 60).astype(np.int32)
        srv.submit(S, T)
        submitted += list(zip(S.tolist(), T.tolist()))
        # 70k new arcs between random pairs, weights from the length scale (heavy, so
        # the Euclidean scale stays) plus a few light ones (the scale drops)
        k = 70_000
        a = rng.integers(0, g.n, k)
        b = rng.integers(0, g.n, k)
        keep = a != b
        a, b = a[keep], b[keep]
        ww = rng.integers(5_000, 50_000, len(a)).astype(np.uint32)
        ww[:20] = 1
        fl = np.ones(len(a), np.int32)
        srv.update(fl, a.astype(np.int32), b.astype(np.int32), ww)
        off, col, w, _ = oracle.apply_batch(len(off), off, col, w, fl, a, b, ww)
        versions.append((np.append(off, len(col)).astype(np.int32), col.copy(), w.copy()))
    ids, costs, lat, ver = srv.drain()
    assert len(ids) == len(submitted)
    for k in range(0, len(ids), 5):
        i = int(ids[k])
        s_, t_ = submitted[i]
        vo, vc, vw = versions[int(ver[k])]
        gv = d.CSR(g.n, vo, vc, vw, xy=g.xy)
        assert costs[k] == _oracle(oracle, gv, s_, t_, 0), (i, int(ver[k]))
    assert srv.stats()["version"] == 4
    srv.close()


@pytest.mark.parametrize("count,bits", [(8, 16), (16, 8)])
def test_serving_with_landmarks_on_a_fixed_graph(gpu, oracle, count, bits):
    """Landmark serving (the 4M-node batch heuristic in continuous
    batching), 16- and 8-bit tables: exact answers; updates are refused,
    since they would void the landmark bounds."""
    d = gpu
    g = d.gen_random_chain(20000, 6, 1, 100, 57)
    dg = d.DeviceGraph.from_csr(g)
    dg.build_landmarks(count, seed=1, bits=bits)
    srv = d.Server(dg, d.H_LANDMARK, max_requests=4096, grid=32)
    rng = np.random.default_rng(2)
    S = rng.integers(0, g.n, 100).astype(np.int32)
    T = rng.integers(0, g.n, 100).astype(np.int32)
    first = srv.submit(S, T)
    ids, costs, _, _ = srv.drain()
    gs = g.with_sentinel()
    for k in range(0, len(ids), 9):
        i = int(ids[k]) - first
        f, c, _, _, _ = oracle.astar(gs.n, gs.off[:-1], gs.col, gs.w, np.zeros(gs.n, np.int32), int(S[i]), int(T[i]))
        assert costs[k] == (c if f else d.INF)
    with pytest.raises(d.DdpError):
        srv.update([1], [0], [5], [1])
    srv.close()


def test_serving_paths(gpu, oracle):
    """Recorded paths (ddp_serve_record_paths): every polled request's path is
    an s..t path of its reported cost, for Euclidean A* and bidirectional
    slots; asking before the poll, recording after the first submit, or a
    path longer than the capacity is an error."""
    d = gpu
    g, dg = _geo(d, 30_000, 51)
    for hk in (d.H_EUCLID, d.H_BIDIR):
        srv = d.Server(dg, hk, max_requests=1024, grid=32)
        srv.record_paths(4096)
        rng = np.random.default_rng(7)
        S = rng.integers(0, g.n, 120).astype(np.int32)
        T = rng.integers(0, g.n, 120).astype(np.int32)
        T[:3] = S[:3]
        first = srv.submit(S, T)
        with pytest.raises(d.DdpError):
            srv.record_paths(4096)
        with pytest.raises(d.DdpError):
            srv.path(first)  # not polled yet
        ids, costs, lat, ver = srv.drain()
        assert len(ids) == 120
        for k in range(len(ids)):
            i = int(ids[k]) - first
            p = srv.path(int(ids[k]))
            if costs[k] == d.INF:
                assert len(p) == 0, i
                continue
            ok, why = oracle.check_path(g.off, g.col, g.w, p, int(S[i]), int(T[i]), int(costs[k]))
            assert ok, (hk, i, why)
        srv.close()
    srv = d.Server(dg, d.H_EUCLID, max_requests=64, grid=8)
    srv.record_paths(2)
    rng = np.random.default_rng(8)
    S = rng.integers(0, g.n, 20).astype(np.int32)
    T = rng.integers(0, g.n, 20).astype(np.int32)
    srv.submit(S, T)
    ids, costs, _, _ = srv.drain()
    fin = [(int(c), int(i)) for i, c in zip(ids, costs) if c != d.INF]
    assert fin
    with pytest.raises(d.DdpError):
        srv.path(max(fin)[1])  # the costliest random pair: far more than two nodes
    srv.close()
