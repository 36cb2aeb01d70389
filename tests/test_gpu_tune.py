"""Autotuner: the options it returns run the batch engine with exact costs,
and every configuration it timed agreed on the costs (else it errors)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tuner_returns_working_options(gpu, oracle):
    d = gpu
    g = d.gen_random_chain(30000, 6, 1, 100, 81)
    dg = d.DeviceGraph.from_csr(g)
    dg.build_landmarks(8, seed=2)
    rng = np.random.default_rng(3)
    S = rng.integers(0, g.n, 200).astype(np.int32)
    T = rng.integers(0, g.n, 200).astype(np.int32)
    opts, qps, trials = d.tune_batch(dg, d.H_LANDMARK, S, T)
    assert qps > 0 and trials >= 6
    assert opts["group"] >= 1 and opts["block"] in (256, 512)
    cost, _ = d.BatchEngine(dg, d.H_LANDMARK, **opts).solve(S[:40], T[:40])
    gs = g.with_sentinel()
    for i in range(0, 40, 5):
        f, c, _, _, _ = oracle.astar(gs.n, gs.off[:-1], gs.col, gs.w, np.zeros(gs.n, np.int32), int(S[i]), int(T[i]))
        assert cost[i] == (c if f else d.INF)
