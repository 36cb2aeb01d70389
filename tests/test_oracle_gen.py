"""The oracle's generators (oracle/gen_oracle.c) against the product's
(ddp_gen_random_chain, ddp_gen_pairs): the same bytes for the same
arguments.  The benchmark's reference arm and the fixture scripts build
their inputs with the oracle's, so that they never load the product
library; this equality makes their workloads the product's workloads."""
import numpy as np
import pytest


@pytest.mark.parametrize("n,deg,wmin,wmax,seed", [(3, 1, 1, 1, 1), (1000, 3, 1, 100, 7), (50_000, 8, 1, 100, 4004),
                                                  (20_000, 10, 1, 1000, 3003)])
def test_random_chain_identical(ddp, oracle, n, deg, wmin, wmax, seed):
    g = ddp.gen_random_chain(n, deg, wmin, wmax, seed)
    off, col, w, perm = oracle.gen_random_chain(n, deg, wmin, wmax, seed)
    assert np.array_equal(g.off, off) and np.array_equal(g.col, col)
    assert np.array_equal(g.w, w) and np.array_equal(g.perm, perm)


@pytest.mark.parametrize("npairs,lo,hi,cap", [(300, 4, 400, 6), (64, 1, 3, 6), (64, 2, 9, 0)])
def test_pairs_identical(ddp, oracle, npairs, lo, hi, cap):
    g = ddp.gen_random_chain(30_000, 8, 1, 100, 4004)
    S, T, want = ddp.gen_pairs(g, npairs, lo, hi, 4400, bfs_cap_level=cap, threads=3)
    S2, T2, want2 = oracle.gen_pairs(g.n, g.off, g.col, npairs, lo, hi, 4400, bfs_cap_level=cap, threads=5)
    assert np.array_equal(S, S2) and np.array_equal(T, T2) and np.array_equal(want, want2)
    assert (S != T).all()
