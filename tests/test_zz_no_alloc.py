"""The allocation-free entry point (ddp_bfs_hops_noalloc).

It exists for callers that cannot let the library call cudaMalloc; it keeps
its scratch in a fixed array inside the library.  This file is named to be
collected last.  It checks, through the C-ABI, that two calls in a row give
the same hop counts as the oracle's reverse BFS and as the allocating
heuristic build (ddp_heuristic_build with DDP_H_BFS_HOPS on a graph whose
minimum weight is 1, so h = hops)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_bfs_matches_oracle_and_allocating_build(gpu, oracle):
    torch = pytest.importorskip("torch")
    d = gpu
    L = d.lib()
    # min weight 1; the appended isolated node cannot reach any target
    g = d.gen_random_chain(200_000, 3, 1, 50, 2718).with_sentinel()
    perm = d.gen_random_chain(200_000, 3, 1, 50, 2718).perm
    r = g.reverse()
    dev = torch.device("cuda", 0)
    roff = torch.from_numpy(r.off.astype(np.int32)).to(dev)
    rsrc = torch.from_numpy(r.col.astype(np.int32)).to(dev)
    hops = torch.full((g.n,), 7, dtype=torch.int32, device=dev)
    dg = d.DeviceGraph.from_csr(g)
    for target in (int(perm[len(perm) // 2]), int(perm[-1])):   # two calls in a row
        rc = L.ddp_bfs_hops_noalloc(g.n, C.c_void_p(roff.data_ptr()), C.c_void_p(rsrc.data_ptr()), target,
                                    C.c_void_p(hops.data_ptr()), None)
        assert rc == 0, L.ddp_last_error()
        got = hops.cpu().numpy()
        # the oracle's reverse BFS (hops, -1 = cannot reach the target)
        want = oracle.bfs_heuristic(g.n, g.off[:-1], g.col, g.w, target, wmin=1)
        bad = np.flatnonzero(got != want)
        assert bad.size == 0, f"{bad.size} mismatches, first {bad[:5]}: {got[bad[:5]]} vs {want[bad[:5]]}"
        alloc = dg.heuristic(target, d.H_BFS_HOPS, want_values=True).values
        assert np.array_equal(got, alloc)
        assert got[target] == 0 and got[g.n - 1] == -1


def test_noalloc_rejects_oversized_graph(gpu):
    L = gpu.lib()
    rc = L.ddp_bfs_hops_noalloc(2 * 1048576, C.c_void_p(1), C.c_void_p(1), 0, C.c_void_p(1), None)
    assert rc == 1 and b"DDP_NOALLOC_MAX_NODES" in L.ddp_last_error()
