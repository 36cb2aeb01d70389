"""Generates the full-size cost fixtures (TEST INFRASTRUCTURE).

Every cost comes from the oracle (oracle/astar_oracle.c, the reference's
serial CPU A* restated and pinned to the reference binary by astar_ref.npz),
run on the CPU with no GPU.  The benchmark compares the GPU's answers for
the same seeded inputs against these files, every item, and checks the
input digests first, so a fixture never applies to other inputs.

    python tests/golden/make_fixtures.py [c4] [c3] [c2] [--threads N]

  c4_costs.npz  all 4,096 pairs of the batched workload: 4M-node random
                digraph (chain + uniform arcs, out-degree 8, w U[1,100],
                graph seed 4004), pairs seed 4400, hops log-uniform in
                [4,400]; graph and pairs from the oracle's own generators.
  c3_costs.npz  the dynamic workload: 1M-node random digraph (out-degree 10,
                w U[1,1000], seed 3003), s/t = the chain's ends, 100 batches
                x 1,000 updates (500 inserts, 500 deletes, seed 3303); the
                cost before the first batch and after every batch, each from
                scratch on the updated graph (the reference's own check:
                whole graph + GA* after each batch).  The update stream comes
                from the product's CPU generator (ddp_gen_updates).
  c2_cost.npz   the 2048 x 2048 maze (30 % walls, seed 2002) query
                (0,0) -> (2047,2047), Manhattan heuristic.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make_c4(threads):
    n, deg, wmin, wmax, gseed, pairs, lo, hi, pseed = 4_000_000, 8, 1, 100, 4004, 4096, 4, 400, 4400
    off, col, w, _ = O.gen_random_chain(n, deg, wmin, wmax, gseed)
    S, T, _ = O.gen_pairs(n, off, col, pairs, lo, hi, pseed)
    # reference layout with a sentinel row: n + 1 nodes, offsets = off (the
    # sentinel's row is empty, so the oracle's last-row bound drops nothing)
    t0 = time.time()
    cost, ss, _, done = O.astar_many(n + 1, off, col, w, S, T, hkind=0, mode=O.HEAP_POSMAP, threads=threads,
                                     budget_s=1e9)
    assert done == pairs
    print(f"c4: {pairs} queries in {time.time() - t0:.0f} s (mean search {ss.mean():.2f} s)", flush=True)
    np.savez_compressed(os.path.join(HERE, "c4_costs.npz"), costs=cost.astype(np.int32),
                        graph_digest=digest(off, col, w), pairs_digest=digest(S, T),
                        params=np.array([n, deg, wmin, wmax, gseed, pairs, lo, hi, pseed], np.int64))


def make_c3(threads):
    import ddp_gb300 as d
    n, deg, wmin, wmax, gseed, useed, nb, per, ins = 1_000_000, 10, 1, 1000, 3003, 3303, 100, 1000, 500
    off, col, w, perm = O.gen_random_chain(n, deg, wmin, wmax, gseed)
    g = d.CSR(n, off, col, w, perm=perm)
    fl, u, v, uw = d.gen_updates(g, nb, per, ins, wmin, wmax, useed)
    s, t = int(perm[0]), int(perm[-1])
    # sentinel node n (isolated), reference layout (n + 1 offsets)
    N = n + 1
    roff, rcol, rw = off.copy(), col.copy(), w.copy()
    costs = []
    t0 = time.time()

    def solve(o, c, ww):
        h = np.maximum(O.bfs_heuristic(N, o, c, ww, t), 0)
        found, cost, _, _, _ = O.astar(N, o, c, ww, h, s, t, mode=O.HEAP_POSMAP)
        return cost if found else O.INF

    costs.append(solve(roff, rcol, rw))
    for b in range(nb):
        sl = slice(b * per, (b + 1) * per)
        roff, rcol, rw, _ = O.apply_batch(N, roff, rcol, rw, fl[sl], u[sl], v[sl], uw[sl])
        costs.append(solve(roff, rcol, rw))
    print(f"c3: {nb} batches in {time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(os.path.join(HERE, "c3_costs.npz"), costs=np.array(costs, np.int32),
                        graph_digest=digest(off, col, w), updates_digest=digest(fl, u, v, uw),
                        params=np.array([n, deg, wmin, wmax, gseed, useed, nb, per, ins], np.int64))


def make_c2(threads):
    import ddp_gb300 as d
    rows, cols, wall, gseed = 2048, 2048, 0.30, 2002
    m = d.gen_maze(rows, cols, wall, gseed)
    t = m.n - 1
    tx, ty = m.xy[t]
    h = np.concatenate([np.abs(m.xy[:, 0] - tx) + np.abs(m.xy[:, 1] - ty), [0]]).astype(np.int32)
    ms = m.with_sentinel()
    found, cost, _, _, secs = O.astar(ms.n, ms.off[:-1], ms.col, ms.w, h, 0, t, mode=O.HEAP_POSMAP)
    assert found
    print(f"c2: cost {cost} in {secs:.3f} s", flush=True)
    np.savez_compressed(os.path.join(HERE, "c2_cost.npz"), cost=np.int32(cost),
                        graph_digest=digest(m.off, m.col, m.w),
                        params=np.array([rows, cols, int(wall * 1000), gseed], np.int64))


def main():
    p = argparse.ArgumentParser()
    p.add_argument("which", nargs="*", default=["c2", "c3", "c4"])
    p.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    a = p.parse_args()
    O.build()
    for k in a.which:
        {"c4": make_c4, "c3": make_c3, "c2": make_c2}[k](a.threads)


if __name__ == "__main__":
    main()
