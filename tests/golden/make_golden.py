"""Generates tests/golden/astar_ref.npz from the reference's own CPU A*.

Run where the reference tree exists (it is compiled into oracle/_ref by
`make -C oracle ref`):

    python tests/golden/make_golden.py

Each case stores its full input (graph in the reference's N-offset layout,
h, s, t) and the reference binary's output (cost, path), so the fixture does
not depend on this repository's generators.  The reference programs print
the cost and the path from target to source; the path is stored s..t.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import ddp_gb300 as d  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main():
    if not O.have_reference_binary():
        raise SystemExit("oracle/_ref/a_star_cpu missing: run `make -C oracle ref` where the reference exists")
    cases = {}

    def add(name, n, off_ref, col, w, h, s, t):
        cost, path = O.run_reference_astar(n, off_ref, col, w, h, s, t)
        cases[name] = dict(n=np.int32(n), off=np.asarray(off_ref, np.int32), col=np.asarray(col, np.int32),
                           w=np.asarray(w, np.uint32), h=np.asarray(h, np.int32), s=np.int32(s), t=np.int32(t),
                           cost=np.int32(-1 if cost is None else cost), path=path)

    # the 8-node hand-checkable graph (cost 6, path 0 2 4 6 7)
    add("kat8", 8, [0, 2, 3, 5, 7, 9, 10, 11], [1, 2, 3, 3, 4, 4, 5, 5, 6, 7, 7, 0],
        [4, 1, 2, 6, 3, 1, 2, 5, 1, 3, 1, 9], [0] * 8, 0, 7)
    # random chain graphs (C1 shape, small), BFS-hop heuristic, sentinel node
    for (n, deg, seed, s, t) in [(50, 3, 1, 0, 49), (300, 4, 2, 5, 200), (2000, 8, 3, 17, 1234),
                                 (8000, 8, 4, 4000, 7)]:
        g = d.gen_random_chain(n, deg, 1, 100, seed).with_sentinel()
        h = np.maximum(O.bfs_heuristic(g.n, g.off[:-1], g.col, g.w, t), 0)
        add(f"chain_n{n}_s{seed}", g.n, g.off[:-1], g.col, g.w, h, s, t)
        add(f"chain_n{n}_s{seed}_h0", g.n, g.off[:-1], g.col, g.w, np.zeros(g.n, np.int32), s, t)
    # zero-weight arcs (GA_star/randomGraph.py draws weights in [0,100])
    g = d.gen_random_chain(1500, 5, 0, 100, 9).with_sentinel()
    add("chain_w0", g.n, g.off[:-1], g.col, g.w, np.zeros(g.n, np.int32), 3, 1400)
    # maze (C2 shape, small), Manhattan heuristic; sentinel appended
    m = d.gen_maze(48, 64, 0.3, 13)
    mg = m.with_sentinel()
    tx, ty = m.xy[m.n - 1]
    hm = np.concatenate([np.abs(m.xy[:, 0] - tx) + np.abs(m.xy[:, 1] - ty), [0]]).astype(np.int32)
    add("maze48x64", mg.n, mg.off[:-1], mg.col, mg.w, hm, 0, m.n - 1)
    # unreachable target (sentinel node)
    g = d.gen_random_chain(400, 4, 1, 100, 21).with_sentinel()
    add("unreachable", g.n, g.off[:-1], g.col, g.w, np.zeros(g.n, np.int32), 0, g.n - 1)
    # no sentinel: the last node has arcs, and the reference skips its last one
    g = d.gen_random_chain(200, 4, 1, 100, 22)
    add("last_row_quirk", g.n, g.off[:-1], g.col, g.w, np.zeros(g.n, np.int32), int(g.perm[-2]),
        int(g.perm[0]))

    flat = {}
    for name, c in cases.items():
        for k, v in c.items():
            flat[f"{name}.{k}"] = v
    # LIB demo (LIB/main.cpp CPU half) on the 8-node graph: its last line is the path
    lines = O.run_reference_lib_main(8, [0, 2, 3, 5, 7, 9, 10, 11], [1, 2, 3, 3, 4, 4, 5, 5, 6, 7, 7, 0],
                                     [4, 1, 2, 6, 3, 1, 2, 5, 1, 3, 1, 9])
    flat["lib_main.path"] = np.array([int(x) for x in lines[-1].split()], np.int32)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "astar_ref.npz")
    np.savez_compressed(out, **flat)
    print(f"wrote {out}: {len(cases)} cases")
    for name, c in cases.items():
        print(f"  {name}: n={int(c['n'])} e={len(c['col'])} cost={int(c['cost'])} path_len={len(c['path'])}")


if __name__ == "__main__":
    main()
