"""Host-side product logic on the CPU: library exports, generators, text
I/O in the reference formats, LIB-mirror conventions that need no GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(ddp_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(ddp):
    declared = _declared_symbols()
    assert len(declared) > 30
    out = subprocess.run(["nm", "-D", "--defined-only", ddp._lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(ddp_[a-z0-9_]+)", out))
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    L = ctypes.CDLL(ddp._lib.LIB_PATH)
    for name in declared:
        getattr(L, name)


def test_ctypes_signatures_cover_header(ddp):
    assert _declared_symbols() <= set(ddp._lib.SIGNATURES)


def test_random_chain_properties(ddp):
    a = ddp.gen_random_chain(20000, 8, 1, 100, 42)
    b = ddp.gen_random_chain(20000, 8, 1, 100, 42)
    c = ddp.gen_random_chain(20000, 8, 1, 100, 43)
    assert np.array_equal(a.col, b.col) and np.array_equal(a.w, b.w) and np.array_equal(a.off, b.off)
    assert not np.array_equal(a.col, c.col)
    assert a.e == 160000 and a.off[0] == 0 and a.off[-1] == a.e
    src = np.repeat(np.arange(a.n), np.diff(a.off))
    assert not np.any(src == a.col)                      # no self loops
    keys = src.astype(np.int64) * a.n + a.col
    assert len(np.unique(keys)) == a.e                   # no duplicates
    assert a.w.min() >= 1 and a.w.max() <= 100
    assert sorted(a.perm.tolist()) == list(range(a.n))   # chain arcs exist
    chain = set((a.perm[:-1].astype(np.int64) * a.n + a.perm[1:]).tolist())
    assert chain <= set(keys.tolist())


def test_maze_properties(ddp):
    m = ddp.gen_maze(40, 50, 0.3, 5)
    cn = m.extra["cell_node"].reshape(40, 50)
    assert cn[0, 0] == 0 and cn[39, 49] == m.n - 1
    walls = (cn < 0).mean()
    assert 0.2 < walls < 0.4
    # arcs are between 4-neighbours and symmetric, unit weight
    src = np.repeat(np.arange(m.n), np.diff(m.off))
    d = np.abs(m.xy[src] - m.xy[m.col]).sum(1)
    assert (d == 1).all() and (m.w == 1).all()
    fwd = set((src.astype(np.int64) * m.n + m.col).tolist())
    assert all((int(v) * m.n + int(u)) in fwd for u, v in zip(src[:500], m.col[:500]))


def test_updates_model(ddp):
    g = ddp.gen_random_chain(3000, 10, 1, 1000, 9)
    fl, u, v, w = ddp.gen_updates(g, 5, 100, 50, 1, 1000, 17)
    assert (fl.reshape(5, 100)[:, :50] == 1).all() and (fl.reshape(5, 100)[:, 50:] == 0).all()
    live = set((np.repeat(np.arange(g.n), np.diff(g.off)).astype(np.int64) * g.n + g.col).tolist())
    chain = set((g.perm[:-1].astype(np.int64) * g.n + g.perm[1:]).tolist())
    for b in range(5):
        sl = slice(100 * b, 100 * b + 100)
        keys = (u[sl].astype(np.int64) * g.n + v[sl]).tolist()
        ins, dels = keys[:50], keys[50:]
        assert not (set(ins) & live)          # inserts are new arcs
        assert set(dels) <= live              # deletes hit live arcs
        assert not (set(dels) & chain)        # chain protected
        assert (u[sl] != v[sl]).all()
        live |= set(ins)
        live -= set(dels)


def test_pairs(ddp):
    g = ddp.gen_random_chain(20000, 8, 1, 100, 1)
    S, T, want = ddp.gen_pairs(g, 200, 4, 400, 77, threads=4)
    S2, T2, _ = ddp.gen_pairs(g, 200, 4, 400, 77, threads=1)
    assert np.array_equal(S, S2) and np.array_equal(T, T2)   # thread-count independent
    assert (want >= 4).all() and (want <= 400).all()
    assert ((S >= 0) & (S < g.n) & (T >= 0) & (T < g.n) & (S != T)).all()


def test_text_io_roundtrip(ddp, tmp_path):
    g = ddp.gen_random_chain(500, 4, 0, 100, 2)
    p = str(tmp_path / "graph.txt")
    ddp.write_graph_text(p, g)
    h = open(p).readline().split()
    assert h == ["500", "2000"]
    r = ddp.read_graph_text(p)
    assert r.n == g.n and np.array_equal(r.off, g.off) and np.array_equal(r.col, g.col)
    assert np.array_equal(r.w, g.w)
    hx = np.arange(500, dtype=np.int32) - 3
    ddp.write_ints_text(str(tmp_path / "Hx.txt"), hx)
    assert np.array_equal(ddp.read_ints_text(str(tmp_path / "Hx.txt"), 1000), hx)
    batches = [(np.array([1, 0], np.int32), np.array([3, 4], np.int32), np.array([5, 6], np.int32),
                np.array([7, 8], np.uint32)), (np.array([0], np.int32), np.array([1], np.int32),
                                               np.array([2], np.int32), np.array([9], np.uint32))]
    ddp.write_updates_text(str(tmp_path / "Updates.txt"), batches)
    assert open(tmp_path / "Updates.txt").read() == "2\n1 3 5 7\n0 4 6 8\n1\n0 1 2 9\n"
    rb = ddp.read_updates_text(str(tmp_path / "Updates.txt"))
    assert len(rb) == 2 and rb[0][1].tolist() == [3, 4] and rb[1][3].tolist() == [9]


def test_text_reader_rejects_truncated(ddp, tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("4 3\n1 2 3\n0 1\n")
    with pytest.raises(ddp.DdpError) as ei:
        ddp.read_graph_text(str(p))
    assert ei.value.code == 3  # DDP_ERR_IO
    with pytest.raises(ddp.DdpError):
        ddp.read_graph_text(str(tmp_path / "missing.txt"))


def test_lib_mirror_without_heuristic(ddp):
    g = ddp.Graph.from_csr(ddp.gen_random_chain(10, 2, 1, 5, 1))
    a = ddp.A_Star(ddp.Dynamic_Graph(g), 0, 5, 4)
    assert a.get_path() == [-1]   # a_star.h:198-201: h not set


def test_graph_validation_needs_no_gpu(ddp):
    # argument checks run before any device call
    L = ddp.lib()
    h = ctypes.c_void_p()
    off = np.array([0, 2, 1], np.int32)
    col = np.array([1, 0], np.int32)
    w = np.array([1, 1], np.uint32)
    rc = L.ddp_graph_from_csr(2, 2, ddp.ptr(off), 3, ddp.ptr(col), ddp.ptr(w, ctypes.c_uint32), ctypes.byref(h))
    assert rc == 1  # DDP_ERR_INVALID: offsets not ending at e
    assert b"offsets" in L.ddp_last_error()


def test_maze_moves_are_consistent(ddp, oracle):
    """Obstacle-move batches applied with the reference's batch semantics
    give exactly the maze of the final wall mask."""
    d = ddp
    rows, cols = 40, 50
    wall = d.maze_walls(rows, cols, 0.3, 5)
    g0 = d.grid_from_walls(rows, cols, wall)
    prot = np.zeros(rows * cols, np.uint8)
    prot[0] = prot[-1] = 1
    w2 = wall.copy()
    counts, fl, u, v, w = d.gen_maze_moves(rows, cols, w2, 6, 30, 9, prot)
    assert (w2 != wall).sum() > 0 and prot[w2.astype(bool)].sum() == 0
    off, col, ww = g0.off[:-1].copy(), g0.col.copy(), g0.w.copy()
    pos = 0
    for c in counts:
        sl = slice(pos, pos + c)
        pos += c
        off, col, ww, _ = oracle.apply_batch(len(off), off, col, ww, fl[sl], u[sl], v[sl], w[sl])
    g1 = d.grid_from_walls(rows, cols, w2)

    def rows_of(off_n, col, w):
        o = np.append(off_n, len(col))
        return [sorted((int(a), int(b)) for a, b in zip(col[o[i]:o[i + 1]], w[o[i]:o[i + 1]]) if a >= 0)
                for i in range(rows * cols)]

    assert rows_of(off, col, ww) == rows_of(g1.off[:-1], g1.col, g1.w)


def test_parallel_text_and_binary_io(ddp, tmp_path):
    """A graph large enough for several parse threads round-trips through the
    text format and the binary format; a truncated binary file is rejected."""
    d = ddp
    g = d.gen_random_chain(400_000, 8, 1, 1000, 77)  # ~30 MB of text: 4 chunks
    pt, pb = str(tmp_path / "g.txt"), str(tmp_path / "g.bin")
    d.write_graph_text(pt, g)
    d.write_graph_bin(pb, g)
    for r in (d.read_graph_text(pt), d.read_graph_bin(pb)):
        assert r.n == g.n and np.array_equal(r.off, g.off) and np.array_equal(r.col, g.col)
        assert np.array_equal(r.w, g.w)
    data = open(pb, "rb").read()
    open(pb, "wb").write(data[:-4])
    with pytest.raises(d.DdpError):
        d.read_graph_bin(pb)
