"""ddp_gb300: GA* and dynamic A* on int32 CSR graphs for GB300 (sm_103a).

Python host mirror of the C-ABI in include/ddp_gb300.h.  Every compute call
goes to libddp_gb300.so; there is no CPU fallback — if the library or the
GPU is missing the calls raise.

Two layers:
  * functional API: DeviceGraph, Heuristic, BatchEngine, DynamicSearch and
    the generators / text I/O;
  * LIB mirror: Graph, GPU_Graph, Dynamic_Graph, GPU_Dynamic_Graph, A_Star,
    GPU_A_Star with the reference's names and return conventions
    (lkoshale/DDP LIB/include/graph.h, dynamic_graph.h, a_star.h, a_star.cuh):
    get_path() returns [-1] when no heuristic was set, [] when the target is
    unreachable, else the node ids source..target.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from ._lib import DdpError, Opts, check, lib, ptr  # noqa: F401

H_ZERO, H_BFS_HOPS, H_MANHATTAN, H_USER, H_BFS_CAPPED, H_EUCLID, H_LANDMARK, H_BIDIR = 0, 1, 2, 3, 4, 5, 6, 7
H_BIDIR_EUCLID, H_BIDIR_MANHATTAN = 8, 9
INF = 2147483647
# per-query counters: expanded, scanned, relaxed, phases, bfs_reached,
# bfs_scanned, far_scanned, touched
STATS = 8

__all__ = [
    "CSR", "DeviceGraph", "Heuristic", "SolveResult", "BatchEngine", "DdpError", "INF",
    "H_ZERO", "H_BFS_HOPS", "H_MANHATTAN", "H_USER", "H_BFS_CAPPED", "H_EUCLID", "gen_geometric",
    "euclid_rho_fp", "gen_random_chain", "gen_maze",
    "gen_updates", "gen_pairs", "read_graph_text", "write_graph_text", "read_ints_text",
    "write_ints_text", "read_updates_text", "write_updates_text", "Graph", "GPU_Graph",
    "Dynamic_Graph", "GPU_Dynamic_Graph", "A_Star", "GPU_A_Star", "DynamicSearch", "Server",
]


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


# ---------------------------------------------------------------------------
# host CSR container
@dataclass
class CSR:
    """Host CSR with n+1 offsets (off[n] = e).  col < 0 marks a dead arc."""
    n: int
    off: np.ndarray
    col: np.ndarray
    w: np.ndarray
    xy: Optional[np.ndarray] = None      # (n, 2) int32 coordinates
    perm: Optional[np.ndarray] = None    # Hamiltonian chain order (generators)
    extra: dict = field(default_factory=dict)

    @property
    def e(self) -> int:
        return int(self.off[-1])

    def row(self, u: int):
        return self.col[self.off[u]:self.off[u + 1]], self.w[self.off[u]:self.off[u + 1]]

    def reverse(self) -> "CSR":
        """Reverse CSR (sources of arcs into v, increasing source order)."""
        live = self.col >= 0
        src = np.repeat(np.arange(self.n, dtype=np.int32), np.diff(self.off))[live]
        dst = self.col[live]
        ww = self.w[live]
        order = np.lexsort((np.arange(len(dst)), dst))
        roff = np.zeros(self.n + 1, dtype=np.int32)
        np.add.at(roff, dst + 1, 1)
        roff = np.cumsum(roff, dtype=np.int64).astype(np.int32)
        return CSR(self.n, roff, _i32(src[order]), _u32(ww[order]))

    def with_sentinel(self) -> "CSR":
        """Appends an isolated node n (the reference CPU A* reads the last
        row only up to e-1, GA_star/A_star_cpu.cpp:170; a sentinel last row
        makes that harmless)."""
        off = np.concatenate([self.off, [self.off[-1]]]).astype(np.int32)
        return CSR(self.n + 1, off, self.col, self.w)

    def protect_next(self) -> Optional[np.ndarray]:
        """next[u] = chain successor of u (or -1), from the generator's perm."""
        if self.perm is None:
            return None
        nxt = np.full(self.n, -1, dtype=np.int32)
        nxt[self.perm[:-1]] = self.perm[1:]
        return nxt


# ---------------------------------------------------------------------------
# generators (seeded; ddp_gen_* in csrc/gen.c)
def gen_random_chain(n: int, avg_deg: int, wmin: int, wmax: int, seed: int) -> CSR:
    """Directed graph: Hamiltonian chain over a seeded permutation, then
    uniform extra arcs (no self-loops, no duplicates) up to n*avg_deg arcs,
    weights uniform in [wmin, wmax]."""
    e = int(n) * int(avg_deg)
    off = np.empty(n + 1, np.int32)
    col = np.empty(e, np.int32)
    w = np.empty(e, np.uint32)
    perm = np.empty(n, np.int32)
    rc = lib().ddp_gen_random_chain(n, e, wmin, wmax, seed, ptr(off), ptr(col), ptr(w, C.c_uint32), ptr(perm))
    if rc:
        raise DdpError(rc, "ddp_gen_random_chain failed")
    return CSR(n, off, col, w, perm=perm)


def gen_maze(rows: int, cols: int, wall_p: float, seed: int) -> CSR:
    """4-connected grid, walls with probability wall_p, a carved monotone
    corridor (0,0) -> (rows-1, cols-1), unit weights.  extra['cell_node']
    maps cells to node ids (-1 = wall)."""
    cells = rows * cols
    cell_node = np.empty(cells, np.int32)
    off = np.empty(cells + 1, np.int32)
    col = np.empty(4 * cells, np.int32)
    w = np.empty(4 * cells, np.uint32)
    xy = np.empty(2 * cells, np.int32)
    nn = C.c_int32()
    ne = C.c_int64()
    rc = lib().ddp_gen_maze(rows, cols, int(round(wall_p * 1000)), seed, ptr(cell_node), C.byref(nn),
                            C.byref(ne), ptr(off), ptr(col), ptr(w, C.c_uint32), ptr(xy))
    if rc:
        raise DdpError(rc, "ddp_gen_maze failed")
    n, e = nn.value, ne.value
    g = CSR(n, off[:n + 1].copy(), col[:e].copy(), w[:e].copy(), xy=xy[:2 * n].reshape(n, 2).copy())
    g.extra["cell_node"] = cell_node
    g.extra["shape"] = (rows, cols)
    return g


def maze_walls(rows: int, cols: int, wall_p: float, seed: int) -> np.ndarray:
    """The wall mask of gen_maze(rows, cols, wall_p, seed) (uint8, 1 = wall)."""
    return (gen_maze(rows, cols, wall_p, seed).extra["cell_node"] < 0).astype(np.uint8)


def grid_from_walls(rows: int, cols: int, wall: np.ndarray) -> CSR:
    """Maze with every cell a node (walls have no arcs), the reference's
    maze/create_maze.cpp layout; xy = (col, row)."""
    cells = rows * cols
    wall = np.ascontiguousarray(wall, np.uint8)
    off = np.empty(cells + 1, np.int32)
    col = np.empty(4 * cells, np.int32)
    w = np.empty(4 * cells, np.uint32)
    ne = C.c_int64()
    rc = lib().ddp_gen_grid_from_walls(rows, cols, wall.ctypes.data_as(C.POINTER(C.c_uint8)), ptr(off),
                                       ptr(col), ptr(w, C.c_uint32), C.byref(ne))
    if rc:
        raise DdpError(rc, "ddp_gen_grid_from_walls failed")
    e = ne.value
    idx = np.arange(cells, dtype=np.int32)
    xy = np.stack([idx % cols, idx // cols], axis=1).astype(np.int32)
    return CSR(cells, off, col[:e].copy(), w[:e].copy(), xy=xy)


def gen_maze_moves(rows: int, cols: int, wall: np.ndarray, nbatches: int, moves: int, seed: int,
                   protect: Optional[np.ndarray] = None):
    """Obstacle-move batches (ddp_gen_maze_moves); updates `wall` in place.
    Returns (counts, flag, u, v, w)."""
    assert wall.dtype == np.uint8 and wall.flags["C_CONTIGUOUS"]
    cap = max(1, 16 * moves * nbatches)
    counts = np.empty(max(nbatches, 1), np.int32)
    flag = np.empty(cap, np.int32)
    u = np.empty(cap, np.int32)
    v = np.empty(cap, np.int32)
    w = np.empty(cap, np.uint32)
    tot = C.c_int64()
    pr = None if protect is None else np.ascontiguousarray(protect, np.uint8)
    u8 = C.POINTER(C.c_uint8)
    rc = lib().ddp_gen_maze_moves(rows, cols, wall.ctypes.data_as(u8), None if pr is None else pr.ctypes.data_as(u8),
                                  nbatches, moves, seed, ptr(counts), ptr(flag), ptr(u), ptr(v),
                                  ptr(w, C.c_uint32), cap, C.byref(tot))
    if rc:
        raise DdpError(rc, "ddp_gen_maze_moves failed")
    k = tot.value
    return counts[:nbatches].copy(), flag[:k].copy(), u[:k].copy(), v[:k].copy(), w[:k].copy()


def gen_updates(g: CSR, nbatches: int, per_batch: int, inserts_per_batch: int, wmin: int, wmax: int,
                seed: int, protect_next: Optional[np.ndarray] = None):
    """Update batches in the Updates.txt model: per batch, `inserts_per_batch`
    inserts of arcs absent from the pre-batch graph, then deletes drawn
    uniformly over live unprotected arcs.  Returns (flag, u, v, w) arrays of
    nbatches*per_batch entries."""
    m = nbatches * per_batch
    flag = np.empty(m, np.int32)
    u = np.empty(m, np.int32)
    v = np.empty(m, np.int32)
    w = np.empty(m, np.uint32)
    pn = protect_next if protect_next is not None else g.protect_next()
    rc = lib().ddp_gen_updates(g.n, g.e, ptr(g.off), ptr(g.col), ptr(g.w, C.c_uint32),
                               ptr(_i32(pn)) if pn is not None else None, nbatches, per_batch,
                               inserts_per_batch, wmin, wmax, seed, ptr(flag), ptr(u), ptr(v),
                               ptr(w, C.c_uint32))
    if rc:
        raise DdpError(rc, "ddp_gen_updates failed")
    return flag, u, v, w


def gen_geometric(n: int, k: int = 6, side: int = 1 << 20, wscale: int = 1000, seed: int = 5005,
                  threads: int = 0) -> CSR:
    """Points uniform on an integer grid [0, side)^2, each joined both ways to
    its k nearest neighbours; w = max(1, round(wscale * length / spacing)),
    spacing = side / sqrt(n).  Returns a CSR with xy set."""
    xy = np.empty(2 * n, np.int32)
    off = np.empty(n + 1, np.int32)
    col = np.empty(2 * k * n, np.int32)
    w = np.empty(2 * k * n, np.uint32)
    m = C.c_int64()
    threads = threads or min(16, os.cpu_count() or 1)
    rc = lib().ddp_gen_geometric(n, k, side, wscale, seed, threads, ptr(xy), ptr(off), ptr(col),
                                 ptr(w, C.c_uint32), C.byref(m))
    if rc:
        raise DdpError(rc, "ddp_gen_geometric failed")
    e = m.value
    return CSR(n, off, col[:e].copy(), w[:e].copy(), xy=xy.reshape(n, 2))


def euclid_rho_fp(g: CSR) -> int:
    """Largest 16.16 fixed-point rho with rho <= w / length on every live arc
    (minus one unit of slack), the scale of the Euclidean heuristic."""
    live = g.col >= 0
    src = np.repeat(np.arange(g.n), np.diff(g.off))[live]
    dst = g.col[live]
    d = g.xy[dst].astype(np.float64) - g.xy[src].astype(np.float64)
    ln = np.sqrt((d * d).sum(1))
    ok = ln > 0
    rho = float((g.w[live][ok].astype(np.float64) / ln[ok]).min()) if ok.any() else 0.0
    return max(0, int(np.floor(rho * 65536.0)) - 1)


def gen_pairs(g: CSR, npairs: int, hop_lo: int, hop_hi: int, seed: int, bfs_cap_level: int = 6,
              threads: int = 0):
    """(S, T, wanted_hops): per pair a seeded source, a hop target drawn
    log-uniformly in [hop_lo, hop_hi]; targets up to bfs_cap_level hops are
    taken from a truncated BFS level, deeper ones uniformly at random."""
    S = np.empty(npairs, np.int32)
    T = np.empty(npairs, np.int32)
    want = np.empty(npairs, np.int32)
    threads = threads or min(16, os.cpu_count() or 1)
    rc = lib().ddp_gen_pairs(g.n, ptr(g.off), ptr(g.col), npairs, hop_lo, hop_hi, bfs_cap_level, seed,
                             threads, ptr(S), ptr(T), ptr(want))
    if rc:
        raise DdpError(rc, "ddp_gen_pairs failed")
    return S, T, want


# ---------------------------------------------------------------------------
# text I/O in the reference's formats
def read_graph_text(path: str, binary: bool = False) -> CSR:
    """Graph file in the reference's text format (parsed in parallel), or
    the binary format of write_graph_bin."""
    n = C.c_int32()
    e = C.c_int64()
    off = C.POINTER(C.c_int32)()
    col = C.POINTER(C.c_int32)()
    w = C.POINTER(C.c_uint32)()
    fn = lib().ddp_io_read_graph_bin if binary else lib().ddp_io_read_graph_text
    check(fn(path.encode(), C.byref(n), C.byref(e), C.byref(off), C.byref(col), C.byref(w)))
    try:
        N, E = n.value, e.value
        g = CSR(N, np.ctypeslib.as_array(off, (N + 1,)).copy(),
                np.ctypeslib.as_array(col, (max(E, 1),))[:E].copy(),
                np.ctypeslib.as_array(w, (max(E, 1),))[:E].copy())
    finally:
        for p in (off, col, w):
            lib().ddp_free(C.cast(p, C.c_void_p))
    return g


def read_graph_bin(path: str) -> CSR:
    return read_graph_text(path, binary=True)


def write_graph_bin(path: str, g: CSR) -> None:
    check(lib().ddp_io_write_graph_bin(path.encode(), g.n, g.e, ptr(_i32(g.off)), ptr(_i32(g.col)),
                                       ptr(_u32(g.w), C.c_uint32)))


def write_graph_text(path: str, g: CSR) -> None:
    check(lib().ddp_io_write_graph_text(path.encode(), g.n, g.e, ptr(_i32(g.off)), ptr(_i32(g.col)),
                                        ptr(_u32(g.w), C.c_uint32)))


def read_ints_text(path: str, max_count: int) -> np.ndarray:
    out = np.empty(max_count, np.int32)
    cnt = C.c_int64()
    check(lib().ddp_io_read_ints_text(path.encode(), max_count, ptr(out), C.byref(cnt)))
    return out[:cnt.value].copy()


def write_ints_text(path: str, vals) -> None:
    v = _i32(vals)
    check(lib().ddp_io_write_ints_text(path.encode(), len(v), ptr(v)))


def read_updates_text(path: str):
    """Returns a list of batches, each (flag, u, v, w) arrays."""
    nb = C.c_int32()
    cnt = C.POINTER(C.c_int32)()
    fl, uu, vv = C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)()
    ww = C.POINTER(C.c_uint32)()
    check(lib().ddp_io_read_updates_text(path.encode(), C.byref(nb), C.byref(cnt), C.byref(fl), C.byref(uu),
                                         C.byref(vv), C.byref(ww)))
    try:
        counts = np.ctypeslib.as_array(cnt, (max(nb.value, 1),))[:nb.value].copy()
        tot = int(counts.sum())
        arr = [np.ctypeslib.as_array(p, (max(tot, 1),))[:tot].copy() for p in (fl, uu, vv, ww)]
    finally:
        for p in (cnt, fl, uu, vv, ww):
            lib().ddp_free(C.cast(p, C.c_void_p))
    out, k = [], 0
    for c in counts:
        out.append(tuple(a[k:k + c] for a in arr))
        k += int(c)
    return out


def write_updates_text(path: str, batches) -> None:
    counts = _i32([len(b[0]) for b in batches])
    cat = [np.concatenate([b[i] for b in batches]) if batches else np.empty(0) for i in range(4)]
    check(lib().ddp_io_write_updates_text(path.encode(), len(counts), ptr(counts), ptr(_i32(cat[0])),
                                          ptr(_i32(cat[1])), ptr(_i32(cat[2])), ptr(_u32(cat[3]), C.c_uint32)))


# ---------------------------------------------------------------------------
# device objects
OPT_SYNC, OPT_ONE_CTA, OPT_HASH = 1, 2, 4


def _opts(K=0, delta=0, block=0, grid=0, queue_cap=0, stream=None, group=0, flags=0) -> Opts:
    """stream: a cudaStream_t as an int (e.g. torch's stream.cuda_stream);
    group: CTAs per query slot in the batch engine; flags: OPT_* bits."""
    return Opts(int(K), int(delta), int(block), int(grid), int(queue_cap), stream or None, int(group), int(flags))


@dataclass
class SolveResult:
    cost: int
    path: np.ndarray
    stats: np.ndarray  # expanded, scanned, relaxed, phases, bfs_reached, bfs_scanned

    @property
    def found(self) -> bool:
        return self.cost != INF


class Heuristic:
    def __init__(self, graph: "DeviceGraph", target: int, kind: int, user_h=None, want_values=False):
        self.graph, self.target, self.kind = graph, int(target), int(kind)
        self.values = np.empty(graph.n, np.int32) if want_values else None
        uh = _i32(user_h) if user_h is not None else None
        h = C.c_void_p()
        check(lib().ddp_heuristic_build(graph.handle, int(target), int(kind), ptr(uh), ptr(self.values),
                                        C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib().ddp_heuristic_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceGraph:
    """A graph uploaded to the GPU (ddp_graph)."""

    def __init__(self, handle: C.c_void_p, n: int, e: int):
        self.handle, self.n, self.e = handle, n, e

    @classmethod
    def from_csr(cls, g: CSR) -> "DeviceGraph":
        h = C.c_void_p()
        check(lib().ddp_graph_from_csr(g.n, g.e, ptr(_i32(g.off)), len(g.off), ptr(_i32(g.col)),
                                       ptr(_u32(g.w), C.c_uint32), C.byref(h)))
        dg = cls(h, g.n, g.e)
        if g.xy is not None:
            dg.set_coords(g.xy)
        return dg

    @classmethod
    def load_text(cls, path: str) -> "DeviceGraph":
        h = C.c_void_p()
        check(lib().ddp_graph_load_text(path.encode(), C.byref(h)))
        n = C.c_int32()
        e = C.c_int64()
        check(lib().ddp_graph_info(h, C.byref(n), C.byref(e), None, None))
        return cls(h, n.value, e.value)

    def set_coords(self, xy) -> None:
        a = _i32(np.asarray(xy).reshape(-1))
        check(lib().ddp_graph_set_coords(self.handle, ptr(a)))

    def set_euclid(self, rho_fp: int) -> None:
        check(lib().ddp_graph_set_euclid(self.handle, int(rho_fp)))

    def build_landmarks(self, count: int = 16, seed: int = 1, bits: int = 16) -> np.ndarray:
        """Landmark table for H_LANDMARK with `bits` (16 or 8) per entry;
        returns the landmark ids."""
        ids = np.empty(count, np.int32)
        check(lib().ddp_landmarks_build_bits(self.handle, int(count), int(bits), int(seed), ptr(ids)))
        return ids

    def info(self):
        n, e, lo, hi = C.c_int32(), C.c_int64(), C.c_uint32(), C.c_uint32()
        check(lib().ddp_graph_info(self.handle, C.byref(n), C.byref(e), C.byref(lo), C.byref(hi)))
        return dict(n=n.value, e=e.value, wmin=lo.value, wmax=hi.value)

    def read_csr(self) -> CSR:
        off = np.empty(self.n + 1, np.int32)
        check(lib().ddp_graph_read_csr(self.handle, ptr(off), None, None))
        e = int(off[-1])
        col = np.empty(e, np.int32)
        w = np.empty(e, np.uint32)
        check(lib().ddp_graph_read_csr(self.handle, None, ptr(col), ptr(w, C.c_uint32)))
        return CSR(self.n, off, col, w)

    def heuristic(self, target: int, kind: int = H_BFS_HOPS, user_h=None, want_values=False) -> Heuristic:
        return Heuristic(self, target, kind, user_h, want_values)

    def solve(self, s: int, t: int, heuristic: Optional[Heuristic] = None, **opts) -> SolveResult:
        q = C.c_void_p()
        o = _opts(**opts)
        check(lib().ddp_solve(self.handle, heuristic.handle if heuristic else None, int(s), int(t),
                              C.byref(o), C.byref(q)))
        try:
            cost = C.c_int32()
            check(lib().ddp_query_cost(q, C.byref(cost)))
            ln = C.c_int32()
            check(lib().ddp_path_read(q, None, 0, C.byref(ln)))
            path = np.empty(ln.value, np.int32)
            if ln.value:
                check(lib().ddp_path_read(q, ptr(path), ln.value, C.byref(ln)))
            st = np.empty(STATS, np.int64)
            check(lib().ddp_query_stats(q, st.ctypes.data_as(C.POINTER(C.c_int64))))
        finally:
            lib().ddp_query_free(q)
        return SolveResult(cost.value, path, st)

    def close(self):
        if self.handle:
            lib().ddp_graph_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchEngine:
    """Many (source, target) queries in one persistent kernel (ddp_batch)."""

    def __init__(self, graph: DeviceGraph, hkind: int = H_BFS_HOPS, **opts):
        self.graph = graph
        b = C.c_void_p()
        o = _opts(**opts)
        check(lib().ddp_batch_create(graph.handle, int(hkind), C.byref(o), C.byref(b)))
        self.handle = b
        self.n_last = 0

    def solve(self, S, T, cost=None, plen=None):
        """Host arrays in and out; cost / plen may be caller-owned int32
        arrays of len(S) (for example views of pinned host memory)."""
        S, T = _i32(S), _i32(T)
        n = len(S)
        cost = np.empty(n, np.int32) if cost is None else cost
        plen = np.empty(n, np.int32) if plen is None else plen
        assert cost.dtype == np.int32 and plen.dtype == np.int32 and len(cost) == n and len(plen) == n
        check(lib().ddp_batch_solve(self.handle, n, ptr(S), ptr(T), ptr(cost), ptr(plen)))
        self.n_last = n
        return cost, plen

    def solve_device(self, n: int, d_S: int, d_T: int, d_cost: int, d_plen: int = 0):
        """Device pointers (ints); stream-ordered, call sync() to wait."""
        check(lib().ddp_batch_solve_device(self.handle, int(n), C.c_void_p(d_S), C.c_void_p(d_T),
                                           C.c_void_p(d_cost), C.c_void_p(d_plen or None)))
        self.n_last = n

    def sync(self):
        check(lib().ddp_batch_sync(self.handle))

    def path(self, i: int) -> np.ndarray:
        ln = C.c_int32()
        check(lib().ddp_batch_path(self.handle, int(i), None, 0, C.byref(ln)))
        p = np.empty(max(ln.value, 0), np.int32)
        if ln.value > 0:
            check(lib().ddp_batch_path(self.handle, int(i), ptr(p), ln.value, C.byref(ln)))
        return p

    def stats(self):
        n = self.n_last
        st = np.empty(STATS * n, np.int64)
        t0 = np.empty(n, np.int64)
        t1 = np.empty(n, np.int64)
        P = C.POINTER(C.c_int64)
        check(lib().ddp_batch_stats(self.handle, st.ctypes.data_as(P), t0.ctypes.data_as(P),
                                    t1.ctypes.data_as(P)))
        return st.reshape(n, STATS), t0, t1

    def info(self):
        sl, cap, blk, grp = C.c_int32(), C.c_int64(), C.c_int32(), C.c_int32()
        check(lib().ddp_batch_info(self.handle, C.byref(sl), C.byref(cap), C.byref(blk)))
        check(lib().ddp_batch_group(self.handle, C.byref(grp)))
        return dict(slots=sl.value, queue_cap=cap.value, block=blk.value, group=grp.value)

    def launches(self) -> int:
        x = C.c_int32()
        check(lib().ddp_batch_launches(self.handle, C.byref(x)))
        return x.value

    def close(self):
        if self.handle:
            lib().ddp_batch_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_batch(graph: DeviceGraph, hkind: int, S, T, **base) -> tuple:
    """Autotuner (ddp_batch_tune): times the batch engine on the sample
    (S, T) and returns (options dict for BatchEngine, queries/s, trials)."""
    S, T = _i32(S), _i32(T)
    b = _opts(**base)
    o = Opts()
    q = C.c_double()
    n = C.c_int32()
    check(lib().ddp_batch_tune(graph.handle, int(hkind), len(S), ptr(S), ptr(T), C.byref(b), C.byref(o),
                               C.byref(q), C.byref(n)))
    return (dict(K=o.K, delta=o.delta, block=o.block, grid=o.grid, group=o.group, queue_cap=o.queue_cap), q.value,
            n.value)


def k_paths(graph: DeviceGraph, s: int, t: int, k: int, hkind: int = H_BFS_HOPS, restore: bool = True):
    """Up to k successive paths by last-arc deletion (ddp_kpaths, the
    reference's k-short method).  Returns [(cost, path)] for the paths found."""
    costs = np.empty(k, np.int32)
    offs = np.zeros(k + 1, np.int64)
    found = C.c_int32()
    cap = max(1024, 4 * k * 64)
    while True:
        buf = np.empty(cap, np.int32)
        rc = lib().ddp_kpaths(graph.handle, int(s), int(t), int(hkind), int(k), int(bool(restore)), ptr(costs),
                              ptr(buf), cap, offs.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(found))
        if rc == 0:
            break
        if offs[-1] > cap:  # buffer too small: the graph state was restored only if asked; retry larger
            if not restore:
                raise DdpError(rc, "path buffer too small (use restore=True to retry)")
            cap = int(offs[-1])
            continue
        check(rc)
    return [(int(costs[i]), buf[offs[i]:offs[i + 1]].copy()) for i in range(found.value)]


class DynamicSearch:
    """A resident A* search that follows edge-update batches (ddp_dyn):
    replaces DA_star/DA_dyn_cpu.cu.  The graph switches to growable rows."""

    def __init__(self, graph: DeviceGraph, source: int, target: int, hkind: int = H_BFS_HOPS, **opts):
        self.graph = graph
        o = _opts(**opts)
        h = C.c_void_p()
        check(lib().ddp_dyn_create(graph.handle, int(source), int(target), int(hkind), C.byref(o), C.byref(h)))
        self.handle = h

    @property
    def cost(self) -> int:
        c = C.c_int32()
        check(lib().ddp_dyn_cost(self.handle, C.byref(c)))
        return c.value

    def update(self, flag, u, v, w) -> int:
        """One batch: flag 1 insert, 0 delete, 2 set weight.  Returns the cost."""
        flag, u, v, w = _i32(flag), _i32(u), _i32(v), _u32(w)
        c = C.c_int32()
        check(lib().ddp_dyn_update(self.handle, len(flag), ptr(flag), ptr(u), ptr(v), ptr(w, C.c_uint32),
                                   C.byref(c)))
        return c.value

    def path(self) -> np.ndarray:
        ln = C.c_int32()
        check(lib().ddp_dyn_path(self.handle, None, 0, C.byref(ln)))
        p = np.empty(ln.value, np.int32)
        if ln.value:
            check(lib().ddp_dyn_path(self.handle, ptr(p), ln.value, C.byref(ln)))
        return p

    def stats(self) -> dict:
        st = np.empty(10, np.int64)
        check(lib().ddp_dyn_stats(self.handle, st.ctypes.data_as(C.POINTER(C.c_int64))))
        keys = ["cost", "path_len", "status", "phases", "invalidated", "reseeded", "relaxed", "hops_lowered",
                "expanded", "scanned"]
        return dict(zip(keys, st.tolist()))

    @property
    def grid(self) -> tuple:
        """(CTAs of the initial search, CTAs of each update batch)."""
        a, b = C.c_int32(), C.c_int32()
        check(lib().ddp_dyn_grid(self.handle, C.byref(a), C.byref(b)))
        return a.value, b.value

    def close(self):
        if self.handle:
            lib().ddp_dyn_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching A* service on a resident graph (ddp_server)."""

    def __init__(self, graph: DeviceGraph, hkind: int = H_EUCLID, max_requests: int = 1 << 20, versions: int = 8,
                 **opts):
        self.graph = graph
        o = _opts(**opts)
        h = C.c_void_p()
        check(lib().ddp_serve_create(graph.handle, int(hkind), C.byref(o), int(max_requests), int(versions),
                                     C.byref(h)))
        self.handle = h

    def submit(self, S, T) -> int:
        S, T = _i32(S), _i32(T)
        first = C.c_int64()
        check(lib().ddp_serve_submit(self.handle, len(S), ptr(S), ptr(T), C.byref(first)))
        return first.value

    def poll(self, max_results: int = 1 << 16):
        ids = np.empty(max_results, np.int64)
        costs = np.empty(max_results, np.int32)
        lat = np.empty(max_results, np.int64)
        ver = np.empty(max_results, np.int32)
        k = C.c_int32()
        P = C.POINTER(C.c_int64)
        check(lib().ddp_serve_poll(self.handle, max_results, ids.ctypes.data_as(P), ptr(costs),
                                   lat.ctypes.data_as(P), ptr(ver), C.byref(k)))
        n = k.value
        return ids[:n], costs[:n], lat[:n], ver[:n]

    def update(self, flag, u, v, w) -> None:
        flag, u, v, w = _i32(flag), _i32(u), _i32(v), _u32(w)
        check(lib().ddp_serve_update(self.handle, len(flag), ptr(flag), ptr(u), ptr(v), ptr(w, C.c_uint32)))

    def record_paths(self, path_cap: int) -> None:
        """Keep each request's path (at most path_cap nodes); before the first submit."""
        check(lib().ddp_serve_record_paths(self.handle, int(path_cap)))

    def path(self, request_id: int) -> np.ndarray:
        """s..t path of a polled request over the graph version it ran on
        (empty when t is unreachable)."""
        ln = C.c_int32()
        check(lib().ddp_serve_path(self.handle, int(request_id), None, 0, C.byref(ln)))
        p = np.empty(ln.value, np.int32)
        if ln.value:
            check(lib().ddp_serve_path(self.handle, int(request_id), ptr(p), ln.value, C.byref(ln)))
        return p

    def stats(self) -> dict:
        st = np.empty(6, np.int64)
        check(lib().ddp_serve_stats(self.handle, st.ctypes.data_as(C.POINTER(C.c_int64))))
        return dict(zip(["submitted", "completed", "slots", "launches", "version", "reruns"], st.tolist()))

    def drain(self, timeout_s: float = 60.0):
        """Polls until every submitted request is back; returns them."""
        import time as _t
        out = [[], [], [], []]
        t0 = _t.monotonic()
        while True:
            r = self.poll()
            for i in range(4):
                out[i].append(r[i])
            st = self.stats()
            if st["completed"] >= st["submitted"]:
                break
            if _t.monotonic() - t0 > timeout_s:
                raise TimeoutError("serving drain timed out")
            _t.sleep(0.0002)
        return tuple(np.concatenate(x) for x in out)

    def close(self):
        if self.handle:
            lib().ddp_serve_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


from .lib_mirror import (A_Star, Dynamic_Graph, GPU_A_Star, GPU_Dynamic_Graph, GPU_Graph,  # noqa: E402
                         Graph)
