"""Python access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs use this module, as the checker.  The product library never imports it.

  * liboracle.so  - the C restatement in astar_oracle.c (built by `make -C oracle`)
  * _ref/a_star_cpu - the reference's own GA_star/A_star_cpu.cpp, compiled from
    the read-only reference tree by `make -C oracle ref` (present only where
    that tree exists)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_ASTAR = os.path.join(HERE, "_ref", "a_star_cpu")
REF_LIB_MAIN = os.path.join(HERE, "_ref", "lib_main_cpu")

HEAP_SCAN, HEAP_POSMAP = 0, 1
INF = 2147483647

_lib = None
i32p = C.POINTER(C.c_int32)
u32p = C.POINTER(C.c_uint32)


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        srcs = [os.path.join(HERE, f) for f in ("astar_oracle.c", "gen_oracle.c")]
        if not os.path.exists(LIB) or any(os.path.getmtime(LIB) < os.path.getmtime(f) for f in srcs):
            build()
        L = C.CDLL(LIB)
        L.oracle_astar.restype = C.c_int
        L.oracle_astar.argtypes = [C.c_int, C.c_int, i32p, i32p, u32p, i32p, C.c_int, C.c_int, C.c_int, i32p,
                                   i32p, C.c_int, i32p, C.POINTER(C.c_int64), C.POINTER(C.c_double)]
        L.oracle_bfs_hops.restype = None
        L.oracle_bfs_hops.argtypes = [C.c_int, C.c_int, i32p, i32p, C.c_int, i32p]
        L.oracle_reverse_csr.restype = None
        L.oracle_reverse_csr.argtypes = [C.c_int, C.c_int, i32p, i32p, u32p, i32p, i32p, u32p]
        L.oracle_apply_batch.restype = C.c_int
        L.oracle_apply_batch.argtypes = [C.c_int, C.c_int, i32p, i32p, u32p, C.c_int, i32p, i32p, i32p, u32p,
                                         i32p, i32p, u32p, i32p]
        L.oracle_astar_many.restype = C.c_int
        L.oracle_astar_many.argtypes = [C.c_int, C.c_int, i32p, i32p, u32p, i32p, i32p, C.c_int, C.c_int, C.c_int,
                                        i32p, i32p, C.c_int, C.c_int, C.c_double, i32p, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]
        L.oracle_gen_random_chain.restype = C.c_int
        L.oracle_gen_random_chain.argtypes = [C.c_int32, C.c_int64, C.c_uint32, C.c_uint32, C.c_uint64, i32p, i32p,
                                              u32p, i32p]
        L.oracle_gen_pairs.restype = C.c_int
        L.oracle_gen_pairs.argtypes = [C.c_int32, i32p, i32p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                       C.c_uint64, C.c_int32, i32p, i32p, i32p]
        _lib = L
    return _lib


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _u(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def _p(a, t=C.c_int32):
    return a.ctypes.data_as(C.POINTER(t))


def ref_layout(off):
    """n+1 offsets -> the reference's n offsets."""
    return _i(off[:-1])


def astar(n, off, col, w, h, s, t, mode=HEAP_POSMAP, path_cap=None):
    """Reference A* (GA_star/A_star_cpu.cpp).  `off` in the reference layout
    (n entries).  Returns (found, cost, path, stats[pops, scans, relax],
    search_seconds)."""
    off, col, w, h = _i(off), _i(col), _u(w), _i(h)
    e = len(col)
    cap = path_cap if path_cap is not None else n
    path = np.empty(max(cap, 1), np.int32)
    cost = C.c_int32()
    plen = C.c_int32()
    stats = np.zeros(3, np.int64)
    secs = C.c_double()
    found = lib().oracle_astar(n, e, _p(off), _p(col), _p(w, C.c_uint32), _p(h), int(s), int(t), mode,
                               C.byref(cost), _p(path), cap, C.byref(plen), _p(stats, C.c_int64),
                               C.byref(secs))
    if found < 0:
        raise ValueError("bad oracle arguments")
    return bool(found), cost.value, path[:min(plen.value, cap)].copy(), stats, secs.value


def bfs_hops(n, roff, rcol, root):
    """bfs_hx.cu restated: hop distance to `root` over the reverse CSR given
    in the reference layout; -1 = unreachable."""
    roff, rcol = _i(roff), _i(rcol)
    dist = np.empty(n, np.int32)
    lib().oracle_bfs_hops(n, len(rcol), _p(roff), _p(rcol), int(root), _p(dist))
    return dist


def reverse_csr(n, off, col, w):
    """genOpCSR.cpp restated; reference layout in and out."""
    off, col, w = _i(off), _i(col), _u(w)
    e = len(col)
    roff = np.empty(n, np.int32)
    rcol = np.empty(max(e, 1), np.int32)
    rw = np.empty(max(e, 1), np.uint32)
    lib().oracle_reverse_csr(n, e, _p(off), _p(col), _p(w, C.c_uint32), _p(roff), _p(rcol), _p(rw, C.c_uint32))
    live = int((col >= 0).sum())
    return roff, rcol[:live].copy(), rw[:live].copy()


def bfs_heuristic(n, off, col, w, target, wmin=None):
    """h(v) = hops(v -> target) x min arc weight, -1 where target is
    unreachable (reference layout in)."""
    roff, rcol, _ = reverse_csr(n, off, col, w)
    d = bfs_hops(n, roff, rcol, target)
    if wmin is None:
        live = np.asarray(col) >= 0
        wmin = int(np.asarray(w)[live].min()) if live.any() else 0
    return np.where(d < 0, -1, d.astype(np.int64) * wmin).astype(np.int32)


def apply_batch(n, off, col, w, flag, u, v, uw):
    """DA_dyn_cpu.cu batch semantics (removeDelEdges + mergeDiff); reference
    layout in and out.  Returns (off, col, w, n_deleted)."""
    off, col, w = _i(off), _i(col), _u(w)
    flag, u, v, uw = _i(flag), _i(u), _i(v), _u(uw)
    e = len(col)
    nins = int((flag == 1).sum())
    noff = np.empty(n, np.int32)
    ncol = np.empty(max(e + nins, 1), np.int32)
    nw = np.empty(max(e + nins, 1), np.uint32)
    nd = C.c_int32()
    ne = lib().oracle_apply_batch(n, e, _p(off), _p(col), _p(w, C.c_uint32), len(flag), _p(flag), _p(u), _p(v),
                                  _p(uw, C.c_uint32), _p(noff), _p(ncol), _p(nw, C.c_uint32), C.byref(nd))
    return noff, ncol[:ne].copy(), nw[:ne].copy(), nd.value


def astar_many(n, off, col, w, S, T, hkind=1, wmin=1, mode=HEAP_SCAN, threads=1, budget_s=10.0):
    """Independent queries on a thread pool.  Returns (costs (-1 = not run),
    search seconds per query, heuristic seconds per query, completed)."""
    off, col, w = _i(off), _i(col), _u(w)
    roff, rcol, _ = reverse_csr(n, off, col, w)
    S, T = _i(S), _i(T)
    nq = len(S)
    cost = np.empty(nq, np.int32)
    ss = np.zeros(nq, np.float64)
    hs = np.zeros(nq, np.float64)
    done = lib().oracle_astar_many(n, len(col), _p(off), _p(col), _p(w, C.c_uint32), _p(roff), _p(rcol), hkind,
                                   wmin, nq, _p(S), _p(T), mode, threads, budget_s, _p(cost),
                                   ss.ctypes.data_as(C.POINTER(C.c_double)),
                                   hs.ctypes.data_as(C.POINTER(C.c_double)))
    return cost, ss, hs, done


def have_reference_binary() -> bool:
    return os.path.exists(REF_ASTAR)


def run_reference_astar(n, off, col, w, h, s, t):
    """Runs the reference's compiled A_star_cpu in a temp dir on graph.txt /
    Hx.txt written in its format.  Returns (cost or None, path s..t)."""
    off, col, w, h = _i(off), _i(col), _u(w), _i(h)
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "graph.txt"), "w") as f:
            f.write(f"{n} {len(col)}\n")
            f.write(" ".join(map(str, col.tolist())) + "\n")
            f.write(" ".join(map(str, off.tolist())) + "\n")
            f.write(" ".join(map(str, w.tolist())) + "\n")
        with open(os.path.join(d, "Hx.txt"), "w") as f:
            f.write(" ".join(map(str, h.tolist())))
        p = subprocess.run([REF_ASTAR], input=f"{s} {t}\n", cwd=d, capture_output=True, text=True, timeout=600)
    lines = [x.strip() for x in p.stdout.splitlines() if x.strip()]
    for i, ln in enumerate(lines):
        if ln.startswith("cost"):
            cost = int(ln.split()[1])
            path = [int(x) for x in lines[i + 1].split()][::-1]
            return cost, np.array(path, np.int32)
    return None, np.zeros(0, np.int32)


def run_reference_lib_main(n, off, col, w):
    """Runs the reference's LIB demo (CPU half of LIB/main.cpp) on graph.txt;
    returns its stdout lines."""
    off, col, w = _i(off), _i(col), _u(w)
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "graph.txt"), "w") as f:
            f.write(f"{n} {len(col)}\n")
            f.write(" ".join(map(str, col.tolist())) + "\n")
            f.write(" ".join(map(str, off.tolist())) + "\n")
            f.write(" ".join(map(str, w.tolist())) + "\n")
        p = subprocess.run([REF_LIB_MAIN], cwd=d, capture_output=True, text=True, timeout=60)
    return p.stdout.splitlines()


def check_path(off_full, col, w, path, s, t, cost, h_t=0):
    """Path validity: starts at s, ends at t, each hop is a live arc, and the
    summed weight (min over parallel arcs) + h(t) equals cost.  off_full has
    n+1 entries."""
    path = np.asarray(path)
    if len(path) == 0 or path[0] != s or path[-1] != t:
        return False, "endpoints"
    total = 0
    for a, b in zip(path[:-1], path[1:]):
        row = slice(off_full[a], off_full[a + 1])
        cs = np.asarray(col[row])
        ws = np.asarray(w[row])
        m = cs == b
        if not m.any():
            return False, f"missing arc {a}->{b}"
        total += int(ws[m].min())
    if total + h_t != cost:
        return False, f"weight {total}+{h_t} != cost {cost}"
    return True, ""


def gen_random_chain(n, avg_deg, wmin, wmax, seed):
    """Seeded random digraph (Hamiltonian chain + uniform arcs, no
    self-loops or duplicates, n * avg_deg arcs) from gen_oracle.c.  Returns
    (off[n+1], col, w, perm)."""
    e = int(n) * int(avg_deg)
    off = np.empty(n + 1, np.int32)
    col = np.empty(e, np.int32)
    w = np.empty(e, np.uint32)
    perm = np.empty(n, np.int32)
    rc = lib().oracle_gen_random_chain(int(n), e, int(wmin), int(wmax), int(seed), _p(off), _p(col),
                                       _p(w, C.c_uint32), _p(perm))
    if rc:
        raise ValueError(f"oracle_gen_random_chain failed ({rc})")
    return off, col, w, perm


def gen_pairs(n, off, col, npairs, hop_lo, hop_hi, seed, bfs_cap_level=6, threads=0):
    """Seeded (S, T, wanted hops) from gen_oracle.c; off has n+1 entries."""
    off, col = _i(off), _i(col)
    S = np.empty(npairs, np.int32)
    T = np.empty(npairs, np.int32)
    want = np.empty(npairs, np.int32)
    threads = threads or min(16, os.cpu_count() or 1)
    rc = lib().oracle_gen_pairs(int(n), _p(off), _p(col), int(npairs), int(hop_lo), int(hop_hi),
                                int(bfs_cap_level), int(seed), int(threads), _p(S), _p(T), _p(want))
    if rc:
        raise ValueError(f"oracle_gen_pairs failed ({rc})")
    return S, T, want
