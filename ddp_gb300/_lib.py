"""ctypes binding of libddp_gb300.so (the C-ABI in include/ddp_gb300.h)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libddp_gb300.so")

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
u32p = C.POINTER(C.c_uint32)
vp = C.c_void_p


class Opts(C.Structure):
    _fields_ = [("K", C.c_int32), ("delta", C.c_int32), ("block", C.c_int32), ("grid", C.c_int32),
                ("queue_cap", C.c_int64), ("stream", C.c_void_p), ("group", C.c_int32), ("flags", C.c_int32)]


# name -> (restype, argtypes)
SIGNATURES = {
    "ddp_last_error": (C.c_char_p, []),
    "ddp_version": (C.c_int, []),
    "ddp_device_count": (C.c_int, []),
    "ddp_graph_from_csr": (C.c_int, [C.c_int32, C.c_int64, i32p, C.c_int32, i32p, u32p, C.POINTER(vp)]),
    "ddp_graph_load_text": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
    "ddp_graph_set_coords": (C.c_int, [vp, i32p]),
    "ddp_graph_set_euclid": (C.c_int, [vp, C.c_uint32]),
    "ddp_graph_info": (C.c_int, [vp, i32p, i64p, u32p, u32p]),
    "ddp_graph_read_csr": (C.c_int, [vp, i32p, i32p, u32p]),
    "ddp_graph_free": (C.c_int, [vp]),
    "ddp_landmarks_build": (C.c_int, [vp, C.c_int32, C.c_uint64, C.POINTER(C.c_int32)]),
    "ddp_landmarks_build_bits": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(C.c_int32)]),
    "ddp_heuristic_build": (C.c_int, [vp, C.c_int32, C.c_int32, i32p, i32p, C.POINTER(vp)]),
    "ddp_heuristic_free": (C.c_int, [vp]),
    "ddp_solve": (C.c_int, [vp, vp, C.c_int32, C.c_int32, C.POINTER(Opts), C.POINTER(vp)]),
    "ddp_query_cost": (C.c_int, [vp, i32p]),
    "ddp_path_read": (C.c_int, [vp, i32p, C.c_int32, i32p]),
    "ddp_query_stats": (C.c_int, [vp, i64p]),
    "ddp_query_free": (C.c_int, [vp]),
    "ddp_batch_create": (C.c_int, [vp, C.c_int32, C.POINTER(Opts), C.POINTER(vp)]),
    "ddp_batch_solve": (C.c_int, [vp, C.c_int32, i32p, i32p, i32p, i32p]),
    "ddp_batch_solve_device": (C.c_int, [vp, C.c_int32, vp, vp, vp, vp]),
    "ddp_batch_sync": (C.c_int, [vp]),
    "ddp_batch_path": (C.c_int, [vp, C.c_int32, i32p, C.c_int32, i32p]),
    "ddp_batch_stats": (C.c_int, [vp, i64p, i64p, i64p]),
    "ddp_batch_info": (C.c_int, [vp, i32p, i64p, i32p]),
    "ddp_batch_group": (C.c_int, [vp, i32p]),
    "ddp_batch_launches": (C.c_int, [vp, i32p]),
    "ddp_batch_tune": (C.c_int, [vp, C.c_int32, C.c_int32, i32p, i32p, C.POINTER(Opts), C.POINTER(Opts),
                                  C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "ddp_batch_free": (C.c_int, [vp]),
    "ddp_dyn_create": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int32, C.POINTER(Opts), C.POINTER(vp)]),
    "ddp_dyn_update": (C.c_int, [vp, C.c_int32, i32p, i32p, i32p, u32p, i32p]),
    "ddp_dyn_cost": (C.c_int, [vp, i32p]),
    "ddp_dyn_path": (C.c_int, [vp, i32p, C.c_int32, i32p]),
    "ddp_dyn_stats": (C.c_int, [vp, i64p]),
    "ddp_dyn_grid": (C.c_int, [vp, i32p, i32p]),
    "ddp_kpaths": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, i32p, i32p, C.c_int64,
                              C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "ddp_dyn_free": (C.c_int, [vp]),
    "ddp_serve_create": (C.c_int, [vp, C.c_int32, C.POINTER(Opts), C.c_int64, C.c_int32, C.POINTER(vp)]),
    "ddp_serve_submit": (C.c_int, [vp, C.c_int32, i32p, i32p, i64p]),
    "ddp_serve_poll": (C.c_int, [vp, C.c_int32, i64p, i32p, i64p, i32p, i32p]),
    "ddp_serve_update": (C.c_int, [vp, C.c_int32, i32p, i32p, i32p, u32p]),
    "ddp_serve_stats": (C.c_int, [vp, i64p]),
    "ddp_serve_record_paths": (C.c_int, [vp, C.c_int32]),
    "ddp_serve_path": (C.c_int, [vp, C.c_int64, i32p, C.c_int32, i32p]),
    "ddp_serve_free": (C.c_int, [vp]),
    "ddp_bfs_hops_noalloc": (C.c_int, [C.c_int32, vp, vp, C.c_int32, vp, vp]),
    "ddp_io_read_graph_text": (C.c_int, [C.c_char_p, i32p, i64p, C.POINTER(i32p), C.POINTER(i32p), C.POINTER(u32p)]),
    "ddp_io_write_graph_text": (C.c_int, [C.c_char_p, C.c_int32, C.c_int64, i32p, i32p, u32p]),
    "ddp_io_write_graph_bin": (C.c_int, [C.c_char_p, C.c_int32, C.c_int64, i32p, i32p, u32p]),
    "ddp_io_read_graph_bin": (C.c_int, [C.c_char_p, i32p, i64p, C.POINTER(i32p), C.POINTER(i32p), C.POINTER(u32p)]),
    "ddp_io_read_ints_text": (C.c_int, [C.c_char_p, C.c_int64, i32p, i64p]),
    "ddp_io_write_ints_text": (C.c_int, [C.c_char_p, C.c_int64, i32p]),
    "ddp_io_read_updates_text": (C.c_int, [C.c_char_p, i32p, C.POINTER(i32p), C.POINTER(i32p), C.POINTER(i32p),
                                           C.POINTER(i32p), C.POINTER(u32p)]),
    "ddp_io_write_updates_text": (C.c_int, [C.c_char_p, C.c_int32, i32p, i32p, i32p, i32p, u32p]),
    "ddp_free": (None, [vp]),
    "ddp_gen_random_chain": (C.c_int, [C.c_int32, C.c_int64, C.c_uint32, C.c_uint32, C.c_uint64, i32p, i32p,
                                       u32p, i32p]),
    "ddp_gen_grid_from_walls": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_uint8), i32p, i32p, u32p, C.POINTER(C.c_int64)]),
    "ddp_gen_maze_moves": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_uint8), C.POINTER(C.c_uint8), C.c_int32, C.c_int32, C.c_uint64, i32p, i32p,
                                     i32p, i32p, u32p, C.c_int64, C.POINTER(C.c_int64)]),
    "ddp_gen_maze": (C.c_int, [C.c_int32, C.c_int32, C.c_uint32, C.c_uint64, i32p, i32p, i64p, i32p, i32p,
                               u32p, i32p]),
    "ddp_gen_updates": (C.c_int, [C.c_int32, C.c_int64, i32p, i32p, u32p, i32p, C.c_int32, C.c_int32, C.c_int32,
                                  C.c_uint32, C.c_uint32, C.c_uint64, i32p, i32p, i32p, u32p]),
    "ddp_gen_geometric": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_uint32, C.c_uint64, C.c_int32, i32p, i32p,
                                    i32p, u32p, i64p]),
    "ddp_gen_pairs": (C.c_int, [C.c_int32, i32p, i32p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                                C.c_int32, i32p, i32p, i32p]),
}

_lib = None


class DdpError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ddp error {code}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Loads the library; raises (never falls back) when it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m ddp_gb300.build` "
                              "(or __graft_entry__.build()) first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != 0:
        raise DdpError(rc, lib().ddp_last_error().decode(errors="replace"))


def ptr(a: np.ndarray, ct=C.c_int32):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(ct))
