"""Builds libddp_gb300.so in-tree (nvcc for sm_103a, gcc for host C).

    python -m ddp_gb300.build            # incremental
    python -m ddp_gb300.build --force    # rebuild everything

Translation units compile in parallel; objects go to ddp_gb300/_build/ and
the shared library to ddp_gb300/libddp_gb300.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libddp_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                     "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]
# extra nvcc flags for tuning builds, e.g. DDP_NVCC_EXTRA="-DDDP_ARCS=2"
NVCC_FLAGS += os.environ.get("DDP_NVCC_EXTRA", "").split()
CC_FLAGS = ["-O2", "-fPIC", "-std=c11", "-Wall", "-pthread", "-I" + INCLUDE, "-I" + CSRC]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    c = sorted(f for f in os.listdir(CSRC) if f.endswith(".c"))
    return cu, c


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(obj: str, src: str, headers) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src, *headers])


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cu, c = _sources()
    headers = _headers()
    nvcc = _nvcc()
    jobs = []
    for f in cu:
        src, obj = os.path.join(CSRC, f), os.path.join(BUILD, f[:-3] + ".o")
        if force or _stale(obj, src, headers):
            jobs.append([nvcc, *NVCC_FLAGS, "-c", src, "-o", obj])
    for f in c:
        src, obj = os.path.join(CSRC, f), os.path.join(BUILD, f[:-2] + ".o")
        if force or _stale(obj, src, headers):
            jobs.append(["gcc", *CC_FLAGS, "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        return p.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for _ in ex.map(run, jobs):
            pass
    objs = [os.path.join(BUILD, f[:-3] + ".o") for f in cu] + [os.path.join(BUILD, f[:-2] + ".o") for f in c]
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"])
    return LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build(force=force, verbose=True))
