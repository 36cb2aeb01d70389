"""The LIB shim on the GPU: A_Star and GPU_A_Star (through the C ABI) give
the reference's known answer on the 8-node graph (cost 6, path 0 2 4 6 7)
and oracle-exact costs on a random graph, twice in a row."""
import os

import numpy as np
import pytest

from test_lib_shim import KAT8, ROOT, _lib_or_skip, build_shim

pytestmark = pytest.mark.gpu


def _run(exe, graph, s, t):
    import subprocess
    p = subprocess.run([exe, graph, str(s), str(t), "4"], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    out = {}
    for line in p.stdout.splitlines():
        k, _, v = line.partition(":")
        out[k] = [int(x) for x in v.split()]
    return out


def test_shim_on_gpu(gpu, oracle, tmp_path):
    d = gpu
    _lib_or_skip()
    exe = str(tmp_path / "shim")
    build_shim(os.path.join(ROOT, "tests", "lib_shim", "shim_main.cpp"), exe, nvcc=True)
    (tmp_path / "kat8.txt").write_text(KAT8)
    r = _run(exe, str(tmp_path / "kat8.txt"), 0, 7)
    assert r["cpu_class_unset"] == [-1]
    for k in ("cpu_class", "gpu_class", "gpu_class_again"):
        assert r[k] == [0, 2, 4, 6, 7], k
    # a random graph in the reference's text format (N offsets, no sentinel)
    g = d.gen_random_chain(5000, 5, 1, 60, 91)
    path = str(tmp_path / "g.txt")
    d.write_graph_text(path, g)
    rng = np.random.default_rng(1)
    gs = g.with_sentinel()
    for s, t in rng.integers(0, g.n, (4, 2)):
        f, c, _, _, _ = oracle.astar(gs.n, gs.off[:-1], gs.col, gs.w, np.zeros(gs.n, np.int32), int(s), int(t))
        r = _run(exe, path, int(s), int(t))
        for k in ("cpu_class", "gpu_class", "gpu_class_again"):
            ok, why = oracle.check_path(g.off, g.col, g.w, r[k], int(s), int(t), c, 0)
            assert f and ok, (k, why)
