"""Replicas (the multi-GPU form of this path): each rank builds the same
graph, takes its own seeded pairs, and the job time is the MAX over ranks.
Run here as two gloo ranks on the CPU, exercising bench.py's own helpers."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

TINY = dict(n=3000, deg=4, wmin=1, wmax=50, pairs=24, hop_lo=2, hop_hi=30, gseed=11, pseed=12)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    g, S, T, _ = bench.make_workload(TINY, TINY["pairs"], rank)
    graphs = [None] * world
    pairs = [None] * world
    dist.all_gather_object(graphs, int(np.asarray(g.col, np.int64).sum() * 31 + np.asarray(g.w, np.int64).sum()))
    dist.all_gather_object(pairs, (S.tolist(), T.tolist()))
    tmax = bench.max_over_ranks(0.5 + rank, world, torch.device("cpu"))
    # the reference arm: only rank 0 works
    a = type("A", (), {"pairs": TINY["pairs"], "steps": 1, "warmup": 0})()
    ref_other = bench.run_reference(a, TINY, world, rank) if rank != 0 else None
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, graphs, pairs, tmax, ref_other))


def test_two_gloo_replicas():
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for rank, graphs, pairs, tmax, ref_other in res:
        assert graphs[0] == graphs[1]          # one replicated graph
        assert pairs[0] != pairs[1]            # queries sharded by rank seed
        assert tmax == 1.5                     # slowest replica
        assert ref_other is None               # reference arm: ranks > 0 do nothing
