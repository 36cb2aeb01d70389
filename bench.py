#!/usr/bin/env python
"""Benchmark: batched GA* queries/sec on one GB300 (exact costs).

Workload (default, `--config c4`): 4,096 seeded source/target pairs on a
4M-node random digraph (Hamiltonian chain + uniform arcs, average out-degree
8, int32 weights uniform in [1,100]); heuristic h = reverse-BFS hop count to
the target x min weight, built per query inside the batch kernel.  One step
= one batch of all pairs through the persistent batch kernel.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` = queries/sec with inputs resident in
HBM, timed with CUDA events on the launching stream; `e2e` = the same metric
through the C-ABI call with host buffers (H2D + D2H inside the timed region).
N > 1 (torchrun) runs independent replicas, each on its own pairs (weak
scaling, no data-path collective).  `--impl reference` times the reference's
serial CPU A* (the oracle restatement) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # name: (nodes, avg out-degree, wmin, wmax, pairs, hop_lo, hop_hi, graph seed, pair seed)
    "c4": dict(n=4_000_000, deg=8, wmin=1, wmax=100, pairs=4096, hop_lo=4, hop_hi=400, gseed=4004,
               pseed=4400),
    "c4-small": dict(n=400_000, deg=8, wmin=1, wmax=100, pairs=1024, hop_lo=4, hop_hi=400, gseed=4004,
                     pseed=4400),
}


def workload_name(c):
    return (f"batched multi-query GA*: {c['pairs']} seeded (s,t) pairs, target BFS hops log-uniform in "
            f"[{c['hop_lo']},{c['hop_hi']}] (clipped to what the graph realises), on a {c['n']:,}-node "
            f"random digraph (Hamiltonian chain + uniform arcs), avg out-degree {c['deg']}, int32 w U[{c['wmin']},"
            f"{c['wmax']}], h = reverse-BFS hops x min w per target")


def args_parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", default="c4", choices=sorted(CONFIGS))
    p.add_argument("--pairs", type=int, default=0, help="override the number of pairs")
    p.add_argument("--slots", type=int, default=0, help="concurrent query slots (0 = auto)")
    p.add_argument("--block", type=int, default=0)
    p.add_argument("--delta", type=int, default=0)
    p.add_argument("--K", type=int, default=0)
    p.add_argument("--group", type=int, default=19, help="CTAs per query slot")
    p.add_argument("--heuristic", default="capped", choices=["capped", "bfs", "zero"],
                   help="capped: reverse-BFS hops stopped at max(4096, n/32) reached nodes (unreached nodes "
                        "get last level + 1); bfs: full reverse BFS; zero: h = 0")
    p.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU baseline work")
    p.add_argument("--plain-sample", type=int, default=16, help="queries timed on plain single-query GA*")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        rows = [r.strip().split(", ") for r in self.f.read().splitlines() if r.strip()]
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_per_launch(config_name, pairs):
    """dram bytes of one k_batch launch from the committed ncu summary
    (profiles/k_batch_<config>.md, line `traffic_bytes_per_query: X`), scaled
    to this launch's query count."""
    p = os.path.join(ROOT, "profiles", f"k_batch_{config_name}.md")
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_query:"):
                return float(line.split(":")[1]) * pairs
    except OSError:
        pass
    return None


def algorithmic_bytes(st):
    """Per-query bytes of the algorithm (graph-search accounting):
    12 B per expanded node (2 offsets + g), 16 B per scanned arc (head, w,
    h(head), g(head)), 16 B per successful relaxation (g, parent, queue
    push), and for the heuristic BFS 12 B per reached node + 8 B per scanned
    reverse arc."""
    st = np.asarray(st, np.float64)
    return 12 * st[:, 0] + 16 * st[:, 1] + 16 * st[:, 2] + 12 * st[:, 4] + 8 * st[:, 5]


def make_workload(c, pairs, rank):
    import ddp_gb300 as d
    g = d.gen_random_chain(c["n"], c["deg"], c["wmin"], c["wmax"], c["gseed"])
    S, T, want = d.gen_pairs(g, pairs, c["hop_lo"], c["hop_hi"], c["pseed"] + 7919 * rank)
    return g, S, T, want


def run_reference(a, c, world, rank):
    """The reference's CPU A* (oracle restatement of GA_star/A_star_cpu.cpp)
    on all host cores: each step = one bounded sample of the workload."""
    if rank != 0:
        return
    from oracle import oracle as O
    pairs = a.pairs or c["pairs"]
    g, S, T, _ = make_workload(c, pairs, 0)
    threads = os.cpu_count() or 1
    off = g.off[:-1]
    # heap with the position map: the same pops and result as the reference's
    # linear-scan decrease-key, strictly faster (an upper bound on its speed)
    mode = O.HEAP_POSMAP
    per_step = threads
    times, done_total, q = [], 0, 0
    for step in range(a.warmup + a.steps):
        idx = [(q + i) % pairs for i in range(per_step)]
        q += per_step
        t0 = time.perf_counter()
        cost, ss, hs, done = O.astar_many(g.n, off, g.col, g.w, S[idx], T[idx], hkind=1, wmin=c["wmin"],
                                          mode=mode, threads=threads, budget_s=1e9)
        dt = time.perf_counter() - t0
        if step >= a.warmup:
            times.append(dt)
            done_total += done
    total = sum(times)
    value = done_total / total if total > 0 else 0.0
    out = {
        "impl": "reference",
        "metric": "A* queries/sec (batched, exact costs)",
        "value": value, "unit": "queries/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1000 * total / max(1, a.steps), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generators)",
        "config": {"workload": workload_name(c), "pairs_per_step": per_step},
        "cpu_baseline": {"value": value, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"{per_step} queries per step (one per core), heuristic BFS + serial A* "
                                   "per query; position-map decrease-key (same pops as the reference's "
                                   "linear scan, faster)"},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    a = args_parse()
    world, rank, local = dist_env()
    c = dict(CONFIGS[a.config])
    if a.impl == "reference":
        run_reference(a, c, world, rank)
        return

    import torch

    from ddp_gb300 import build as B
    B.build()
    import ddp_gb300 as d

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pairs = a.pairs or c["pairs"]
    g, S, T, want = make_workload(c, pairs, rank)
    dg = d.DeviceGraph.from_csr(g)
    # a dedicated stream: the engine launches on it and the CUDA events that
    # time the steps are recorded on it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    hkind = {"capped": d.H_BFS_CAPPED, "bfs": d.H_BFS_HOPS, "zero": d.H_ZERO}[a.heuristic]
    opts = dict(grid=a.slots, block=a.block, delta=a.delta, K=a.K, group=a.group)
    be = d.BatchEngine(dg, hkind, stream=stream.cuda_stream, **opts)
    dS = torch.from_numpy(S).to(dev)
    dT = torch.from_numpy(T).to(dev)
    dcost = torch.empty(pairs, dtype=torch.int32, device=dev)
    dplen = torch.empty(pairs, dtype=torch.int32, device=dev)

    def step():
        be.solve_device(pairs, dS.data_ptr(), dT.data_ptr(), dcost.data_ptr(), dplen.data_ptr())

    for _ in range(max(3, a.warmup)):
        step()
    torch.cuda.synchronize(dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize(dev)
    with Clocks(local) as ck:
        ev0.record(stream)
        for _ in range(a.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize(dev)
    barrier()
    elapsed = ev0.elapsed_time(ev1) / 1000.0
    tmax = elapsed
    if world > 1:
        t = torch.tensor([elapsed], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        tmax = float(t.item())
    clocks = ck.summary()
    costs = dcost.cpu().numpy()
    st, t0, t1 = be.stats()
    launches = be.launches() * a.steps
    value = world * pairs * a.steps / tmax
    kernel_s = elapsed / a.steps
    alg = float(algorithmic_bytes(st).sum())
    peak, peak_kind = peak_hbm()
    achieved = alg / kernel_s / 1e9
    traffic = traffic_per_launch(a.config, pairs)
    lat_service = (t1 - t0) / 1e6
    lat_complete = (t1 - t0.min()) / 1e6

    # end to end through the C-ABI with host buffers (H2D + D2H inside)
    e2e_times = []
    for i in range(a.steps + 1):
        torch.cuda.synchronize(dev)
        s0 = time.perf_counter()
        hc, hp = be.solve(S, T)
        s1 = time.perf_counter()
        if i > 0:
            e2e_times.append(s1 - s0)
    e2e_qps = world * pairs * len(e2e_times) / sum(e2e_times)
    exact_vs_batch = bool(np.array_equal(hc, costs))

    # plain single-query GA* looped one query at a time (heuristic + solve)
    plain = None
    if a.plain_sample > 0:
        ps = min(a.plain_sample, pairs)
        for i in range(2):  # warm the single-query workspace
            h = dg.heuristic(int(T[i]), hkind)
            dg.solve(int(S[i]), int(T[i]), h)
            h.close()
        torch.cuda.synchronize(dev)
        p0 = time.perf_counter()
        pc = []
        for i in range(ps):
            h = dg.heuristic(int(T[i]), hkind)
            r = dg.solve(int(S[i]), int(T[i]), h)
            h.close()
            pc.append(r.cost)
        pt = time.perf_counter() - p0
        plain = {"qps": ps / pt, "sample": ps, "costs_match_batch": bool(np.array_equal(pc, costs[:ps]))}

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        k = min(pairs, threads)
        cst, ss, hs, done = O.astar_many(g.n, g.off[:-1], g.col, g.w, S[:k], T[:k], hkind=1, wmin=c["wmin"],
                                         mode=O.HEAP_POSMAP, threads=threads, budget_s=a.cpu_budget)
        ok = cst[:k] >= 0
        if done:
            cpu = {"value": threads * done / float(ss[ok].sum() + hs[ok].sum()), "unit": "queries/s",
                   "cores": threads, "kind": "port",
                   "sample": f"{done} of the first {k} pairs, one per core: reverse BFS + serial A* "
                             f"(GA_star/A_star_cpu.cpp restated, position-map decrease-key); mean search "
                             f"{1000 * ss[ok].mean():.0f} ms, heuristic {1000 * hs[ok].mean():.0f} ms per query",
                   "costs_match_gpu": bool(np.array_equal(cst[ok], costs[:k][ok]))}

    out = {
        "metric": "A* queries/sec (batched, exact costs)",
        "value": value, "unit": "queries/s", "n_gpus": world, "steps": a.steps, "warmup": max(3, a.warmup),
        "ms_per_step": 1000 * tmax / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generators)",
        "config": {"workload": workload_name(c), "n": g.n, "e": g.e, "pairs_per_gpu": pairs,
                   "heuristic": a.heuristic,
                   "slots": be.info()["slots"], "block": be.info()["block"], "K": a.K,
                   "group": be.info()["group"],
                   "delta": a.delta or "auto",
                   "l2": "inputs larger than L2 (graph ~%d MB + per-slot state)" % ((g.e * 16 + g.n * 8) >> 20),
                   "parallelism": f"replicas x{world} (queries sharded, no collective)"},
        "latency_ms": {"p50": float(np.percentile(lat_complete, 50)), "p99": float(np.percentile(lat_complete, 99)),
                       "service_p50": float(np.percentile(lat_service, 50)),
                       "service_p99": float(np.percentile(lat_service, 99)),
                       "note": "completion time from batch start (all queries submitted at once); service = on-slot time"},
        "plain_ga": plain,
        "speedup_vs_plain": (value / world / plain["qps"]) if plain else None,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "k_batch<1>", "algorithmic_bytes_per_launch": alg,
                     "kernel_ms": 1000 * kernel_s},
        "work_per_query": {"phases_mean": float(st[:, 3].mean()), "expanded_mean": float(st[:, 0].mean()), "arcs_scanned_mean": float(st[:, 1].mean()),
                           "relaxed_mean": float(st[:, 2].mean()), "bfs_reached_mean": float(st[:, 4].mean()),
                           "far_scanned_mean": float(st[:, 6].mean()), "touched_mean": float(st[:, 7].mean())},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_qps, "unit": "queries/s", "h2d_bytes_per_step": int(S.nbytes + T.nbytes),
                "d2h_bytes_per_step": int(2 * 4 * pairs), "exact_vs_device_run": exact_vs_batch},
        "overflowed_queries": int((costs == -1).sum()),
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    be.close()
    dg.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
