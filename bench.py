#!/usr/bin/env python3
"""Headline benchmark: single-query BFS throughput on RMAT scale 24.

Workload (the spec traversal target): RMAT scale 24, edge factor 16,
a/b/c/d = .57/.19/.19/.05, seed 3, symmetrised, self-loops and duplicates
removed, seeded vertex relabelling; source = first vertex of maximum
out-degree (the rule of include/graph_loader.cuh:132-137).  Synthetic data:
the reference's datasets are not available; the graph is generated on the
device from the seed.

A step is one BFS from the source over the resident graph.  Metric: GTEPS =
m_r / time, m_r = sum of out-degrees of reached vertices.  `value` is timed
with CUDA events on the launching stream (device-resident input and output);
`e2e` is the same BFS through the public API with a pinned HOST output buffer
(the depth array is copied back inside the timed region).  L2 is flushed
(256 MB write) before every timed step, outside its events.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl grus|reference]

`--impl reference` times the CPU path (the reference has no host BFS; the
plain OpenMP level-synchronous BFS of the oracle stands in) on all host cores
on the same graph, generated on the host from the same seed.
Under torchrun each rank runs an independent replica ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = dict(workload="bfs_rmat24_sym", graph="rmat", scale=24, edge_factor=16, seed=3,
                symmetric=True, relabel=True, source="max_degree_vertex")
METRIC = "GTEPS (single-query BFS, RMAT-24 symmetrised)"
UNIT = "GTEPS"
FALLBACK_HBM_GBS = 6800.0


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", FALLBACK_HBM_GBS)), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def bfs_alg_bytes(n, nr, mr):
    """Algorithmic bytes of one BFS: 4(n+1) offsets + 4 m_r column ids + 4n depth
    writes + 8 n_r frontier enqueue/dequeue (the fixed top-down figure, also
    used for direction-optimised runs)."""
    return 4 * (n + 1) + 4 * mr + 4 * n + 8 * nr


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def reduce_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---------------------------------------------------------------------------
def cpu_baseline_bfs(offs, cols, src, budget_s=12.0, max_runs=5):
    """OpenMP top-down BFS of the oracle on all host threads; median GTEPS."""
    import oracle
    g = oracle.CSR(offs, cols)
    threads = oracle.omp_threads()
    d, _ = oracle.omp_bfs(g, src, threads)  # warm-up
    mr = oracle.reached_edges(g, d)
    times = []
    t_start = time.perf_counter()
    while len(times) < max_runs and (time.perf_counter() - t_start) < budget_s:
        _, t = oracle.omp_bfs(g, src, threads)
        times.append(t)
    med = statistics.median(times)
    return {"value": round(mr / med / 1e9, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(times)} full BFS runs from the same source on the same graph "
                      f"(median {med*1e3:.1f} ms), OpenMP level-synchronous top-down BFS"}


def run_grus(args, dist, rank, local):
    import torch
    import grus_framework_gb300 as grus

    torch.cuda.set_device(local)
    grus.device_init(local)
    w = WORKLOAD
    g = grus.Graph.rmat(w["scale"], w["edge_factor"], w["seed"], symmetric=w["symmetric"],
                        relabel=w["relabel"])
    n, m, src = g.n, g.m, g.max_degree_vertex
    stream = torch.cuda.Stream()
    out_dev = torch.empty(n, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    # one call with stats: m_r, n_r (deterministic for the source), kernel time
    _, st = grus.bfs(g, src, out=out_dev, stream=stream, stats=True)
    mr, nr = st["edges_reached"], st["vertices_reached"]
    for _ in range(args.warmup):
        grus.bfs(g, src, out=out_dev, stream=stream)
    torch.cuda.synchronize()
    barrier(dist)

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ev[i][0].record(stream)
            grus.bfs(g, src, out=out_dev, stream=stream)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    barrier(dist)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = reduce_max(dist, sum(step_ms))
    ws = dist.get_world_size() if dist else 1
    total_edges = reduce_sum(dist, mr * args.steps)
    value = total_edges / (total_ms * 1e-3) / 1e9
    mean_ms = sum(step_ms) / len(step_ms)

    # end to end through the public API: pinned host output, D2H inside
    out_host = torch.empty(n, dtype=torch.int32, pin_memory=True)
    grus.bfs(g, src, out=out_host, stream=stream)
    e2e_s = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        stream.synchronize()
        t0 = time.perf_counter()
        grus.bfs(g, src, out=out_host, stream=stream)
        e2e_s.append(time.perf_counter() - t0)
    e2e_total = reduce_max(dist, sum(e2e_s))
    e2e_value = total_edges / e2e_total / 1e9

    # correctness of the timed configuration (cheap checks; full parity in tests)
    d = out_host.numpy().view(np.uint32)
    assert d[src] == 0 and int(np.count_nonzero(d != 4294967294)) == nr

    peak, peak_kind = measured_peaks()
    alg = bfs_alg_bytes(n, nr, mr)
    achieved = alg / (mean_ms * 1e-3) / 1e9
    traffic = None
    prof = ROOT / "profiles" / "bfs_persistent_rmat24.json"
    if prof.exists():
        traffic = json.loads(prof.read_text()).get("dram_bytes_per_launch")
    result = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            offs, cols, _ = g.copy_csr()
            cpu = cpu_baseline_bfs(offs, cols, src)
        clocks = clk.summary()
        result = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(mean_ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (RMAT generated on device from the seed)",
            "config": {**w, "n": n, "m": m, "src": src, "l2": "flushed (256 MB write) before each step",
                       "parallelism": f"replicas x{ws}", "levels": st["levels"],
                       "bottom_up_levels": st["bottom_up_levels"],
                       "vertices_reached": nr, "edges_reached": mr},
            "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": 4,
                    "d2h_bytes_per_step": 4 * n,
                    "note": "grus_bfs with a pinned host output buffer; graph resident in HBM"},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_source": peak_kind, "kernel": "bfs_persistent",
                         "algorithmic_bytes_per_launch": alg},
            "cpu_baseline": cpu,
            "clocks": clocks,
        }
    g.free()
    return result


def run_reference(args, dist, rank):
    """CPU path: OpenMP BFS of the oracle on the host cores (rank 0 only)."""
    if rank != 0:
        return None
    import oracle
    w = WORKLOAD
    flags = oracle.GEN_SYMMETRIC | (oracle.GEN_RELABEL if w["relabel"] else 0)
    g = oracle.rmat(w["scale"], w["edge_factor"], w["seed"], flags)
    src = oracle.max_degree_vertex(g)
    threads = oracle.omp_threads()
    d, _ = oracle.omp_bfs(g, src, threads)
    mr = oracle.reached_edges(g, d)
    for _ in range(max(args.warmup - 1, 0)):
        oracle.omp_bfs(g, src, threads)
    times = [oracle.omp_bfs(g, src, threads)[1] for _ in range(args.steps)]
    total = sum(times)
    value = mr * args.steps / total / 1e9
    return {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total / args.steps * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (RMAT generated on the host from the seed)", "impl": "reference",
        "config": {**w, "n": g.n, "m": g.m, "src": src, "edges_reached": mr},
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "each step = one full OpenMP BFS from the source"},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["grus", "reference"], default="grus")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "grus" else args.warmup
    ws, rank, local = dist_env()
    dist = init_dist(ws)
    if args.impl == "reference":
        res = run_reference(args, dist, rank)
    else:
        res = run_grus(args, dist, rank, local)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
