#!/usr/bin/env python3
"""Traversal benchmark: single-query BFS throughput on RMAT scale 24 (default).

Default workload (the traversal-rate target of the path): RMAT scale 24,
edge factor 16, a/b/c/d = .57/.19/.19/.05, seed 3, symmetrised, self-loops
and duplicates removed, seeded vertex relabelling; source = first vertex of
maximum out-degree (the rule of include/graph_loader.cuh:132-137).  Synthetic
data: the reference's datasets are not available; graphs are generated on
the device from the seed.

A step is one query over the resident graph.  Metric: GTEPS = traversed
edges / time (BFS/SSSP: m_r = sum of out-degrees of reached vertices; CC: m;
PageRank: m x iterations; multi-source BFS/SSSP: the sum of m_r over the
sources).
`value` is timed with CUDA events on the launching stream (device-resident
input and output); `e2e` is the same query through the public API with a
pinned HOST output buffer (the result is copied back inside the timed
region).  L2 is flushed (256 MB write) before every timed step, outside its
events.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl grus|reference]
                  [--workload NAME] [--scale S]

Other workloads (`--workload`): sssp-rmat22, cc-rmat22, pagerank-rmat24
(directed), bfs-grid4096, bfs-rmat26-managed (managed memory, device budget
half the CSR bytes), msbfs-rmat23 (64 sources), msssp-rmat22 (32 sources),
and the two systems forms in queries/s: batch-sssp256 (256 SSSP queries over 32
resident RMAT graphs of scales 14-20 in one batched call per step; also the
same queries as back-to-back plain calls) and serve-mixed (Poisson arrivals at
8,000 queries/s against 8 resident RMAT graphs of scales 16-24, half SSSP,
through the query server; a step is 1,000 queries; p50/p99 latency, a sweep
of lower arrival rates, and back-to-back plain calls of the same mix).
`--scale` overrides the RMAT scale (or the grid side as a power of two) for
small profiling runs.

`--impl reference` times the CPU path (the reference has no host traversal;
the plain OpenMP version of the same algorithm in the oracle stands in) on
all host cores on the same graph, generated on the host from the same seed.
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

FALLBACK_HBM_GBS = 6800.0
UNIT = "GTEPS"
INFINIT = 4294967294

# Graph sets of the batched and served workloads: (scale, edge factor,
# generator seed), symmetrised, weighted, relabelled.
def batch_graph_specs(seed):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(32):
        sc = int(rng.integers(14, 21))
        ef = int(rng.choice([8, 16, 32]))
        specs.append((sc, ef, 900 + i))
    return specs, rng


SERVE_SCALES = [16, 17, 18, 19, 20, 21, 22, 24]


def serve_graph_specs():
    return [(s, 16, 50 + s) for s in SERVE_SCALES]


def draw_source(rng, offs):
    """A random vertex of degree > 0 (the rule for multi-source and served queries)."""
    n = len(offs) - 1
    while True:
        v = int(rng.integers(n))
        if offs[v + 1] > offs[v]:
            return v


WORKLOADS = {
    "bfs-rmat24": dict(algo="bfs", graph="rmat", scale=24, edge_factor=16, seed=3,
                       symmetric=True, weighted=False, kernel="bfs_persistent",
                       metric="GTEPS (single-query BFS, RMAT-24 symmetrised)"),
    "sssp-rmat22": dict(algo="sssp", graph="rmat", scale=22, edge_factor=16, seed=2,
                        symmetric=True, weighted=True, kernel="sssp_persistent",
                        metric="GTEPS (single-query SSSP, RMAT-22 symmetrised, w in [1,255])"),
    "cc-rmat22": dict(algo="cc", graph="rmat", scale=22, edge_factor=16, seed=2,
                      symmetric=True, weighted=False, kernel="cc (all kernels)",
                      metric="GTEPS (connected components, RMAT-22 symmetrised)"),
    "pagerank-rmat24": dict(algo="pagerank", graph="rmat", scale=24, edge_factor=16, seed=3,
                            symmetric=False, weighted=False, kernel="pr_persistent", iters=20,
                            metric="GTEPS (pull PageRank, 20 iterations, RMAT-24 directed)"),
    "bfs-grid4096": dict(algo="bfs", graph="grid", scale=12, seed=0,
                         kernel="bfs_persistent+bfs_narrow",
                         metric="GTEPS (single-query BFS, 4096x4096 grid, source 4097)"),
    "msbfs-rmat23": dict(algo="msbfs", graph="rmat", scale=23, edge_factor=16, seed=4,
                         symmetric=True, weighted=False, kernel="msbfs_persistent", sources=64,
                         metric="GTEPS (64-source BFS in one launch, RMAT-23 symmetrised)"),
    "bfs-rmat26-managed": dict(algo="bfs", graph="rmat", scale=26, edge_factor=16, seed=3,
                               symmetric=True, weighted=False, kernel="bfs_persistent",
                               managed=True, budget_fraction=0.5,
                               metric="GTEPS (single-query BFS, RMAT-26 symmetrised, managed "
                                      "memory, device budget 50% of the CSR bytes)"),
    "batch-sssp256": dict(algo="batch", graph="rmat-set", seed=4, queries=256, kernel="batch_kernel "
                      "(cluster workers) + msssp_persistent / msssp_union (graphs of 2^21+ "
                      "edges, several per launch while their distance rows fit 2^23 entries)",
                      metric="queries/s (256 SSSP queries over 32 resident RMAT graphs, scales "
                             "14-20, edge factors 8-32, one batched call)"),
    "serve-mixed": dict(algo="serve", graph="rmat-set", seed=5, rate=8000, sweep_rates=[500, 2000],
                     sweep_queries=2000, step_queries=1000, sssp_fraction=0.5,
                     kernel="server lanes: batch_kernel slots + whole-GPU bfs/sssp/msssp launches",
                     metric="queries/s served (Poisson arrivals at 8,000/s, 8 resident RMAT graphs "
                            "s16-24, half SSSP), p50/p99 latency"),
    "msssp-rmat22": dict(algo="msssp", graph="rmat", scale=22, edge_factor=16, seed=2,
                         symmetric=True, weighted=True, kernel="msssp_persistent", sources=32,
                         metric="GTEPS (32-source SSSP in one launch, RMAT-22 symmetrised, w in [1,255])"),
}
DEFAULT_WORKLOAD = "bfs-rmat24"


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", FALLBACK_HBM_GBS)), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def alg_bytes(algo, n, m, nr, mr, iters=1, sources=1):
    """Algorithmic bytes of one launch.

    bfs:  4(n+1) offsets + 4 m_r column ids + 4n depth writes + 8 n_r frontier
          enqueue/dequeue (the top-down figure, also used for direction-
          optimised runs);
    sssp: as bfs with 8 m_r (column id + weight per relaxed edge);
    cc:   4(n+1) + 4m + 8n (labels read and written once);
    pagerank: per iteration 4(n+1) + 8m (column id + contribution) + 8n;
    msbfs: 4(n+1) + 4m + 8n (visit/frontier words) + 4 * sources * n depths;
    msssp: 4(n+1) + 8m (column id + weight, read once for all sources) +
           8 * sources * n (distance matrix initialised once, outputs written once).
    """
    if algo == "bfs":
        return 4 * (n + 1) + 4 * mr + 4 * n + 8 * nr
    if algo == "sssp":
        return 4 * (n + 1) + 8 * mr + 4 * n + 8 * nr
    if algo == "cc":
        return 4 * (n + 1) + 4 * m + 8 * n
    if algo == "pagerank":
        return iters * (4 * (n + 1) + 8 * m + 8 * n)
    if algo == "msbfs":
        return 4 * (n + 1) + 4 * m + 8 * n + 4 * sources * n
    if algo == "msssp":
        return 4 * (n + 1) + 8 * m + 8 * sources * n
    raise ValueError(algo)


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
            time.sleep(0.3)  # first sample before the timed region
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


def reduce_op(dist, x, op):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=op(dist))
    return float(t.item())


def reduce_max(dist, x):
    return reduce_op(dist, x, lambda d: d.ReduceOp.MAX)


def reduce_sum(dist, x):
    return reduce_op(dist, x, lambda d: d.ReduceOp.SUM)


def barrier(dist):
    if dist is not None:
        dist.barrier()


def host_threads():
    """Every core this process may run on (torchrun sets OMP_NUM_THREADS=1 for
    its workers; the CPU baselines ask for all cores explicitly)."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def workload_spec(args):
    w = dict(WORKLOADS[args.workload])
    if args.scale:
        w["scale"] = args.scale
    w["workload"] = args.workload if not args.scale else f"{args.workload}@scale{args.scale}"
    return w


def grid_source(side):
    return side + 1  # vertex (1, 1)


def msbfs_sources(n, offs_or_degree_fn, k, seed):
    """k distinct sources with degree > 0 drawn with a seeded generator."""
    rng = np.random.default_rng(seed)
    out = []
    seen = set()
    while len(out) < k:
        v = int(rng.integers(n))
        if v not in seen and offs_or_degree_fn(v) > 0:
            seen.add(v)
            out.append(v)
    return np.array(out, dtype=np.uint32)


# ---------------------------------------------------------------------------
# CPU path (the oracle's OpenMP versions; bounded samples)
def cpu_run(w, csr, csc, src, srcs, threads, budget_s=12.0, max_runs=5, nsrc=4):
    """Times the OpenMP version of the workload's algorithm on `threads` host
    threads (multi-source workloads: one run from each of the first `nsrc`
    sources).  Returns (units per second, sample description, results), the
    results being what the runs computed, for the parity check of the GPU
    output: {"rows": [(row, values), ...]} (row 0 for a single query, the
    source's row for multi-source workloads) or {} for PageRank, whose bounded
    sample runs fewer iterations than the GPU."""
    import oracle
    algo = w["algo"]
    times, units = [], 0
    results = {}
    t_start = time.perf_counter()
    if algo in ("bfs", "sssp"):
        fn = oracle.omp_bfs if algo == "bfs" else oracle.omp_sssp
        d, _ = fn(csr, src, threads)
        units = oracle.reached_edges(csr, d)
        results = {"rows": [(0, d)]}
        while len(times) < max_runs and (not times or time.perf_counter() - t_start < budget_s):
            times.append(fn(csr, src, threads)[1])
        desc = f"{len(times)} full {algo.upper()} runs from the source"
    elif algo == "cc":
        results = {"rows": [(0, oracle.omp_cc(csr, threads)[0])]}
        units = csr.m
        while len(times) < max_runs and (not times or time.perf_counter() - t_start < budget_s):
            times.append(oracle.omp_cc(csr, threads)[1])
        desc = f"{len(times)} full CC runs"
    elif algo == "pagerank":
        outdeg = np.diff(csr.offs.astype(np.int64)).astype(np.uint32)
        it = 2  # bounded sample: 2 iterations, rate per iteration-edge
        oracle.omp_pagerank(csc, outdeg, 0.85, it, threads)
        units = csr.m * it
        while len(times) < max_runs and (not times or time.perf_counter() - t_start < budget_s):
            times.append(oracle.omp_pagerank(csc, outdeg, 0.85, it, threads)[1])
        desc = f"{len(times)} runs of {it} pull iterations"
    elif algo in ("msbfs", "msssp"):
        fn = oracle.omp_bfs if algo == "msbfs" else oracle.omp_sssp
        per = []
        results = {"rows": []}
        for i, s in enumerate(srcs[:nsrc]):  # bounded sample: nsrc of the sources, one run each
            d, t = fn(csr, int(s), threads)
            per.append((oracle.reached_edges(csr, d), t))
            results["rows"].append((i, d))
        units = sum(p[0] for p in per)
        times = [sum(p[1] for p in per)]
        desc = (f"one OpenMP {'BFS' if algo == 'msbfs' else 'SSSP'} from each of the first "
                f"{min(nsrc, len(srcs))} of the {len(srcs)} sources")
    med = statistics.median(times)
    return units / med / 1e9, f"{desc}, median {med*1e3:.1f} ms, OpenMP level-synchronous", results


def parity_entry(res, results, what):
    """Compares rows of the GPU output `res` (1-D for one query, 2-D per
    source) with the CPU port's results; the bench line carries the outcome."""
    rows = results.get("rows", [])
    if not rows:
        return {"checked": "none in the bench (PageRank: tolerance tests in tests/)"}
    bad = 0
    for i, ref in rows:
        got = res[i] if res.ndim == 2 else res
        bad += int(np.count_nonzero(got.view(np.uint32) != ref))
    return {"checked": f"{len(rows)} {what} of the timed configuration against the oracle's "
                       "OpenMP port (bit-exact)", "mismatches": bad, "ok": bad == 0}


def host_graph(w):
    """The workload's graph generated on the host by the oracle (same bits)."""
    import oracle
    if w["graph"] == "grid":
        side = 1 << w["scale"]
        return oracle.grid(side, side, w.get("seed", 0), 0)
    flags = ((oracle.GEN_SYMMETRIC if w["symmetric"] else 0)
             | (oracle.GEN_WEIGHTED if w["weighted"] else 0) | oracle.GEN_RELABEL)
    return oracle.rmat(w["scale"], w["edge_factor"], w["seed"], flags)


# ---------------------------------------------------------------------------
def run_grus(args, dist, rank, local):
    import torch
    import grus_framework_gb300 as grus

    torch.cuda.set_device(local)
    grus.device_init(local)
    w = workload_spec(args)
    algo = w["algo"]
    if w["graph"] == "grid":
        side = 1 << w["scale"]
        g = grus.Graph.grid2d(side, side, w.get("seed", 0))
        src = grid_source(side)
    else:
        budget = 0
        if w.get("managed"):
            # the budget is a fraction of the CSR bytes, known once the graph exists
            g0 = grus.Graph.rmat(w["scale"], w["edge_factor"], w["seed"], symmetric=w["symmetric"],
                                 weighted=w["weighted"], relabel=True)
            budget = int(w["budget_fraction"] * (4 * (g0.n + 1) + 4 * g0.m))
            g0.free()
            w["budget_bytes"] = budget
        g = grus.Graph.rmat(w["scale"], w["edge_factor"], w["seed"], symmetric=w["symmetric"],
                            weighted=w["weighted"], relabel=True, managed=bool(w.get("managed")),
                            budget_bytes=budget)
        src = g.max_degree_vertex
    n, m = g.n, g.m
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    srcs = None
    iters = w.get("iters", 1)
    k = w.get("sources", 1)
    if algo in ("msbfs", "msssp"):
        offs_h, _, _ = g.copy_csr()
        srcs = msbfs_sources(n, lambda v: int(offs_h[v + 1]) - int(offs_h[v]), k, 4)
        del offs_h
    if algo == "pagerank":
        g.build_csc()

    def make_out(host):
        shape = (k, n) if algo in ("msbfs", "msssp") else (n,)
        dt = torch.float32 if algo == "pagerank" else torch.int32
        if host:
            return torch.empty(shape, dtype=dt, pin_memory=True)
        return torch.empty(shape, dtype=dt, device="cuda")

    def call(out, stats=False):
        if algo == "bfs":
            return grus.bfs(g, src, out=out, stream=stream, stats=stats)
        if algo == "sssp":
            return grus.sssp(g, src, out=out, stream=stream, stats=stats)
        if algo == "cc":
            return grus.cc(g, out=out, stream=stream, stats=stats)
        if algo == "pagerank":
            return grus.pagerank(g, 0.85, iters, out=out, stream=stream, stats=stats)
        if algo == "msssp":
            return grus.sssp_multi(g, srcs, out=out, stream=stream, stats=stats)
        return grus.bfs_multi(g, srcs, out=out, stream=stream, stats=stats)

    # BFS: the per-graph pull index (4 bytes per vertex) is built before the
    # first call, like the graph itself; its build time goes into the line
    index = None
    if algo == "bfs" and (w.get("symmetric", True) or w["graph"] == "grid"):
        index = {"bytes": 8 * n, "build_ms": round(g.build_index(), 3),
                 "what": "per vertex, an in-neighbour of high out-degree and the vertex's "
                         "out-degree, tested before the vertex's adjacency in pull levels"}
    out_dev = make_out(False)
    _, st = call(out_dev, stats=True)
    nr, mr = st["vertices_reached"], st["edges_reached"]
    launches = max(int(st["kernel_launches"]), 1)
    units = {"bfs": mr, "sssp": mr, "cc": m, "pagerank": m * iters, "msbfs": mr, "msssp": mr}[algo]
    for _ in range(args.warmup):
        call(out_dev)
    torch.cuda.synchronize()
    barrier(dist)

    # Each step's time is the pair of CUDA events the C ABI records on the
    # launching stream right before its first and after its last kernel
    # (stats["device_ms"]), so host work between a step's flush and its launch
    # (Python, ctypes) is not counted as device time; the events of this loop
    # around each call are kept as a cross-check that does include it.
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    step_ms = []
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ev[i][0].record(stream)
            _, st_i = call(out_dev, stats=True)
            ev[i][1].record(stream)
            step_ms.append(st_i["device_ms"])
        torch.cuda.synchronize()
    barrier(dist)
    outer_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = reduce_max(dist, sum(step_ms))
    ws = dist.get_world_size() if dist else 1
    total_units = reduce_sum(dist, units * args.steps)
    value = total_units / (total_ms * 1e-3) / 1e9
    mean_ms = sum(step_ms) / len(step_ms)

    # end to end through the public API: pinned host output, D2H inside
    out_host = make_out(True)
    call(out_host)
    e2e_s = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        stream.synchronize()
        t0 = time.perf_counter()
        call(out_host)
        e2e_s.append(time.perf_counter() - t0)
    e2e_total = reduce_max(dist, sum(e2e_s))
    e2e_value = total_units / e2e_total / 1e9
    d2h = out_host.numel() * 4
    h2d = 4 * (k if algo in ("msbfs", "msssp") else (1 if algo in ("bfs", "sssp") else 0))

    # cheap checks of the timed configuration (full parity lives in tests/)
    res = out_host.numpy()
    if algo in ("bfs", "sssp"):
        d = res.view(np.uint32)
        assert d[src] == 0 and int(np.count_nonzero(d != INFINIT)) == nr
    elif algo in ("msbfs", "msssp"):
        d = res.view(np.uint32)
        assert all(d[i, s] == 0 for i, s in enumerate(srcs))
    elif algo == "cc":
        lab = res.view(np.uint32)
        assert np.all(lab <= np.arange(n, dtype=np.uint32))
    else:
        assert np.isfinite(res).all()

    peak, peak_kind = measured_peaks()
    alg = alg_bytes(algo, n, m, nr, mr, iters, k)
    achieved = alg / (mean_ms * 1e-3) / 1e9
    traffic, traffic_note = None, None
    prof = ROOT / "profiles" / "dram_traffic.json"
    if prof.exists():
        rec = json.loads(prof.read_text()).get(w["workload"])
        if rec:
            traffic, traffic_note = rec.get("dram_bytes_per_launch"), rec.get("note")
    result = None
    if rank == 0:
        cpu = None
        parity = {"checked": "skipped (--no-cpu-baseline)"}
        if not args.no_cpu_baseline:
            import oracle
            offs, cols, wts = g.copy_csr()
            csr = oracle.CSR(offs, cols, wts)
            csc = None
            if algo == "pagerank":
                co, cc_, _ = g.copy_csc()
                csc = oracle.CSR(co, cc_)
            threads = host_threads()
            v, sample, cpu_results = cpu_run(w, csr, csc, src, srcs, threads)
            cpu = {"value": round(v, 4), "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": sample}
            parity = parity_entry(res, cpu_results,
                                  "source rows" if algo in ("msbfs", "msssp") else "result")
            # the same port on one thread, one run (one source for multi-source;
            # skipped above 2^30 edges, where it would take minutes)
            if csr.m <= (1 << 30):
                v1, sample1, _ = cpu_run(w, csr, csc, src, srcs, 1, budget_s=0.0, max_runs=1,
                                         nsrc=1)
                cpu["single_thread"] = {"value": round(v1, 4), "unit": UNIT, "cores": 1,
                                        "sample": sample1}
        clocks = clk.summary()
        cfg = {k_: v_ for k_, v_ in w.items() if k_ not in ("metric", "kernel")}
        cfg.update({"n": n, "m": m, "src": src if algo not in ("msbfs", "msssp") else f"{k} seeded (seed 4)",
                    "l2": "flushed (256 MB write) before each step",
                    "parallelism": f"replicas x{ws}", "levels": st["levels"],
                    "bottom_up_levels": st["bottom_up_levels"],
                    "vertices_reached": nr, "edges_reached": mr})
        if index:
            cfg["bfs_pull_index"] = index
        result = {
            "metric": w["metric"], "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(mean_ms, 4),
            "ms_per_step_outer_events": round(sum(outer_ms) / len(outer_ms), 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if algo == "pagerank" else "u32",
            "data": "synthetic (generated on device from the seed)",
            "config": cfg,
            "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "note": "public API call with a pinned host output buffer; graph " + (
                        "in managed memory, device budget %d bytes" % w["budget_bytes"]
                        if w.get("managed") else "resident in HBM")},
            "gpu_launches": launches * args.steps,
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "traffic_note": traffic_note, "peak_source": peak_kind,
                         "kernel": w["kernel"], "algorithmic_bytes_per_launch": alg},
            "cpu_baseline": cpu,
            "parity": parity,
            "clocks": clocks,
        }
    g.free()
    return result


# ---------------------------------------------------------------------------
# batched and served forms
QPS = "queries/s"


def sssp_or_bfs_bytes(algo_id, n, deg, d):
    """Algorithmic bytes of one BFS (algo 0) or SSSP (algo 1) query from its result."""
    reached = d != INFINIT
    nr = int(np.count_nonzero(reached))
    mr = int(deg[reached].sum())
    return alg_bytes("sssp" if algo_id == 1 else "bfs", n, 0, nr, mr)


def cpu_queries(graphs_host, queries, threads):
    """OpenMP BFS/SSSP of `queries` ((graph, algo, src) tuples) on host CSRs.
    Returns (queries per second, total seconds, the results in query order)."""
    import oracle
    total = 0.0
    results = []
    for gi, algo_id, src in queries:
        fn = oracle.omp_sssp if algo_id == 1 else oracle.omp_bfs
        d, t = fn(graphs_host[gi], int(src), threads)
        total += t
        results.append(d)
    return len(queries) / total, total, results


def roofline_entry(alg, seconds, traffic_key, kernel, note=None):
    peak, peak_kind = measured_peaks()
    achieved = alg / seconds / 1e9
    traffic, note = None, None
    prof = ROOT / "profiles" / "dram_traffic.json"
    if prof.exists():
        rec = json.loads(prof.read_text()).get(traffic_key)
        if rec:
            traffic, note = rec.get("dram_bytes_per_launch"), rec.get("note")
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "traffic_note": note,
            "peak_source": peak_kind, "kernel": kernel, "algorithmic_bytes_per_launch": alg,
            **({"algorithmic_bytes_note": note} if note else {})}


def run_batch(args, dist, rank, local):
    """256 SSSP queries over 32 resident graphs in one batched call per step."""
    import ctypes
    import torch
    import grus_framework_gb300 as grus

    torch.cuda.set_device(local)
    grus.device_init(local)
    w = workload_spec(args)
    specs, rng = batch_graph_specs(w["seed"])
    gs = [grus.Graph.rmat(sc, ef, sd, symmetric=True, weighted=True, relabel=True)
          for sc, ef, sd in specs]
    offs = [g.copy_offsets() for g in gs]
    degs = [np.diff(o.astype(np.int64)) for o in offs]
    queries = []
    for i in range(w["queries"]):
        gi = i % len(gs)
        queries.append((gi, grus.ALGO_SSSP, draw_source(rng, offs[gi])))
    # the project's autotuner chooses the engine's knobs for this mix (cached
    # by graph set and mix; tuned here, outside the timed region, when new)
    tuning = {"source": "library defaults (--no-tune)"}
    bkw = {}
    if not args.no_tune:
        from grus_framework_gb300 import tuning_cache
        tc = tuning_cache.load_or_tune_batch(gs, queries)
        bkw = tc["config"]
        tuning = {"source": "cache" if tc["cached"] else "grus_batch_autotune, this run",
                  "config": bkw, "tuned_device_ms": round(tc["device_ms"], 3)}
    b = grus.Batch(gs, **bkw)
    layout, total = b.layout(queries)
    out = torch.empty(total, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    st = b.run(queries, out, layout, use_graph=True, stats=True)
    launches = max(int(st["kernel_launches"]), 1)
    for _ in range(args.warmup):
        b.run(queries, out, layout, use_graph=True)
    torch.cuda.synchronize()
    barrier(dist)
    step_ms = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            step_ms.append(b.run(queries, out, layout, use_graph=True, stats=True)["device_ms"])
        torch.cuda.synchronize()
    barrier(dist)
    nq = len(queries)
    total_ms = reduce_max(dist, sum(step_ms))
    value = reduce_sum(dist, nq * args.steps) / (total_ms * 1e-3)
    mean_ms = sum(step_ms) / len(step_ms)

    # end to end: the batched call plus every result copied to pinned host memory
    out_host = torch.empty(total, dtype=torch.int32, pin_memory=True)
    e2e_s = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.run(queries, out, layout, use_graph=True)
        out_host.copy_(out)
        e2e_s.append(time.perf_counter() - t0)
    e2e_value = reduce_sum(dist, nq * args.steps) / reduce_max(dist, sum(e2e_s))
    res = out_host.numpy().view(np.uint32)
    alg = 0
    for (gi, algo_id, src), off in zip(queries, layout):
        d = res[off: off + gs[gi].n]
        assert d[src] == 0
        alg += sssp_or_bfs_bytes(algo_id, gs[gi].n, degs[gi], d)

    # the comparison the batched form is for: the same queries as plain calls
    outs = [torch.empty(g.n, dtype=torch.int32, device="cuda") for g in gs]
    for gi, _, src in queries[:32]:
        grus.sssp(gs[gi], src, out=outs[gi])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for gi, _, src in queries:
        grus.sssp(gs[gi], src, out=outs[gi])
    torch.cuda.synchronize()
    plain_qps = nq / (time.perf_counter() - t0)

    result = None
    if rank == 0:
        cpu = None
        parity = {"checked": "skipped (--no-cpu-baseline)"}
        if not args.no_cpu_baseline:
            sample = queries[:16]
            hosts = {}
            for gi, _, _ in sample:
                if gi not in hosts:
                    import oracle
                    o_, c_, wt_ = gs[gi].copy_csr()
                    hosts[gi] = oracle.CSR(o_, c_, wt_)
            threads = host_threads()
            v, sec, cpu_res = cpu_queries(hosts, sample, threads)
            v1, sec1, _ = cpu_queries(hosts, sample[:4], 1)
            bad = sum(int(np.count_nonzero(res[off:off + gs[gi].n] != ref))
                      for (gi, _, _), off, ref in zip(sample, layout, cpu_res))
            parity = {"checked": f"the first {len(sample)} of the {nq} results against the "
                                 "oracle's OpenMP port (bit-exact)", "mismatches": bad,
                      "ok": bad == 0}
            cpu = {"value": round(v, 2), "unit": QPS, "cores": threads, "kind": "port",
                   "sample": f"OpenMP SSSP of the first {len(sample)} queries, {sec:.2f} s",
                   "single_thread": {"value": round(v1, 2), "unit": QPS, "cores": 1,
                                     "sample": f"the first 4 queries, {sec1:.2f} s"}}
        info = b.info()
        cfg = {"workload": w["workload"], "graphs": len(gs),
               "graph_specs": "RMAT scale 14-20, edge factor 8/16/32 drawn with seed 4, "
                              "generator seeds 900-931, symmetrised, w in [1,255]",
               "queries": nq, "sources": "degree > 0, seed 4", "sum_n": int(sum(g.n for g in gs)),
               "sum_m": int(sum(g.m for g in gs)), "workers": info["workers"],
               "cluster_size": info["cluster_size"], "big_edges": info["big_edges"],
               "launch_entries": info["launch_entries"], "tuning": tuning,
               "l2": "flushed (256 MB write) before each step", "parallelism": f"replicas x{dist.get_world_size() if dist else 1}"}
        result = {
            "metric": w["metric"], "value": round(value, 1), "unit": QPS,
            "n_gpus": dist.get_world_size() if dist else 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(mean_ms, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (generated on device from the seeds)", "config": cfg,
            "e2e": {"value": round(e2e_value, 1), "unit": QPS,
                    "h2d_bytes_per_step": nq * ctypes.sizeof(grus.Query),
                    "d2h_bytes_per_step": int(total) * 4,
                    "note": "batched call through the public API, every result copied to "
                            "pinned host memory inside the timed region"},
            "plain_back_to_back": {"value": round(plain_qps, 1), "unit": QPS,
                                   "note": "the same 256 queries as plain grus_sssp calls, "
                                           "device outputs, host clock"},
            "gpu_launches": launches * args.steps,
            "roofline": roofline_entry(alg, mean_ms * 1e-3, w["workload"], w["kernel"]),
            "cpu_baseline": cpu, "parity": parity, "clocks": clk.summary(),
        }
    b.free()
    return result


def serve_stream(srv, grus, gs, qo, rng, offs, rate, nq, frac, copy=None):
    """Submits nq queries at Poisson arrivals of `rate` per second and polls
    their completions.  Returns (seconds, latencies in us, errors, d2h bytes)."""
    qs = []
    for _ in range(nq):
        gi = int(rng.integers(len(gs)))
        algo_id = grus.ALGO_SSSP if rng.random() < frac else grus.ALGO_BFS
        qs.append((gi, algo_id, draw_source(rng, offs[gi])))
    arr = np.cumsum(rng.exponential(1.0 / rate, size=nq))
    done = {}
    d2h = 0
    t0 = time.perf_counter()
    i = 0
    while len(done) < nq and time.perf_counter() - t0 < 300:
        now = time.perf_counter() - t0
        while i < nq and arr[i] <= now:
            gi, algo_id, src = qs[i]
            srv.submit(gi, algo_id, src, qo[gi][i % len(qo[gi])], i)
            i += 1
        comp = srv.poll(512, wait_ms=0 if i < nq else 1)
        for tag, stt, lat in comp:
            done[tag] = (stt, lat)
            if copy is not None:
                gi = qs[tag][0]
                copy(gi, qo[gi][tag % len(qo[gi])])
                d2h += gs[gi].n * 4
    dt = time.perf_counter() - t0
    lat = np.array([v[1] for v in done.values()])
    errors = sum(1 for v in done.values() if v[0] != 0) + (nq - len(done))
    return dt, lat, errors, d2h, len(done)


def run_serve(args, dist, rank, local):
    """Poisson query stream against 8 resident graphs through the server."""
    import torch
    import grus_framework_gb300 as grus

    torch.cuda.set_device(local)
    grus.device_init(local)
    w = workload_spec(args)
    gs = [grus.Graph.rmat(sc, ef, sd, symmetric=True, weighted=True, relabel=True)
          for sc, ef, sd in serve_graph_specs()]
    offs = [g.copy_offsets() for g in gs]
    degs = [np.diff(o.astype(np.int64)) for o in offs]
    rng = np.random.default_rng(w["seed"])
    frac = w["sssp_fraction"]
    # per-query algorithmic bytes of each (graph, algorithm), from one plain
    # query per pair (random sources of degree > 0 reach the giant component)
    per_q = {}
    outs = [torch.empty(g.n, dtype=torch.int32, device="cuda") for g in gs]
    for gi, g in enumerate(gs):
        src = draw_source(rng, offs[gi])
        for algo_id, fn in ((grus.ALGO_BFS, grus.bfs), (grus.ALGO_SSSP, grus.sssp)):
            d = fn(g, src, out=outs[gi]).cpu().numpy().view(np.uint32)
            per_q[(gi, algo_id)] = sssp_or_bfs_bytes(algo_id, g.n, degs[gi], d)
    # plain back-to-back on 400 queries of the same mix
    plain = []
    for _ in range(400):
        gi = int(rng.integers(len(gs)))
        plain.append((gi, grus.ALGO_SSSP if rng.random() < frac else grus.ALGO_BFS,
                      draw_source(rng, offs[gi])))
    for gi, algo_id, src in plain[:16]:
        (grus.sssp if algo_id else grus.bfs)(gs[gi], src, out=outs[gi])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for gi, algo_id, src in plain:
        (grus.sssp if algo_id else grus.bfs)(gs[gi], src, out=outs[gi])
        torch.cuda.synchronize()
    plain_qps = len(plain) / (time.perf_counter() - t0)

    qo = [[torch.empty(g.n, dtype=torch.int32, device="cuda") for _ in range(16)] for g in gs]
    # the server's knobs from the project's autotuner: saturated bursts of a
    # mix drawn like the stream's (its own seed), cached by graph set and mix
    tuning = {"source": "library defaults (--no-tune)"}
    skw = {}
    if not args.no_tune:
        from grus_framework_gb300 import tuning_cache
        trng = np.random.default_rng(w["seed"] + 1000)
        tq = []
        for _ in range(600):
            gi = int(trng.integers(len(gs)))
            tq.append((gi, grus.ALGO_SSSP if trng.random() < frac else grus.ALGO_BFS,
                       draw_source(trng, offs[gi])))
        tc = tuning_cache.load_or_tune_server(gs, tq)
        skw = tc["config"]
        tuning = {"source": "cache" if tc["cached"] else "grus_server_autotune, this run",
                  "config": skw, "tuned_saturated_qps": round(tc["qps"], 1),
                  "mix": "600 queries drawn like the stream (seed + 1000)"}
    srv = grus.Server(gs, **skw)
    for _ in range(args.warmup):
        serve_stream(srv, grus, gs, qo, rng, offs, w["rate"], 200, frac)
    torch.cuda.synchronize()
    barrier(dist)
    secs, lats, errors, completed = 0.0, [], 0, 0
    st0 = srv.stats()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            dt, lat, err, _, nd = serve_stream(srv, grus, gs, qo, rng, offs, w["rate"],
                                               w["step_queries"], frac)
            secs += dt
            lats.append(lat)
            errors += err
            completed += nd
    barrier(dist)
    st1 = srv.stats()
    launches = st1["kernel_launches"] - st0["kernel_launches"]
    lat_all = np.concatenate(lats)
    value = reduce_sum(dist, completed) / reduce_max(dist, secs)
    # end to end: every completed result copied to pinned host memory as it completes
    host = [torch.empty(g.n, dtype=torch.int32, pin_memory=True) for g in gs]
    cs = torch.cuda.Stream()

    def copy(gi, buf):
        with torch.cuda.stream(cs):
            host[gi].copy_(buf, non_blocking=True)

    e_secs, e_done, e_d2h = 0.0, 0, 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, _, err, d2h, nd = serve_stream(srv, grus, gs, qo, rng, offs, w["rate"],
                                          w["step_queries"], frac, copy=copy)
        cs.synchronize()
        e_secs += time.perf_counter() - t0
        e_done += nd
        e_d2h += d2h
        errors += err
    e2e_value = reduce_sum(dist, e_done) / reduce_max(dist, e_secs)
    sweep = []
    for rate in w["sweep_rates"]:
        dt, lat, err, _, nd = serve_stream(srv, grus, gs, qo, rng, offs, rate,
                                           w["sweep_queries"], frac)
        sweep.append({"offered_per_s": rate, "queries": int(nd), "queries_per_s": round(nd / dt, 1),
                      "p50_ms": round(float(np.percentile(lat, 50)) / 1e3, 3),
                      "p99_ms": round(float(np.percentile(lat, 99)) / 1e3, 3), "errors": int(err)})
        errors += err
    # the parity sample: 12 queries of the mix served once more into their own
    # outputs (compared below with the CPU port's results of the same queries)
    check = plain[:12]
    check_out = [torch.full((gs[gi].n,), -7, dtype=torch.int32, device="cuda") for gi, _, _ in check]
    for j, (gi, algo_id, src) in enumerate(check):
        srv.submit(gi, algo_id, src, check_out[j], 1 << 40 | j)
    got_status = {}
    t_chk = time.perf_counter()
    while len(got_status) < len(check) and time.perf_counter() - t_chk < 60:
        for tag, stt, _ in srv.poll(64, wait_ms=5):
            got_status[tag] = stt
    srv.close()
    # algorithmic bytes of the timed queries: the mean per-query figure of the mix
    mean_q = sum((frac if a == grus.ALGO_SSSP else 1 - frac) * v / len(gs)
                 for (gi, a), v in per_q.items())
    result = None
    if rank == 0:
        cpu = None
        parity = {"checked": "skipped (--no-cpu-baseline)"}
        if not args.no_cpu_baseline:
            import oracle
            sample = check
            hosts = {}
            for gi, _, _ in sample:
                if gi not in hosts:
                    o_, c_, wt_ = gs[gi].copy_csr()
                    hosts[gi] = oracle.CSR(o_, c_, wt_)
            threads = host_threads()
            v, sec, cpu_res = cpu_queries(hosts, sample, threads)
            bad = sum(int(np.count_nonzero(o.cpu().numpy().view(np.uint32) != ref))
                      for o, ref in zip(check_out, cpu_res))
            bad += sum(1 for stt in got_status.values() if stt != 0) + len(check) - len(got_status)
            parity = {"checked": f"{len(check)} queries of the mix served into their own outputs "
                                 "against the oracle's OpenMP port (bit-exact)",
                      "mismatches": bad, "ok": bad == 0}
            cpu = {"value": round(v, 2), "unit": QPS, "cores": threads, "kind": "port",
                   "sample": f"OpenMP BFS/SSSP of {len(sample)} queries of the mix, {sec:.2f} s"}
        cfg = {"workload": w["workload"], "graphs": "RMAT scales 16-22 and 24, edge factor 16, "
                                                     "seeds 50+scale, symmetrised, w in [1,255]",
               "offered_per_s": w["rate"], "queries": int(completed), "sssp_fraction": frac,
               "sources": "degree > 0, seed 5", "tuning": tuning,
               "big_launches": int(st1["big_launches"] - st0["big_launches"]),
               "big_queries": int(st1["big_queries"] - st0["big_queries"]), "errors": int(errors),
               "parallelism": f"replicas x{dist.get_world_size() if dist else 1}"}
        result = {
            "metric": w["metric"], "value": round(value, 1), "unit": QPS,
            "n_gpus": dist.get_world_size() if dist else 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(secs / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (generated on device from the seeds)", "config": cfg,
            "latency": {"p50_ms": round(float(np.percentile(lat_all, 50)) / 1e3, 3),
                        "p99_ms": round(float(np.percentile(lat_all, 99)) / 1e3, 3),
                        "measured": "submission to completion, per query, host clock"},
            "sweep": sweep,
            "e2e": {"value": round(e2e_value, 1), "unit": QPS, "h2d_bytes_per_step": 16 * w["step_queries"],
                    "d2h_bytes_per_step": int(e_d2h / max(args.steps, 1)),
                    "note": "the same stream with every result copied to pinned host memory as "
                            "it completes"},
            "plain_back_to_back": {"value": round(plain_qps, 1), "unit": QPS,
                                   "note": "400 queries of the same mix as plain calls, one at a "
                                           "time, host clock"},
            "gpu_launches": int(launches),
            "roofline": roofline_entry(int(mean_q * completed), secs, w["workload"], w["kernel"],
                                       note="all queries of the timed region: per query the "
                                            "BFS/SSSP figure of its graph, averaged over the mix"),
            "cpu_baseline": cpu, "parity": parity, "clocks": clk.summary(),
        }
    return result



def run_reference_queries(args, w):
    """CPU path of the batched / served workloads: the same graphs generated on
    the host, the same queries, each step a bounded sample of them through the
    OpenMP port on all host cores (queries per second)."""
    import oracle
    flags = oracle.GEN_SYMMETRIC | oracle.GEN_WEIGHTED | oracle.GEN_RELABEL
    if w["algo"] == "batch":
        specs, rng = batch_graph_specs(w["seed"])
        hosts = [oracle.rmat(sc, ef, sd, flags) for sc, ef, sd in specs]
        queries = [(i % len(hosts), 1, draw_source(rng, hosts[i % len(hosts)].offs))
                   for i in range(w["queries"])]
        per_step = 8
    else:
        hosts = [oracle.rmat(sc, ef, sd, flags) for sc, ef, sd in serve_graph_specs()]
        rng = np.random.default_rng(w["seed"])
        queries = []
        for _ in range(400):
            gi = int(rng.integers(len(hosts)))
            queries.append((gi, 1 if rng.random() < w["sssp_fraction"] else 0,
                            draw_source(rng, hosts[gi].offs)))
        per_step = 6
    threads = host_threads()
    for k in range(max(args.warmup - 1, 0)):
        cpu_queries(hosts, queries[:1], threads)
    rates = []
    for k in range(args.steps):
        sample = [queries[(k * per_step + j) % len(queries)] for j in range(per_step)]
        rates.append(cpu_queries(hosts, sample, threads)[0])
    value = statistics.median(rates)
    cfg = {"workload": w["workload"], "graphs": len(hosts), "queries_per_step": per_step,
           "sum_n": int(sum(h.n for h in hosts)), "sum_m": int(sum(h.m for h in hosts))}
    return {
        "metric": w["metric"], "value": round(value, 2), "unit": QPS, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic (generated on the host from the seeds)",
        "impl": "reference", "config": cfg,
        "cpu_baseline": {"value": round(value, 2), "unit": QPS, "cores": threads, "kind": "port",
                         "sample": f"each step: {per_step} of the queries, one OpenMP BFS/SSSP "
                                   "each, back to back"},
        "e2e": {"value": round(value, 2), "unit": QPS, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference(args, dist, rank):
    """CPU path: the oracle's OpenMP version on the host cores (rank 0 only)."""
    if rank != 0:
        return None
    import oracle
    w = workload_spec(args)
    algo = w["algo"]
    if algo in ("batch", "serve"):
        return run_reference_queries(args, w)
    g = host_graph(w)
    src = grid_source(1 << w["scale"]) if w["graph"] == "grid" else oracle.max_degree_vertex(g)
    csc = oracle.csr_to_csc(g) if algo == "pagerank" else None
    srcs = None
    if algo in ("msbfs", "msssp"):
        srcs = msbfs_sources(g.n, lambda v: int(g.offs[v + 1]) - int(g.offs[v]), w["sources"], 4)
    threads = host_threads()
    for _ in range(max(args.warmup - 1, 0)):
        cpu_run(w, g, csc, src, srcs, threads, budget_s=0.0, max_runs=1)
    rates = []
    sample = ""
    for _ in range(args.steps):
        r, sample, _ = cpu_run(w, g, csc, src, srcs, threads, budget_s=0.0, max_runs=1)
        rates.append(r)
    value = statistics.median(rates)
    cfg = {k_: v_ for k_, v_ in w.items() if k_ not in ("metric", "kernel")}
    cfg.update({"n": g.n, "m": g.m, "src": src})
    return {
        "metric": w["metric"], "value": round(value, 4), "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if algo == "pagerank" else "u32",
        "data": "synthetic (generated on the host from the seed)", "impl": "reference",
        "config": cfg,
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"each step: {sample}"},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def systems_summary(args, dist, rank, local):
    """The batched and served forms, measured in the same process after the
    headline workload: one summary per form, for the default bench line."""
    out = {}
    for name, workload, fn in (("batch", "batch-sssp256", run_batch),
                               ("serve", "serve-mixed", run_serve)):
        a = argparse.Namespace(**vars(args))
        a.workload, a.scale = workload, 0
        r = fn(a, dist, rank, local)
        if rank != 0 or r is None:
            continue
        plain = r["plain_back_to_back"]["value"]
        e = {"workload": workload, "metric": r["metric"], "qps": r["value"],
             "e2e_qps": r["e2e"]["value"], "plain_back_to_back_qps": plain,
             "steps": r["steps"], "warmup": r["warmup"], "ms_per_step": r["ms_per_step"],
             "gpu_launches": r["gpu_launches"], "parity": r.get("parity"),
             "clocks": r.get("clocks")}
        if name == "batch":
            # host clock against host clock: the e2e rate (batched call plus
            # every result copied to the host) over plain calls' rate
            e["speedup_vs_plain"] = round(r["e2e"]["value"] / plain, 2)
            e["speedup_note"] = ("e2e queries/s (host clock, results copied to the host) over "
                                 "back-to-back plain grus_sssp calls (host clock)")
        else:
            e["speedup_vs_plain"] = round(r["value"] / plain, 2)
            e["speedup_note"] = ("served queries/s over back-to-back plain calls of the same "
                                 "mix, both on the host clock")
            e["p50_ms"] = r["latency"]["p50_ms"]
            e["p99_ms"] = r["latency"]["p99_ms"]
            e["sweep"] = r.get("sweep")
        out[name] = e
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["grus", "reference"], default="grus")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--scale", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="batched/served workloads: library defaults instead of the autotuner's")
    ap.add_argument("--no-systems", action="store_true",
                    help="default workload only: skip the batched and served summaries")
    args = ap.parse_args()
    if args.impl == "grus":
        args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_env()
    dist = init_dist(ws)
    algo = WORKLOADS[args.workload]["algo"]
    if args.impl == "reference":
        res = run_reference(args, dist, rank)
    elif algo == "batch":
        res = run_batch(args, dist, rank, local)
    elif algo == "serve":
        res = run_serve(args, dist, rank, local)
    else:
        res = run_grus(args, dist, rank, local)
        if args.workload == DEFAULT_WORKLOAD and not args.scale and not args.no_systems:
            sysres = systems_summary(args, dist, rank, local)
            if rank == 0 and res is not None:
                res["systems"] = sysres
    failed = False
    if rank == 0 and res is not None:
        print(json.dumps(res))
        checks = [res.get("parity")] + [v.get("parity") for v in res.get("systems", {}).values()]
        failed = any(c is not None and c.get("ok") is False for c in checks)
        if failed:
            print("bench: GPU results differ from the oracle's (see \"parity\")", file=sys.stderr)
    if dist is not None:
        dist.destroy_process_group()
    if failed:
        sys.exit(3)


if __name__ == "__main__":
    main()
