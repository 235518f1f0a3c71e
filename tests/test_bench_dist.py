"""CPU: the multi-process paths of bench.py -- world size 2 over gloo.

Replicas only: each rank runs its own traversal and the ranks meet only in
the max/sum reductions of the timing; the reference arm runs on rank 0 and
the other ranks exit without work."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _reduce_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    dist = bench.init_dist(world)
    mx = bench.reduce_max(dist, 1.5 + rank)
    sm = bench.reduce_sum(dist, 10.0 * (rank + 1))
    bench.barrier(dist)
    q.put((rank, mx, sm))
    dist.destroy_process_group()


def test_reductions_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29611
    ps = [ctx.Process(target=_reduce_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [2.5, 2.5]  # max over ranks
    assert [g[2] for g in got] == [30.0, 30.0]  # sum over ranks


def test_reference_arm_under_torchrun_prints_one_line():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", "29612", str(ROOT / "bench.py"),
           "--impl", "reference", "--scale", "12", "--steps", "2", "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["cores"] >= 1 and d["e2e"]["h2d_bytes_per_step"] == 0


def test_query_workload_helpers():
    """The graph sets and source rule of the batched and served workloads are
    deterministic, and the CPU rate of a query sample is positive."""
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import bench
    import oracle
    a, _ = bench.batch_graph_specs(4)
    b, _ = bench.batch_graph_specs(4)
    assert a == b and len(a) == 32
    assert all(14 <= sc <= 20 and ef in (8, 16, 32) for sc, ef, _ in a)
    assert [sc for sc, _, _ in bench.serve_graph_specs()] == [16, 17, 18, 19, 20, 21, 22, 24]
    g = oracle.rmat(10, 8, 3, oracle.GEN_SYMMETRIC | oracle.GEN_WEIGHTED | oracle.GEN_RELABEL)
    rng = np.random.default_rng(5)
    srcs = [bench.draw_source(rng, g.offs) for _ in range(50)]
    assert all(g.offs[v + 1] > g.offs[v] for v in srcs)
    qps, sec, res = bench.cpu_queries({0: g}, [(0, 1, srcs[0]), (0, 0, srcs[1])], 2)
    assert qps > 0 and sec > 0
    # the results the bench's parity check compares against: the oracle's
    assert np.array_equal(res[0], oracle.sssp(g, srcs[0]))
    assert np.array_equal(res[1], oracle.bfs(g, srcs[1]))


def test_parity_entry_counts_mismatches():
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import bench
    ref = np.arange(10, dtype=np.uint32)
    ok = bench.parity_entry(ref.copy(), {"rows": [(0, ref)]}, "result")
    assert ok["ok"] and ok["mismatches"] == 0
    bad = ref.copy()
    bad[3] = 99
    e = bench.parity_entry(bad, {"rows": [(0, ref)]}, "result")
    assert not e["ok"] and e["mismatches"] == 1
    two = np.stack([ref, bad])
    e2 = bench.parity_entry(two, {"rows": [(0, ref), (1, ref)]}, "source rows")
    assert e2["mismatches"] == 1
    assert "none" in bench.parity_entry(ref, {}, "result")["checked"]

