"""GPU: parity at the sizes the bench times, for the batched, served,
multi-source and managed configurations, with exactly the bench's inputs
(bench.py's graph sets, source draws and seeds).

Each test compares every result with the same query run alone through the
plain entry point (the batched and served forms promise results identical to
single queries) and a sample of them with the oracle, so each configuration
is also closed against the CPU restatement at its own size:

  * 64-source BFS on RMAT-23 (seed 4 sources): all 64 rows against 64 single
    BFS calls, 4 rows against the oracle;
  * 256 SSSP queries over the 32 RMAT graphs of scales 14-20: all against
    single SSSP calls, 16 against the oracle (Dijkstra);
  * the served stream: 200 Poisson-arrival BFS/SSSP queries against the 8
    resident RMAT graphs of scales 16-24, all against single calls, one per
    graph against the oracle;
  * BFS on RMAT-26 in managed memory with half the CSR bytes as device
    budget, against the oracle.
"""
import time

import numpy as np
import pytest

import bench

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def _host(g):
    import oracle
    offs, cols, wts = g.copy_csr()
    return oracle.CSR(offs, cols, wts)


def test_msbfs_rmat23_64_sources_at_size(grus, oracle_mod):
    g = grus.Graph.rmat(23, 16, 4, symmetric=True)
    offs = g.copy_offsets()
    srcs = bench.msbfs_sources(g.n, lambda v: int(offs[v + 1]) - int(offs[v]), 64, 4)
    d = grus.bfs_multi(g, srcs)
    for i, s in enumerate(srcs):
        assert np.array_equal(d[i], grus.bfs(g, int(s))), f"row {i} (source {s})"
    h = _host(g)
    for i in (0, 21, 42, 63):
        assert np.array_equal(d[i], oracle_mod.bfs(h, int(srcs[i]))), f"row {i} vs oracle"
    g.free()


def test_batch_sssp256_at_size(grus, oracle_mod):
    torch = pytest.importorskip("torch")
    specs, rng = bench.batch_graph_specs(4)
    gs = [grus.Graph.rmat(sc, ef, sd, symmetric=True, weighted=True) for sc, ef, sd in specs]
    offs = [g.copy_offsets() for g in gs]
    queries = [(i % len(gs), grus.ALGO_SSSP, bench.draw_source(rng, offs[i % len(gs)]))
               for i in range(256)]
    b = grus.Batch(gs)
    layout, total = b.layout(queries)
    out = torch.full((total,), -7, dtype=torch.int32, device="cuda")
    b.run(queries, out, layout, use_graph=True)
    res = out.cpu().numpy().view(np.uint32)
    for qi, ((gi, _, src), o) in enumerate(zip(queries, layout)):
        alone = grus.sssp(gs[gi], src)
        assert np.array_equal(res[o:o + gs[gi].n], alone), f"query {qi}"
    for qi in range(16):  # graphs 0-15, one query each
        gi, _, src = queries[qi]
        ref = oracle_mod.sssp(_host(gs[gi]), src)
        assert np.array_equal(res[layout[qi]:layout[qi] + gs[gi].n], ref), f"query {qi} vs oracle"
    b.free()
    for g in gs:
        g.free()


def test_serve_mixed_stream_at_size(grus, oracle_mod):
    torch = pytest.importorskip("torch")
    gs = [grus.Graph.rmat(sc, ef, sd, symmetric=True, weighted=True)
          for sc, ef, sd in bench.serve_graph_specs()]
    offs = [g.copy_offsets() for g in gs]
    rng = np.random.default_rng(5)
    nq, rate = 200, 8000.0
    qs = []
    for _ in range(nq):
        gi = int(rng.integers(len(gs)))
        algo = grus.ALGO_SSSP if rng.random() < 0.5 else grus.ALGO_BFS
        qs.append((gi, algo, bench.draw_source(rng, offs[gi])))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=nq))
    outs = [torch.full((gs[gi].n,), -7, dtype=torch.int32, device="cuda") for gi, _, _ in qs]
    srv = grus.Server(gs)
    done = {}
    t0 = time.perf_counter()
    i = 0
    while len(done) < nq and time.perf_counter() - t0 < 300:
        now = time.perf_counter() - t0
        while i < nq and arrivals[i] <= now:
            gi, algo, src = qs[i]
            srv.submit(gi, algo, src, outs[i], i)
            i += 1
        for tag, status, _ in srv.poll(256, wait_ms=0 if i < nq else 1):
            done[tag] = status
    srv.close()
    assert len(done) == nq and all(s == 0 for s in done.values())
    for qi, (gi, algo, src) in enumerate(qs):
        fn = grus.sssp if algo == grus.ALGO_SSSP else grus.bfs
        got = outs[qi].cpu().numpy().view(np.uint32)
        assert np.array_equal(got, fn(gs[gi], src)), f"query {qi}"
    # one query per graph against the oracle: BFS on the two largest graphs
    # (a serial Dijkstra there would take minutes), the first query otherwise
    for gi in range(len(gs)):
        want = grus.ALGO_BFS if gi >= len(gs) - 2 else None
        cand = [q for q, (g_, a, _) in enumerate(qs) if g_ == gi and (want is None or a == want)]
        if not cand:
            continue
        qi = cand[0]
        _, algo, src = qs[qi]
        h = _host(gs[gi])
        ref = (oracle_mod.sssp if algo == grus.ALGO_SSSP else oracle_mod.bfs)(h, src)
        assert np.array_equal(outs[qi].cpu().numpy().view(np.uint32), ref), f"query {qi} vs oracle"
    for g in gs:
        g.free()


def test_managed_rmat26_half_budget_against_oracle(grus, oracle_mod):
    torch = pytest.importorskip("torch")
    g0 = grus.Graph.rmat(26, 16, 3, symmetric=True)
    budget = (4 * (g0.n + 1) + 4 * g0.m) // 2
    src = g0.max_degree_vertex
    g0.free()
    g = grus.Graph.rmat(26, 16, 3, symmetric=True, managed=True, budget_bytes=budget)
    assert g.info().budget_bytes == budget
    d = torch.empty(g.n, dtype=torch.int32, device="cuda")
    grus.bfs(g, src, out=d)
    torch.cuda.synchronize()
    got = d.cpu().numpy().view(np.uint32)
    del d
    h = _host(g)
    g.free()
    assert np.array_equal(got, oracle_mod.bfs(h, src))
