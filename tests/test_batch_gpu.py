"""GPU: batched queries (many graphs, many BFS/SSSP queries, one launch of
cluster workers) -- every result bit-exact against the single-query path,
plain launch and CUDA-graph replay, several cluster sizes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graphs(grus):
    gs = []
    for i, (scale, ef) in enumerate([(10, 8), (11, 16), (12, 32), (13, 8), (12, 16), (9, 4)]):
        gs.append(grus.Graph.rmat(scale, ef, 100 + i, symmetric=True, weighted=True))
    gs.append(grus.Graph.grid2d(40, 50, seed=7, weighted=True))
    return gs


def make_queries(grus, graphs, count, seed):
    rng = np.random.default_rng(seed)
    q = []
    for _ in range(count):
        gi = int(rng.integers(len(graphs)))
        algo = int(rng.integers(2))
        q.append((gi, algo, int(rng.integers(graphs[gi].n))))
    return q


def reference(grus, graphs, q):
    gi, algo, src = q
    return grus.sssp(graphs[gi], src) if algo == grus.ALGO_SSSP else grus.bfs(graphs[gi], src)


@pytest.mark.parametrize("cluster", [1, 2, 8])
def test_batch_matches_single_queries(grus, graphs, cluster):
    torch = pytest.importorskip("torch")
    b = grus.Batch(graphs, cluster_size=cluster)
    queries = make_queries(grus, graphs, 96, cluster)
    offs, total = b.layout(queries)
    out = torch.full((total,), -7, dtype=torch.int32, device="cuda")
    st = b.run(queries, out, offs, stats=True)
    assert st["kernel_launches"] == 1
    res = out.cpu().numpy().view(np.uint32)
    for q, o in zip(queries, offs):
        ref = reference(grus, graphs, q)
        assert np.array_equal(res[o:o + len(ref)], ref), q
    b.free()


def test_batch_cuda_graph_replay(grus, graphs):
    torch = pytest.importorskip("torch")
    b = grus.Batch(graphs)
    for rep in range(3):
        queries = make_queries(grus, graphs, 64, 1000 + rep)
        offs, total = b.layout(queries)
        out = torch.zeros(total, dtype=torch.int32, device="cuda")
        b.run(queries, out, offs, use_graph=True, stats=True)
        res = out.cpu().numpy().view(np.uint32)
        for q, o in zip(queries, offs):
            ref = reference(grus, graphs, q)
            assert np.array_equal(res[o:o + len(ref)], ref), (rep, q)
    b.free()


def test_batch_256_sssp_over_32_graphs(grus):
    """256 SSSP queries over 32 resident graphs of mixed scale and edge
    factor, at small scale."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    gs = [grus.Graph.rmat(int(rng.integers(8, 13)), int(rng.choice([8, 16, 32])), 500 + i,
                          symmetric=True, weighted=True) for i in range(32)]
    b = grus.Batch(gs)
    queries = [(i % 32, grus.ALGO_SSSP, int(rng.integers(gs[i % 32].n))) for i in range(256)]
    offs, total = b.layout(queries)
    out = torch.zeros(total, dtype=torch.int32, device="cuda")
    b.run(queries, out, offs, use_graph=True)
    torch.cuda.synchronize()
    res = out.cpu().numpy().view(np.uint32)
    for q, o in zip(queries, offs):
        ref = grus.sssp(gs[q[0]], q[2])
        assert np.array_equal(res[o:o + len(ref)], ref)
    b.free()


def test_batch_rejects_bad_queries(grus, graphs):
    torch = pytest.importorskip("torch")
    b = grus.Batch(graphs)
    out = torch.zeros(graphs[0].n, dtype=torch.int32, device="cuda")
    with pytest.raises(grus.GrusError):
        b.run([(0, grus.ALGO_BFS, graphs[0].n)], out, [0])
    with pytest.raises(grus.GrusError):
        b.run([(99, grus.ALGO_BFS, 0)], out, [0])
    host = np.zeros(graphs[0].n, np.uint32)
    with pytest.raises(grus.GrusError):
        b.run([(0, grus.ALGO_BFS, 0)], host, [0])
    b.free()


def test_batch_single_worker_high_diameter(grus, oracle_mod):
    """One cluster worker on a long path-like grid: many levels, each ended by
    the hardware cluster barrier; fresh state reports no error."""
    torch = pytest.importorskip("torch")
    g = grus.Graph.grid2d(300, 40)
    for cl in (16, 4):
        b = grus.Batch([g], cluster_size=cl, workers=1)
        out = torch.zeros(g.n, dtype=torch.int32, device="cuda")
        b.run([(0, grus.ALGO_BFS, 41)], out, [0], stats=True)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), grus.bfs(g, 41))
        b.free()


@pytest.mark.parametrize("group", [1, 5, 16, 32])
def test_batch_sssp_groups(grus, graphs, group):
    """SSSP queries on one graph are packed `group` at a time into
    multi-source tasks (1 = no packing); every result equals the single
    query, with plain launches and CUDA-graph replays, and repeated sources."""
    torch = pytest.importorskip("torch")
    b = grus.Batch(graphs, group_sources=group)
    assert b.info()["group_sources"] == group
    rng = np.random.default_rng(group)
    queries = []
    for gi in (0, 2, 3, 6):
        for _ in range(int(rng.integers(1, 40))):
            queries.append((gi, grus.ALGO_SSSP, int(rng.integers(graphs[gi].n))))
    queries.append((2, grus.ALGO_SSSP, queries[-1][2]))  # a repeated source
    queries += make_queries(grus, graphs, 20, 77)  # mixed BFS/SSSP singles
    for use_graph in (False, True, True):
        offs, total = b.layout(queries)
        out = torch.full((total,), -3, dtype=torch.int32, device="cuda")
        b.run(queries, out, offs, use_graph=use_graph, stats=True)
        res = out.cpu().numpy().view(np.uint32)
        for q, o in zip(queries, offs):
            ref = reference(grus, graphs, q)
            assert np.array_equal(res[o:o + len(ref)], ref), (group, use_graph, q)
    b.free()


def test_batch_rejects_bad_group_size(grus, graphs):
    with pytest.raises(grus.GrusError):
        grus.Batch(graphs, group_sources=33)


@pytest.mark.parametrize("big_edges", [1 << 12, 1])
def test_batch_big_graphs_run_whole_gpu(grus, graphs, big_edges):
    """Queries on graphs at or above big_edges run as whole-GPU launches
    before the cluster workers (all of them with big_edges=1); results equal
    the single queries with plain launches and CUDA-graph replays."""
    torch = pytest.importorskip("torch")
    b = grus.Batch(graphs, big_edges=big_edges)
    assert b.info()["big_edges"] == big_edges
    queries = make_queries(grus, graphs, 80, 31 + big_edges)
    queries += [(2, grus.ALGO_SSSP, s) for s in (0, 5, 77, 4000)]  # a pack on one graph
    for use_graph in (False, True, True):
        offs, total = b.layout(queries)
        out = torch.full((total,), -5, dtype=torch.int32, device="cuda")
        st = b.run(queries, out, offs, use_graph=use_graph, stats=True)
        assert st["kernel_launches"] >= 1
        res = out.cpu().numpy().view(np.uint32)
        for q, o in zip(queries, offs):
            ref = reference(grus, graphs, q)
            assert np.array_equal(res[o:o + len(ref)], ref), (big_edges, use_graph, q)
    b.free()


def test_batch_packs_bfs_on_whole_gpu_lane(grus, graphs):
    """With every graph on the whole-GPU lane, 40 BFS queries on one graph run
    as one 64-source-capable pack and a lone BFS query on another graph as a
    single launch (persistent kernel + tail): the reported launches are the
    real ones, and every result equals the single query."""
    torch = pytest.importorskip("torch")
    b = grus.Batch(graphs, big_edges=1)
    rng = np.random.default_rng(17)
    queries = [(0, grus.ALGO_BFS, int(rng.integers(graphs[0].n))) for _ in range(40)]
    queries.append((1, grus.ALGO_BFS, 3))
    offs, total = b.layout(queries)
    out = torch.full((total,), -5, dtype=torch.int32, device="cuda")
    st = b.run(queries, out, offs, stats=True)
    assert st["kernel_launches"] == 1 + 2  # one pack, one single BFS
    res = out.cpu().numpy().view(np.uint32)
    for q, o in zip(queries, offs):
        ref = reference(grus, graphs, q)
        assert np.array_equal(res[o:o + len(ref)], ref), q
    b.free()



def test_batch_sssp_packs_share_one_launch_across_graphs(grus, graphs):
    """With every graph on the whole-GPU lane, the SSSP packs of several
    graphs (32 + 8 queries on one graph, 1, 8, 3 with a repeated source, and
    17 on the grid) run as ONE multi-graph launch for the first packs and the
    second pack of the 40-query graph on its own; a BFS query is a single
    launch (persistent kernel + tail).  Every result equals the single query."""
    torch = pytest.importorskip("torch")
    b = grus.Batch(graphs, big_edges=1)
    rng = np.random.default_rng(23)
    S, B = grus.ALGO_SSSP, grus.ALGO_BFS
    queries = [(0, S, int(rng.integers(graphs[0].n))) for _ in range(40)]
    queries += [(1, S, 5)]
    queries += [(2, S, int(rng.integers(graphs[2].n))) for _ in range(8)]
    queries += [(5, S, 9), (5, S, 9), (5, S, 0)]
    queries += [(6, S, int(rng.integers(graphs[6].n))) for _ in range(17)]
    queries += [(3, B, 4)]
    order = rng.permutation(len(queries))
    queries = [queries[i] for i in order]
    offs, total = b.layout(queries)
    out = torch.full((total,), -3, dtype=torch.int32, device="cuda")
    st = b.run(queries, out, offs, stats=True)
    assert st["kernel_launches"] == 2 + 2
    res = out.cpu().numpy().view(np.uint32)
    for q, o in zip(queries, offs):
        ref = reference(grus, graphs, q)
        assert np.array_equal(res[o:o + len(ref)], ref), q
    # the same batch again reuses the launch workspace
    out2 = torch.full((total,), -4, dtype=torch.int32, device="cuda")
    b.run(queries, out2, offs, stats=True)
    assert torch.equal(out, out2)
    b.free()


def test_batch_multi_graph_launches_split_past_64_graphs(grus):
    """66 small graphs with one SSSP query each on the whole-GPU lane: a launch
    takes at most 64 graphs, so the queries run as two multi-graph launches,
    and every result equals the single query."""
    torch = pytest.importorskip("torch")
    gs = [grus.Graph.rmat(6 + i % 3, 4, 500 + i, symmetric=True, weighted=True) for i in range(66)]
    b = grus.Batch(gs, big_edges=1)
    queries = [(i, grus.ALGO_SSSP, (7 * i) % gs[i].n) for i in range(66)]
    offs, total = b.layout(queries)
    out = torch.full((total,), -1, dtype=torch.int32, device="cuda")
    st = b.run(queries, out, offs, stats=True)
    assert st["kernel_launches"] == 2
    res = out.cpu().numpy().view(np.uint32)
    for (gi, _, src), o in zip(queries, offs):
        ref = grus.sssp(gs[gi], src)
        assert np.array_equal(res[o:o + len(ref)], ref), gi
    b.free()
    for g in gs:
        g.free()


def _serve_all(grus, graphs, queries, **cfg):
    import time
    torch = pytest.importorskip("torch")
    srv = grus.Server(graphs, **cfg)
    outs = [torch.full((graphs[gi].n,), -7, dtype=torch.int32, device="cuda") for gi, _, _ in queries]
    for i, (gi, algo, src) in enumerate(queries):
        srv.submit(gi, algo, src, outs[i], i)
    done = {}
    t0 = time.time()
    while len(done) < len(queries) and time.time() - t0 < 120:
        for tag, st, _ in srv.poll(256, wait_ms=50):
            done[tag] = st
    srv.close()
    assert len(done) == len(queries) and all(v == 0 for v in done.values())
    return [o.cpu().numpy().view(np.uint32) for o in outs]


def test_batch_autotune_keeps_results(grus, graphs):
    """The batch autotuner (grus_batch_autotune) picks the fastest engine
    setting for a query mix; the tuned batch gives the same bits as the
    default one and as single queries."""
    torch = pytest.importorskip("torch")
    queries = make_queries(grus, graphs, 48, 11)
    cfg, ms = grus.batch_autotune(graphs, queries, reps=1)
    assert ms > 0 and set(cfg) >= {"big_edges", "launch_entries", "cluster_size"}
    outs = []
    for kw in ({}, cfg):
        b = grus.Batch(graphs, **kw)
        offs, total = b.layout(queries)
        out = torch.full((total,), -7, dtype=torch.int32, device="cuda")
        b.run(queries, out, offs, use_graph=True)
        outs.append(out.cpu().numpy().view(np.uint32))
        b.free()
    assert np.array_equal(outs[0], outs[1])
    for q, o in zip(queries, offs):
        ref = reference(grus, graphs, q)
        assert np.array_equal(outs[1][o:o + len(ref)], ref), q


def test_server_autotune_keeps_results(grus, graphs):
    """The server autotuner (grus_server_autotune) times saturated bursts of
    the mix under each setting; a server built with the result, and one with
    BFS packs forced from two queued requests, serve the same bits as single
    queries."""
    queries = make_queries(grus, graphs, 64, 12)
    cfg, qps = grus.server_autotune(graphs, queries, reps=1)
    assert qps > 0 and "bfs_pack_min" in cfg
    for kw in (cfg, dict(big_edges=1, bfs_pack_min=2)):
        got = _serve_all(grus, graphs, queries, **kw)
        for q, o in zip(queries, got):
            assert np.array_equal(o, reference(grus, graphs, q)), (kw, q)
