"""GPU: the query server.  Every result must equal the same query run alone
(bit-exact) while many queries overlap on the device; admission refuses work
that does not fit in free HBM."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graphs(grus):
    return [grus.Graph.rmat(s, 16, 700 + s, symmetric=True, weighted=True) for s in (10, 12, 14, 15)]


def drain(srv, want, timeout=120.0):
    done = {}
    t0 = time.time()
    while len(done) < want and time.time() - t0 < timeout:
        for tag, status, lat in srv.poll(256, wait_ms=50):
            done[tag] = (status, lat)
    return done


def test_server_results_same_alone_and_in_mix(grus, graphs):
    torch = pytest.importorskip("torch")
    srv = grus.Server(graphs, slots=12, cluster_size=4)
    rng = np.random.default_rng(5)
    reqs, outs = [], []
    for tag in range(120):
        gi = int(rng.integers(len(graphs)))
        algo = int(rng.integers(2))
        src = int(rng.integers(graphs[gi].n))
        out = torch.empty(graphs[gi].n, dtype=torch.int32, device="cuda")
        reqs.append((gi, algo, src))
        outs.append(out)
        srv.submit(gi, algo, src, out, tag)
    done = drain(srv, len(reqs))
    assert len(done) == len(reqs)
    assert all(st == 0 for st, _ in done.values())
    for (gi, algo, src), out in zip(reqs, outs):
        alone = grus.sssp(graphs[gi], src) if algo == grus.ALGO_SSSP else grus.bfs(graphs[gi], src)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), alone)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["pending"] == 0 and st["slots_ready"] >= 1
    assert st["kernel_launches"] >= len(reqs)  # at least one kernel per query
    srv.close()


def test_server_admission_by_free_hbm(grus, graphs):
    """A reserve larger than the device refuses every query with ENOMEM."""
    torch = pytest.importorskip("torch")
    srv = grus.Server(graphs, slots=4, hbm_reserve_bytes=1 << 50)
    out = torch.empty(graphs[0].n, dtype=torch.int32, device="cuda")
    srv.submit(0, grus.ALGO_BFS, 0, out, 1)
    done = drain(srv, 1, timeout=30)
    assert done[1][0] == grus.ENOMEM
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_server_rejects_bad_submissions(grus, graphs):
    srv = grus.Server(graphs[:1], slots=2)
    host = np.zeros(graphs[0].n, np.uint32)
    with pytest.raises(grus.GrusError):
        srv.submit(0, grus.ALGO_BFS, 0, host, 0)
    srv.close()


def test_server_big_lane_groups_bfs_and_matches_alone(grus, graphs):
    """With big_edges=1 every graph is served by the whole-GPU lane: queued
    SSSP queries on one graph share multi-source launches, BFS queries share
    one when enough are queued for the graph's size and otherwise run alone,
    and each result equals the query run alone."""
    torch = pytest.importorskip("torch")
    srv = grus.Server(graphs, slots=2, big_edges=1)
    rng = np.random.default_rng(7)
    reqs, outs = [], []
    for tag in range(150):
        gi = int(rng.integers(len(graphs)))
        algo = grus.ALGO_SSSP if tag % 5 else grus.ALGO_BFS
        src = int(rng.integers(graphs[gi].n))
        out = torch.empty(graphs[gi].n, dtype=torch.int32, device="cuda")
        reqs.append((gi, algo, src))
        outs.append(out)
        srv.submit(gi, algo, src, out, tag)
    done = drain(srv, len(reqs))
    assert len(done) == len(reqs)
    assert all(st == 0 for st, _ in done.values())
    for (gi, algo, src), out in zip(reqs, outs):
        alone = grus.sssp(graphs[gi], src) if algo == grus.ALGO_SSSP else grus.bfs(graphs[gi], src)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), alone)
    st = srv.stats()
    assert st["big_queries"] == len(reqs) and st["completed"] == len(reqs)
    assert st["big_launches"] < len(reqs)  # queries were packed
    # a BFS alone is two kernels (persistent kernel, narrow tail), a pack one
    n_bfs = sum(1 for _, algo, _ in reqs if algo == grus.ALGO_BFS)
    assert st["big_launches"] <= st["kernel_launches"] <= st["big_launches"] + n_bfs
    srv.close()


def test_server_big_lane_admission_by_free_hbm(grus):
    """A fresh graph whose whole-GPU workspace does not fit under the reserve is refused."""
    torch = pytest.importorskip("torch")
    g = grus.Graph.rmat(11, 8, 71, symmetric=True, weighted=True)
    srv = grus.Server([g], slots=2, big_edges=1, hbm_reserve_bytes=1 << 50)
    out = torch.empty(g.n, dtype=torch.int32, device="cuda")
    srv.submit(0, grus.ALGO_SSSP, 0, out, 3)
    done = drain(srv, 1, timeout=30)
    assert done[3][0] == grus.ENOMEM
    assert srv.stats()["rejected"] == 1
    srv.close()
    g.free()


def test_server_packs_queued_bfs(grus):
    """Many BFS queries queued on one small graph at once are served by
    multi-source launches (fewer launches than queries) with the results of
    single runs; a lone BFS runs as a single launch."""
    torch = pytest.importorskip("torch")
    g = grus.Graph.rmat(12, 8, 4, symmetric=True, weighted=True)
    srv = grus.Server([g], slots=2, big_edges=1)
    rng = np.random.default_rng(11)
    srcs = [int(rng.integers(g.n)) for _ in range(96)]
    outs = [torch.empty(g.n, dtype=torch.int32, device="cuda") for _ in srcs]
    for tag, (src, out) in enumerate(zip(srcs, outs)):
        srv.submit(0, grus.ALGO_BFS, src, out, tag)
    done = drain(srv, len(srcs))
    assert len(done) == len(srcs) and all(st == 0 for st, _ in done.values())
    for src, out in zip(srcs, outs):
        assert np.array_equal(out.cpu().numpy().view(np.uint32), grus.bfs(g, src))
    st = srv.stats()
    assert st["big_queries"] == len(srcs) and st["big_launches"] < len(srcs)
    before = st["big_launches"]
    lone = torch.empty(g.n, dtype=torch.int32, device="cuda")
    srv.submit(0, grus.ALGO_BFS, srcs[0], lone, 1000)
    assert drain(srv, 1)[1000][0] == 0
    st = srv.stats()
    assert st["big_launches"] == before + 1
    assert np.array_equal(lone.cpu().numpy().view(np.uint32), grus.bfs(g, srcs[0]))
    srv.close()

