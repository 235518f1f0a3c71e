"""GPU: 64-source BFS (one persistent launch, 64-bit frontier words) against
k independent oracle BFS runs -- bit-exact, row per source."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
INF = 4294967294


def host_csr(g):
    import oracle
    offs, cols, wts = g.copy_csr()
    return oracle.CSR(offs, cols, wts)


def check(grus, oracle_mod, g, srcs):
    h = host_csr(g)
    d, st = grus.bfs_multi(g, srcs, stats=True)
    ref = oracle_mod.bfs_multi(h, srcs)
    assert d.shape == ref.shape
    bad = np.count_nonzero(d != ref)
    assert bad == 0, f"{bad} mismatching (source, vertex) depths"
    assert st["vertices_reached"] == int(np.count_nonzero(ref != INF))
    return st


@pytest.mark.parametrize("k", [1, 7, 33, 64])
def test_msbfs_rmat_symmetric(grus, oracle_mod, k):
    g = grus.Graph.rmat(14, 16, 4, symmetric=True)
    rng = np.random.default_rng(k)
    deg = np.diff(host_csr(g).offs.astype(np.int64))
    cand = np.flatnonzero(deg > 0)
    srcs = rng.choice(cand, size=k, replace=True).astype(np.uint32)
    st = check(grus, oracle_mod, g, srcs)
    assert st["levels"] >= 2


def test_msbfs_repeated_and_isolated_sources(grus, oracle_mod):
    g = grus.Graph.rmat(12, 8, 2, symmetric=True)
    deg = np.diff(host_csr(g).offs.astype(np.int64))
    iso = int(np.flatnonzero(deg == 0)[0])
    hub = g.max_degree_vertex
    check(grus, oracle_mod, g, np.array([hub, hub, iso, 5, hub, iso], np.uint32))


@pytest.mark.parametrize("alpha", [1e9, 1e-3])
def test_msbfs_push_only_and_pull_heavy(grus, oracle_mod, alpha):
    g = grus.Graph.rmat(13, 16, 9, symmetric=True)
    g.set_tuning(multi_alpha=alpha)
    srcs = np.arange(0, 64 * 97, 97, dtype=np.uint32) % g.n
    check(grus, oracle_mod, g, srcs)


def test_msbfs_directed_with_and_without_csc(grus, oracle_mod):
    g = grus.Graph.rmat(12, 16, 6, symmetric=False)
    srcs = np.arange(64, dtype=np.uint32) * 61 % g.n
    check(grus, oracle_mod, g, srcs)
    g.build_csc()
    g.set_tuning(multi_alpha=1e-3)
    check(grus, oracle_mod, g, srcs)


def test_msbfs_grid(grus, oracle_mod):
    g = grus.Graph.grid2d(64, 90)
    srcs = np.array([0, 91, 5759, 1000, 2500], np.uint32)
    check(grus, oracle_mod, g, srcs)


def test_msbfs_depths_beyond_254_levels(grus, oracle_mod):
    """A 200 x 300 grid (diameter 498) with sources in opposite corners and
    inside: many vertices are reached by some sources within 254 levels and
    by others beyond, where depths are stored directly instead of in the
    per-vertex depth bytes."""
    g = grus.Graph.grid2d(200, 300)
    srcs = np.array([0, 200 * 300 - 1, 299, 100 * 300 + 150, 7, 59999, 12345], np.uint32)
    st = check(grus, oracle_mod, g, srcs)
    assert st["levels"] > 300


def test_msbfs_device_output(grus, oracle_mod):
    torch = pytest.importorskip("torch")
    g = grus.Graph.rmat(11, 16, 8, symmetric=True)
    srcs = np.arange(64, dtype=np.uint32)
    out = torch.empty((64, g.n), dtype=torch.int32, device="cuda")
    grus.bfs_multi(g, srcs, out=out)
    torch.cuda.synchronize()
    ref = oracle_mod.bfs_multi(host_csr(g), srcs)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref)


def test_msbfs_rejects_bad_arguments(grus):
    g = grus.Graph.rmat(8, 4, 1)
    with pytest.raises(grus.GrusError):
        grus.bfs_multi(g, np.zeros(65, np.uint32))
    with pytest.raises(grus.GrusError):
        grus.bfs_multi(g, np.array([g.n], np.uint32))


def test_msbfs_source_outside_the_giant_component(grus, oracle_mod):
    """A source in a small component stops expanding after a few levels; the
    pull levels must stop looking for its bit elsewhere (they search only the
    sources present in the frontier) and every row stays exact.  The graph is
    RMAT-14 with a three-vertex path appended as a component of its own."""
    base = host_csr(grus.Graph.rmat(14, 16, 4, symmetric=True))
    n = base.n
    offs = np.concatenate([base.offs, base.offs[-1] + np.array([1, 3, 4], np.uint32)]).astype(np.uint32)
    cols = np.concatenate([base.cols[:base.m], np.array([n + 1, n, n + 2, n + 1], np.uint32)])
    g = grus.Graph.from_csr(offs, cols, symmetric=True)
    deg = np.diff(offs.astype(np.int64))
    giant = np.flatnonzero(oracle_mod.bfs(host_csr(g), g.max_degree_vertex) != INF)
    srcs = np.concatenate([[n, n + 2], giant[::max(1, len(giant) // 40)][:40]]).astype(np.uint32)
    assert deg[n] > 0 and deg[n + 2] > 0
    check(grus, oracle_mod, g, srcs)  # the default switch
    g.set_tuning(multi_alpha=1e9)     # pull from the second level on
    st = check(grus, oracle_mod, g, srcs)
    assert st["bottom_up_levels"] >= 2
