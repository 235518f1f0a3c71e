"""GPU: multi-source SSSP (up to 32 sources in one persistent launch over a
vertex-major distance matrix) against the oracle's Dijkstra per source --
bit-exact, row per source."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
INF = 4294967294


def host_csr(g):
    import oracle
    offs, cols, wts = g.copy_csr()
    return oracle.CSR(offs, cols, wts)


def check(grus, oracle_mod, g, srcs, h=None):
    h = h or host_csr(g)
    d, st = grus.sssp_multi(g, srcs, stats=True)
    assert d.shape == (len(srcs), g.n)
    reached = 0
    for i, s in enumerate(srcs):
        ref = oracle_mod.sssp(h, int(s))
        bad = np.count_nonzero(d[i] != ref)
        assert bad == 0, f"source {s} (row {i}): {bad} mismatching distances"
        reached += int(np.count_nonzero(ref != INF))
    assert st["vertices_reached"] == reached
    return st


@pytest.mark.parametrize("k", [1, 5, 8, 9, 16, 17, 32])
def test_msssp_rmat_symmetric(grus, oracle_mod, k):
    g = grus.Graph.rmat(13, 16, 12, symmetric=True, weighted=True)
    h = host_csr(g)
    deg = np.diff(h.offs.astype(np.int64))
    rng = np.random.default_rng(k)
    srcs = rng.choice(np.flatnonzero(deg > 0), size=k, replace=False).astype(np.uint32)
    st = check(grus, oracle_mod, g, srcs, h)
    assert st["levels"] >= 2


def test_msssp_repeated_and_isolated_sources(grus, oracle_mod):
    g = grus.Graph.rmat(12, 8, 2, symmetric=True, weighted=True)
    deg = np.diff(host_csr(g).offs.astype(np.int64))
    iso = int(np.flatnonzero(deg == 0)[0])
    hub = g.max_degree_vertex
    check(grus, oracle_mod, g, np.array([hub, hub, iso, 5, hub, iso], np.uint32))


@pytest.mark.parametrize("delta", [1, 7, 96, 5000])
def test_msssp_bucket_widths(grus, oracle_mod, delta):
    """Tiny buckets force many threshold advances and far splits; a huge one
    makes the run pure label correcting.  The distances never change."""
    g = grus.Graph.rmat(11, 16, 31, symmetric=True, weighted=True)
    g.set_tuning(sssp_delta=delta)
    srcs = np.arange(0, 20 * 53, 53, dtype=np.uint32) % g.n
    check(grus, oracle_mod, g, srcs)


def test_msssp_directed_and_grid(grus, oracle_mod):
    g = grus.Graph.rmat(12, 16, 6, symmetric=False, weighted=True)
    check(grus, oracle_mod, g, np.arange(32, dtype=np.uint32) * 61 % g.n)
    grid = grus.Graph.grid2d(40, 50, seed=3, weighted=True)
    check(grus, oracle_mod, grid, np.array([0, 1999, 1000, 77], np.uint32))


def test_msssp_matches_single_source_and_host_output(grus):
    torch = pytest.importorskip("torch")
    g = grus.Graph.rmat(14, 16, 21, symmetric=True, weighted=True)
    srcs = np.array([g.max_degree_vertex, 3, 1000, 16000], np.uint32)
    dev = torch.empty((len(srcs), g.n), dtype=torch.int32, device="cuda")
    grus.sssp_multi(g, srcs, out=dev)
    torch.cuda.synchronize()
    host = grus.sssp_multi(g, srcs)
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), host)
    for i, s in enumerate(srcs):
        assert np.array_equal(host[i], grus.sssp(g, int(s)))


def test_msssp_rejects_bad_arguments(grus):
    g = grus.Graph.rmat(10, 8, 1, symmetric=True, weighted=True)
    with pytest.raises(grus.GrusError):
        grus.sssp_multi(g, np.arange(33, dtype=np.uint32))
    with pytest.raises(grus.GrusError):
        grus.sssp_multi(g, np.array([g.n], np.uint32))
    u = grus.Graph.rmat(10, 8, 1, symmetric=True, weighted=False)
    with pytest.raises(grus.GrusError):
        grus.sssp_multi(u, np.array([0], np.uint32))


@pytest.mark.slow
def test_msssp_rmat22_full_size(grus, oracle_mod):
    """RMAT-22 (the SSSP configuration), 32 sources; three rows checked
    against the oracle, every row against its single-source run."""
    g = grus.Graph.rmat(22, 16, 2, symmetric=True, weighted=True)
    h = host_csr(g)
    deg = np.diff(h.offs.astype(np.int64))
    rng = np.random.default_rng(22)
    srcs = rng.choice(np.flatnonzero(deg > 0), size=32, replace=False).astype(np.uint32)
    d = grus.sssp_multi(g, srcs)
    for i in (0, 13, 31):
        assert np.array_equal(d[i], oracle_mod.sssp(h, int(srcs[i])))
    for i, s in enumerate(srcs):
        assert np.array_equal(d[i], grus.sssp(g, int(s)))
