"""GPU: managed-memory mode with a capped device budget (the reference's UM
policy, include/graph.cuh:170-251, with the budget imposed the way
tools/mem_limit.cu does it).  Results must be identical to HBM mode."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_managed_bfs_sssp_match_device_mode(grus, oracle_mod):
    g_dev = grus.Graph.rmat(16, 16, 1, symmetric=True, weighted=True)
    csr_bytes = 4 * (g_dev.n + 1) + 8 * g_dev.m
    g_man = grus.Graph.rmat(16, 16, 1, symmetric=True, weighted=True, managed=True,
                            budget_bytes=csr_bytes // 2)
    try:
        inf = g_man.info()
        assert inf.mem_mode == grus.MEM_MANAGED and inf.budget_bytes == csr_bytes // 2
        src = g_dev.max_degree_vertex
        assert np.array_equal(grus.bfs(g_man, src), grus.bfs(g_dev, src))
        assert np.array_equal(grus.sssp(g_man, src), grus.sssp(g_dev, src))
        assert np.array_equal(grus.cc(g_man), grus.cc(g_dev))
        o, c, w = g_man.copy_csr()
        ref = oracle_mod.bfs(oracle_mod.CSR(o, c), src)
        assert np.array_equal(grus.bfs(g_man, src), ref)
    finally:
        g_man.free()  # releases the budget balloon
        g_dev.free()


def test_managed_load_gr(grus, tmp_path, oracle_mod):
    g = oracle_mod.rmat(12, 8, 3, oracle_mod.GEN_SYMMETRIC | oracle_mod.GEN_WEIGHTED)
    p = tmp_path / "m.gr"
    oracle_mod.write_gr(p, g)
    gm = grus.Graph.load_gr(p, need_weights=True, managed=True, budget_bytes=1 << 16)
    try:
        src = oracle_mod.max_degree_vertex(g)
        assert np.array_equal(grus.sssp(gm, src), oracle_mod.sssp(g, src))
    finally:
        gm.free()


@pytest.mark.slow
def test_managed_rmat26_half_budget_matches_device_mode(grus):
    """The managed configuration at full size: RMAT-26 (2.1 G edges) with the
    device budget at half the CSR bytes gives the depths of the same graph
    held in HBM, with the same reach counts."""
    torch = pytest.importorskip("torch")
    g_dev = grus.Graph.rmat(26, 16, 3, symmetric=True)
    budget = (4 * (g_dev.n + 1) + 4 * g_dev.m) // 2
    src = g_dev.max_degree_vertex
    d_dev = torch.empty(g_dev.n, dtype=torch.int32, device="cuda")
    _, st_dev = grus.bfs(g_dev, src, out=d_dev, stats=True)
    g_dev.free()
    g_man = grus.Graph.rmat(26, 16, 3, symmetric=True, managed=True, budget_bytes=budget)
    assert g_man.max_degree_vertex == src
    d_man = torch.empty(g_man.n, dtype=torch.int32, device="cuda")
    _, st_man = grus.bfs(g_man, src, out=d_man, stats=True)
    assert torch.equal(d_dev, d_man)
    assert st_man["vertices_reached"] == st_dev["vertices_reached"]
    assert st_man["edges_reached"] == st_dev["edges_reached"]
    assert int(d_man[src]) == 0
    g_man.free()

