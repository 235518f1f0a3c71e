"""GPU: the autotuner picks launch/heuristic settings without changing any
result, stores them on the graph, and the persisted cache reapplies them."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_bfs_and_sssp(grus, tmp_path):
    from grus_framework_gb300 import tuning_cache
    g = grus.Graph.rmat(14, 16, 12, symmetric=True, weighted=True)
    src = g.max_degree_vertex
    before_bfs, before_sssp = grus.bfs(g, src), grus.sssp(g, src)
    t, ms = grus.autotune(g, grus.ALGO_BFS, src, reps=1)
    assert ms > 0 and g.get_tuning() == t
    assert np.array_equal(grus.bfs(g, src), before_bfs)
    entry = tuning_cache.load_or_tune(g, grus.ALGO_SSSP, src, path=tmp_path / "t.json", reps=1)
    assert np.array_equal(grus.sssp(g, src), before_sssp)
    # a fresh handle of the same graph picks the cached entry up
    g2 = grus.Graph.rmat(14, 16, 12, symmetric=True, weighted=True)
    again = tuning_cache.load_or_tune(g2, grus.ALGO_SSSP, src, path=tmp_path / "t.json")
    assert again == entry
    assert g2.get_tuning()["sssp_delta"] == entry["tuning"]["sssp_delta"]
