"""GPU: exact SSSP against the oracle's Dijkstra, through the C ABI.

Distances over integer weights are the unique fixpoint of the relax of
samples/sssp/sssp.cu:51-60 and must match bit for bit, for every bucket width
(Delta), launch shape and graph family, and on RMAT-22 (edge factor 16,
seed 2, weights in [1,255]).
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
INF = 4294967294
ANSWERS = json.loads((GOLDEN / "known_answers.json").read_text())


def host_csr(g):
    import oracle
    offs, cols, wts = g.copy_csr()
    return oracle.CSR(offs, cols, wts)


def check(grus, oracle_mod, g, srcs):
    h = host_csr(g)
    for s in srcs:
        d, st = grus.sssp(g, int(s), stats=True)
        ref = oracle_mod.sssp(h, int(s))
        assert np.array_equal(d, ref), f"src {s}: {np.count_nonzero(d != ref)} mismatches"
        assert st["vertices_reached"] == int(np.count_nonzero(ref != INF))
        assert st["edges_reached"] == oracle_mod.reached_edges(h, ref)
        assert st["edges_relaxed"] >= st["edges_reached"] - h.degrees()[s] * 0


@pytest.mark.parametrize("name", [k for k, v in ANSWERS.items() if v["sssp"]])
def test_sssp_golden(grus, name):
    g = grus.Graph.load_gr(GOLDEN / f"{name}.gr", need_weights=True)
    for s, exp in ANSWERS[name]["sssp"].items():
        assert grus.sssp(g, int(s)).tolist() == exp


@pytest.mark.parametrize("delta", [1, 7, 96, 1000, 1 << 30])
def test_sssp_bucket_widths(grus, oracle_mod, delta):
    g = grus.Graph.rmat(14, 16, 2, symmetric=True, weighted=True)
    g.set_tuning(sssp_delta=delta)
    check(grus, oracle_mod, g, [g.max_degree_vertex, 3, 9999])


@pytest.mark.parametrize("huge,ctas", [(64, 1), (1 << 20, 0)])
def test_sssp_bins_and_launch_shapes(grus, oracle_mod, huge, ctas):
    g = grus.Graph.rmat(13, 32, 8, symmetric=True, weighted=True)
    g.set_tuning(huge_degree=huge, ctas_per_sm=ctas)
    check(grus, oracle_mod, g, [g.max_degree_vertex, 1])


def test_sssp_directed_and_grid(grus, oracle_mod):
    g = grus.Graph.rmat(13, 16, 4, symmetric=False, weighted=True)
    check(grus, oracle_mod, g, [g.max_degree_vertex, 0])
    g = grus.Graph.grid2d(120, 90, seed=3, weighted=True)
    check(grus, oracle_mod, g, [91, 0])


def test_sssp_unweighted_graph_rejected(grus):
    g = grus.Graph.rmat(8, 4, 1)
    with pytest.raises(grus.GrusError) as e:
        grus.sssp(g, 0)
    assert e.value.status == grus.EINVAL


@pytest.mark.slow
def test_sssp_rmat22_full_size(grus, oracle_mod):
    """RMAT-22 ef16 seed 2 symmetrised, weights in [1,255]."""
    g = grus.Graph.rmat(22, 16, 2, symmetric=True, weighted=True)
    check(grus, oracle_mod, g, [g.max_degree_vertex])
