"""GPU: the golden fixtures (a path, a star, two components, duplicate edges
and self loops, odd weights, an edgeless graph; tests/golden/*.gr) through
the paths the single-query golden tests do not reach: 64-source BFS rows
equal the known answers, multi-source SSSP rows equal the oracle's Dijkstra,
PageRank is within the FP64 oracle's tolerance (max relative 1e-4, L1 1e-6),
and a batch over all fixtures -- their SSSP queries sharing one multi-graph
launch on the whole-GPU lane -- equals the oracle query by query."""
import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
ANSWERS = json.loads((GOLDEN / "known_answers.json").read_text())
NAMES = sorted(ANSWERS)


def load(grus, name):
    # unweighted fixtures get weight 1 per edge, as the reference loader does
    return grus.Graph.load_gr(GOLDEN / f"{name}.gr", need_weights=True)


def host_csr(g):
    import oracle
    offs, cols, wts = g.copy_csr()
    return oracle.CSR(offs, cols, wts)


@pytest.mark.parametrize("name", NAMES)
def test_bfs_multi_golden(grus, name):
    g = load(grus, name)
    srcs = [int(s) for s in ANSWERS[name]["bfs"]]
    rows = grus.bfs_multi(g, np.array(srcs + srcs[:1], np.uint32))  # a repeated source too
    for i, s in enumerate(srcs + srcs[:1]):
        assert np.array_equal(rows[i], np.array(ANSWERS[name]["bfs"][str(s)], np.uint32)), (name, s)
    g.free()


@pytest.mark.parametrize("name", NAMES)
def test_sssp_multi_golden(grus, oracle_mod, name):
    g = load(grus, name)
    h = host_csr(g)
    srcs = np.arange(min(g.n, 32), dtype=np.uint32)
    rows = grus.sssp_multi(g, srcs)
    for i, s in enumerate(srcs):
        assert np.array_equal(rows[i], oracle_mod.sssp(h, int(s))), (name, s)
    for s, exp in ANSWERS[name]["sssp"].items():
        assert np.array_equal(rows[int(s)], np.array(exp, np.uint32)), (name, s)
    g.free()


@pytest.mark.parametrize("name", NAMES)
def test_pagerank_golden(grus, oracle_mod, name):
    g = grus.Graph.load_gr(GOLDEN / f"{name}.gr")
    r = grus.pagerank(g, 0.85, 20)
    ref = oracle_mod.pagerank(host_csr(g), 0.85, 20)
    err = np.abs(r.astype(np.float64) - ref)
    assert (err / ref).max() <= 1e-4, name
    assert err.sum() <= 1e-6, name
    g.free()


def test_batch_over_golden_graphs(grus, oracle_mod):
    """Every vertex of every fixture as an SSSP source and the known BFS
    sources, all graphs on the whole-GPU lane: the SSSP queries run as
    multi-graph launches (up to 32 per graph per launch), the BFS queries as
    single launches; every result equals the oracle."""
    torch = pytest.importorskip("torch")
    gs = [load(grus, n) for n in NAMES]
    hs = [host_csr(g) for g in gs]
    queries = []
    for gi, name in enumerate(NAMES):
        queries += [(gi, grus.ALGO_SSSP, s) for s in range(gs[gi].n)]
        queries += [(gi, grus.ALGO_BFS, int(s)) for s in ANSWERS[name]["bfs"]]
    b = grus.Batch(gs, big_edges=1)
    offs, total = b.layout(queries)
    out = torch.full((total,), -9, dtype=torch.int32, device="cuda")
    b.run(queries, out, offs, stats=True)
    res = out.cpu().numpy().view(np.uint32)
    for (gi, algo, s), o in zip(queries, offs):
        ref = oracle_mod.sssp(hs[gi], s) if algo == grus.ALGO_SSSP else oracle_mod.bfs(hs[gi], s)
        assert np.array_equal(res[o:o + gs[gi].n], ref), (NAMES[gi], algo, s)
    b.free()
    for g in gs:
        g.free()
