"""CPU: the oracle against the golden fixtures (tests/golden/make_golden.py).

Pins: the .gr reader and CSR->CSC transpose are compared with the reference's
own host code (ref_pin_*.txt, produced by running graph_loader::ReadGraphGR and
csr_tocsc from the Grus sources); BFS/SSSP/CC with hand-computed answers that
the fixture script checked against networkx; the RMAT generator with a
pure-Python restatement of its specification.
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN

INF = 4294967294
ANSWERS = json.loads((GOLDEN / "known_answers.json").read_text())


def _pin(name):
    txt = (GOLDEN / f"ref_pin_{name}.txt").read_text().split("\n")
    gi = txt.index("# gr")
    ci = txt.index("# csc")
    arr = lambda s: np.array(s.split(), dtype=np.uint32)
    n, m = map(int, txt[gi + 1].split())
    gr = dict(n=n, m=m, offs=arr(txt[gi + 2]), cols=arr(txt[gi + 3]), wts=arr(txt[gi + 4]))
    tn, tm = map(int, txt[ci + 1].split())
    csc = dict(offs=arr(txt[ci + 2]), cols=arr(txt[ci + 3]))
    return gr, csc


@pytest.mark.parametrize("name", sorted(ANSWERS))
def test_read_gr_matches_reference_loader(oracle_mod, name):
    g = oracle_mod.read_gr(GOLDEN / f"{name}.gr")
    ref, _ = _pin(name)
    assert g.n == ref["n"] and g.m == ref["m"]
    assert np.array_equal(g.offs, ref["offs"])
    assert np.array_equal(g.cols, ref["cols"][: g.m])
    assert np.array_equal(g.wts, ref["wts"][: g.m])


@pytest.mark.parametrize("name", sorted(ANSWERS))
def test_transpose_matches_reference_csr_tocsc(oracle_mod, name):
    g = oracle_mod.read_gr(GOLDEN / f"{name}.gr")
    t = oracle_mod.csr_to_csc(g)
    _, ref = _pin(name)
    assert np.array_equal(t.offs, ref["offs"])
    assert np.array_equal(t.cols, ref["cols"][: g.m])


@pytest.mark.parametrize("name", sorted(ANSWERS))
def test_known_answers(oracle_mod, name):
    a = ANSWERS[name]
    g = oracle_mod.read_gr(GOLDEN / f"{name}.gr")
    for s, exp in a["bfs"].items():
        assert oracle_mod.bfs(g, int(s)).tolist() == exp
        d, _ = oracle_mod.omp_bfs(g, int(s), threads=2)
        assert d.tolist() == exp
    for s, exp in a["sssp"].items():
        assert oracle_mod.sssp(g, int(s)).tolist() == exp
        d, _ = oracle_mod.omp_sssp(g, int(s), threads=2)
        assert d.tolist() == exp
    if a["cc"] is not None:
        assert oracle_mod.cc(g).tolist() == a["cc"]
        lab, _ = oracle_mod.omp_cc(g, threads=2)
        assert lab.tolist() == a["cc"]


def test_generator_spec_vectors(oracle_mod):
    spec = json.loads((GOLDEN / "rmat_spec.json").read_text())
    for scale, seed, i, u, v in spec["rmat_edges"]:
        assert oracle_mod.rmat_edge(scale, seed, i) == (u, v)
    for scale, seed, x, y in spec["relabel"]:
        assert oracle_mod.relabel(scale, seed, x) == y
    for seed, u, v, w in spec["weights"]:
        assert oracle_mod.edge_weight(seed, u, v) == w


def test_rmat_csr_properties(oracle_mod):
    g = oracle_mod.rmat(12, 16, 1, oracle_mod.GEN_SYMMETRIC | oracle_mod.GEN_RELABEL | oracle_mod.GEN_WEIGHTED)
    assert g.n == 4096 and g.offs[0] == 0 and g.offs[-1] == g.m
    deg = g.degrees()
    rows = np.repeat(np.arange(g.n, dtype=np.uint32), deg)
    assert not np.any(rows == g.cols), "self-loops must be removed"
    key = rows.astype(np.uint64) << np.uint64(32) | g.cols.astype(np.uint64)
    assert np.all(np.diff(key.astype(np.int64)) > 0), "rows sorted, duplicates removed"
    rkey = g.cols.astype(np.uint64) << np.uint64(32) | rows.astype(np.uint64)
    assert np.array_equal(np.sort(rkey), key), "symmetric"
    # one weight per undirected edge
    order = np.argsort(rkey)
    assert np.array_equal(g.wts[order], g.wts)
    assert g.wts.min() >= 1 and g.wts.max() <= 255


def test_grid_csr(oracle_mod):
    g = oracle_mod.grid(5, 7)
    assert g.n == 35 and g.m == 4 * 35 - 2 * 5 - 2 * 7
    d = oracle_mod.bfs(g, 8)  # row 1, col 1
    r, c = np.divmod(np.arange(35), 7)
    assert np.array_equal(d, (np.abs(r - 1) + np.abs(c - 1)).astype(np.uint32))


@pytest.mark.parametrize("seed", [1, 2])
def test_oracles_match_networkx(oracle_mod, seed):
    nx = pytest.importorskip("networkx")
    g = oracle_mod.rmat(9, 8, seed, oracle_mod.GEN_WEIGHTED | oracle_mod.GEN_RELABEL)
    G = nx.DiGraph()
    G.add_nodes_from(range(g.n))
    for u in range(g.n):
        for e in range(g.offs[u], g.offs[u + 1]):
            G.add_edge(u, int(g.cols[e]), weight=int(g.wts[e]))
    src = oracle_mod.max_degree_vertex(g)
    ref = np.full(g.n, INF, np.uint32)
    for k, v in nx.single_source_dijkstra_path_length(G, src).items():
        ref[k] = v
    assert np.array_equal(oracle_mod.sssp(g, src), ref)
    ref = np.full(g.n, INF, np.uint32)
    for k, v in nx.single_source_shortest_path_length(G, src).items():
        ref[k] = v
    assert np.array_equal(oracle_mod.bfs(g, src), ref)
    pr = oracle_mod.pagerank(g, 0.85, 20)
    # networkx redistributes dangling mass; compare on a graph without sinks
    assert pr.sum() <= 1.0 + 1e-12


def test_pagerank_no_dangling_matches_power_iteration(oracle_mod):
    g = oracle_mod.rmat(8, 8, 4, oracle_mod.GEN_SYMMETRIC | oracle_mod.GEN_RELABEL)
    n = g.n
    deg = g.degrees().astype(np.float64)
    A = np.zeros((n, n))
    rows = np.repeat(np.arange(n), g.degrees())
    np.add.at(A, (g.cols, rows), 1.0)
    r = np.full(n, 1.0 / n)
    inv = np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)
    for _ in range(20):
        r = (1 - 0.85) / n + 0.85 * A @ (r * inv)
    assert np.allclose(oracle_mod.pagerank(g, 0.85, 20), r, rtol=1e-12, atol=1e-15)


def test_gr_roundtrip_and_errors(oracle_mod, tmp_path):
    g = oracle_mod.rmat(7, 4, 11, oracle_mod.GEN_WEIGHTED)
    p = tmp_path / "x.gr"
    oracle_mod.write_gr(p, g)
    h = oracle_mod.read_gr(p)
    assert np.array_equal(h.offs, g.offs) and np.array_equal(h.cols, g.cols)
    assert np.array_equal(h.wts, g.wts)
    raw = p.read_bytes()
    (tmp_path / "trunc.gr").write_bytes(raw[: len(raw) - 9])
    assert oracle_mod.read_gr(tmp_path / "trunc.gr") == -5
    bad = bytearray(raw)
    bad[0] = 2
    (tmp_path / "ver.gr").write_bytes(bytes(bad))
    assert oracle_mod.read_gr(tmp_path / "ver.gr") == -22
    assert oracle_mod.read_gr(tmp_path / "missing.gr") == -2
