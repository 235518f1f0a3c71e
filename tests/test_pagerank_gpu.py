"""GPU: pull PageRank (FP32, compensated sums) against the oracle's FP64
power iteration.  Tolerances (stated by the target): maximum per-vertex
relative error <= 1e-4 and L1 error <= 1e-6."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
MAX_REL, MAX_L1 = 1e-4, 1e-6


def host_csr(g):
    import oracle
    offs, cols, wts = g.copy_csr()
    return oracle.CSR(offs, cols, wts)


def check(grus, oracle_mod, g, damping=0.85, iters=20):
    r, st = grus.pagerank(g, damping, iters, stats=True)
    ref = oracle_mod.pagerank(host_csr(g), damping, iters)
    rel = np.abs(r.astype(np.float64) - ref) / ref
    l1 = np.abs(r.astype(np.float64) - ref).sum()
    assert rel.max() <= MAX_REL, rel.max()
    assert l1 <= MAX_L1, l1
    assert st["levels"] == iters
    return rel.max(), l1


@pytest.mark.parametrize("scale,ef,seed,sym", [(12, 16, 3, False), (14, 8, 1, True), (15, 16, 9, False)])
def test_pagerank_rmat(grus, oracle_mod, scale, ef, seed, sym):
    g = grus.Graph.rmat(scale, ef, seed, symmetric=sym)
    check(grus, oracle_mod, g)


def test_pagerank_csc_matches_oracle_transpose(grus, oracle_mod):
    g = grus.Graph.rmat(12, 8, 5, symmetric=False, weighted=True)
    g.build_csc()
    to, tc, tw = g.copy_csc()
    ref = oracle_mod.csr_to_csc(host_csr(g))
    assert np.array_equal(to, ref.offs) and np.array_equal(tc, ref.cols)
    assert np.array_equal(tw, ref.wts)


def test_pagerank_damping_and_iterations(grus, oracle_mod):
    g = grus.Graph.rmat(11, 16, 2, symmetric=False)
    for d, it in [(0.5, 5), (0.99, 30), (0.85, 1)]:
        check(grus, oracle_mod, g, d, it)
    r0 = grus.pagerank(g, 0.85, 0)
    assert np.allclose(r0, 1.0 / g.n)


def test_pagerank_hub_heavy_graph(grus, oracle_mod):
    """In-degrees far above the CTA threshold exercise the compensated sums."""
    n = 5000
    offs = np.arange(n + 1, dtype=np.uint32)  # every vertex -> vertex 0 (hub)
    offs[0] = 0
    offs[1:] = np.arange(1, n + 1)
    cols = np.zeros(n, np.uint32)
    cols[0] = 1  # 0 -> 1
    g = grus.Graph.from_csr(offs, cols)
    check(grus, oracle_mod, g)


@pytest.mark.slow
def test_pagerank_rmat24_full_size(grus, oracle_mod):
    """Directed RMAT-24 ef16 seed 3, d=0.85, 20 iterations."""
    g = grus.Graph.rmat(24, 16, 3, symmetric=False)
    check(grus, oracle_mod, g)
