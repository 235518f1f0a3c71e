"""GPU: connected components (minimum-id labels) against the oracle."""
import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
ANSWERS = json.loads((GOLDEN / "known_answers.json").read_text())


def host_csr(g):
    import oracle
    offs, cols, wts = g.copy_csr()
    return oracle.CSR(offs, cols, wts)


@pytest.mark.parametrize("name", [k for k, v in ANSWERS.items() if v["cc"] is not None])
def test_cc_golden(grus, name):
    g = grus.Graph.load_gr(GOLDEN / f"{name}.gr")
    assert grus.cc(g).tolist() == ANSWERS[name]["cc"]


@pytest.mark.parametrize("scale,ef,seed", [(12, 2, 1), (14, 16, 2), (16, 4, 3), (10, 1, 5)])
def test_cc_rmat_symmetric(grus, oracle_mod, scale, ef, seed):
    g = grus.Graph.rmat(scale, ef, seed, symmetric=True)
    lab, st = grus.cc(g, stats=True)
    ref = oracle_mod.cc(host_csr(g))
    assert np.array_equal(lab, ref), f"{np.count_nonzero(lab != ref)} mismatches"
    assert len(np.unique(ref)) > 1  # several components, including isolated vertices


def test_cc_directed_is_weak_components(grus, oracle_mod):
    g = grus.Graph.rmat(13, 3, 7, symmetric=False)
    assert np.array_equal(grus.cc(g), oracle_mod.cc(host_csr(g)))


def test_cc_grid_and_device_output(grus, oracle_mod):
    torch = pytest.importorskip("torch")
    g = grus.Graph.grid2d(64, 300)
    out = torch.empty(g.n, dtype=torch.int32, device="cuda")
    grus.cc(g, out=out)
    torch.cuda.synchronize()
    assert np.count_nonzero(out.cpu().numpy()) == 0  # one component, label 0


def test_cc_repeatable(grus, oracle_mod):
    g = grus.Graph.rmat(15, 8, 11, symmetric=True)
    a = grus.cc(g)
    b = grus.cc(g)
    assert np.array_equal(a, b)


@pytest.mark.slow
def test_cc_rmat22_full_size(grus, oracle_mod):
    """RMAT-22 ef16 seed 2 symmetrised."""
    g = grus.Graph.rmat(22, 16, 2, symmetric=True, weighted=True)
    assert np.array_equal(grus.cc(g), oracle_mod.cc(host_csr(g)))
