"""GPU: the product .gr loader (grus_graph_load_gr, the job of
graph_loader::ReadGraphGR, include/graph_loader.cuh:65-159) and the device
transpose (grus_graph_build_csc, the job of csr_tocsc, include/graph.cuh:273-303)
against the outputs of the reference's own host code on the golden fixtures
(tests/golden/ref_pin_*.txt, made by oracle/ref_pin.cu).  Includes the
odd-m weighted file, whose weight section follows a 4-byte pad."""
import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
NAMES = sorted(json.loads((GOLDEN / "known_answers.json").read_text()))


def _pin(name):
    txt = (GOLDEN / f"ref_pin_{name}.txt").read_text().split("\n")
    gi, ci = txt.index("# gr"), txt.index("# csc")
    arr = lambda s: np.array(s.split(), dtype=np.uint32)
    n, m = map(int, txt[gi + 1].split())
    return (n, m, arr(txt[gi + 2]), arr(txt[gi + 3])[:m], arr(txt[gi + 4])[:m],
            arr(txt[ci + 2]), arr(txt[ci + 3])[:m])


@pytest.mark.parametrize("managed", [False, True])
@pytest.mark.parametrize("name", NAMES)
def test_loaded_csr_matches_reference_loader(grus, name, managed):
    n, m, offs, cols, wts, toffs, tcols = _pin(name)
    g = grus.Graph.load_gr(GOLDEN / f"{name}.gr", need_weights=True, managed=managed)
    assert (g.n, g.m) == (n, m)
    go, gc, gw = g.copy_csr()
    assert np.array_equal(go, offs)
    assert np.array_equal(gc, cols)
    # the reference fills weights with 1 when the file has none (graph_loader.cuh:95-101)
    gw = gw if gw is not None else np.empty(0, np.uint32)  # no weight array when m == 0
    assert np.array_equal(gw[:m], wts)
    g.build_csc()
    to, tc, _ = g.copy_csc()
    assert np.array_equal(to, toffs)
    assert np.array_equal(tc, tcols)
    g.free()
