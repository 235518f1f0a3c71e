"""GPU: a device-side wait that cannot finish ends by its time limit with an
error status, and the context stays usable -- tested without a fault: the
persistent kernels' own grid barrier runs in a one-CTA launch whose arrival
count is preset, so the barrier never completes and only the limit ends it."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_grid_barrier_wait_ends_by_its_limit(grus, oracle_mod):
    t0 = time.perf_counter()
    st = grus.check_wait_limit(200)
    dt = time.perf_counter() - t0
    assert st == grus.ETIMEDOUT
    assert 0.15 < dt < 10.0
    # the context still runs work after the timed-out wait
    g = grus.Graph.rmat(12, 8, 3, symmetric=True)
    offs, cols, _ = g.copy_csr()
    d = grus.bfs(g, g.max_degree_vertex)
    assert np.array_equal(d, oracle_mod.bfs(oracle_mod.CSR(offs, cols), g.max_degree_vertex))


def test_wait_limit_bounds(grus):
    assert grus.check_wait_limit(0) == grus.EINVAL
    assert grus.check_wait_limit(20000) == grus.EINVAL
