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


# A launch that timed out at a grid barrier leaves its control block with the
# abort flag raised, a stale arrival count and its error word set.  The next
# launch on that block -- queued right behind it, with no host round trip in
# between, as the server's whole-GPU lane queues them -- must still run to
# completion with exact results: every launch clears its block's barrier and
# error word in its own stream first.  The timed-out wait is the bounded
# one-CTA wait of check_wait_limit, run on the workspace's own block.
@pytest.mark.parametrize("which", ["bfs", "sssp", "bfs_multi", "sssp_multi", "pagerank"])
def test_launch_after_a_timed_out_launch_is_clean(grus, oracle_mod, which):
    import torch
    g = grus.Graph.rmat(13, 8, 7, symmetric=which != "pagerank", weighted=True)
    offs, cols, wts = g.copy_csr()
    csr = oracle_mod.CSR(offs, cols, wts)
    deg = np.diff(offs)
    srcs = np.flatnonzero(deg > 0)[[0, 5, 17, 40]].astype(np.uint32)
    s = torch.cuda.Stream()
    if which == "pagerank":
        g.build_csc()
        ref = oracle_mod.pagerank(csr, 0.85, 20)
        grus.pagerank(g)  # creates the workspace
        out = torch.zeros(g.n, dtype=torch.float32, device="cuda")
        grus.check_stale_barrier(g, grus.CHECK_PAGERANK, 150, stream=s)
        grus.pagerank(g, out=out, stream=s)
        s.synchronize()
        # the PageRank tolerances against FP64: max relative 1e-4, L1 1e-6
        for got in (out.cpu().numpy(), grus.pagerank(g, stats=True)[0]):
            err = np.abs(got.astype(np.float64) - ref)
            assert (err / ref).max() <= 1e-4 and err.sum() <= 1e-6
        g.free()
        return
    multi = which.endswith("multi")
    algo = grus.bfs_multi if which == "bfs_multi" else grus.sssp_multi
    single = grus.bfs if which == "bfs" else grus.sssp
    ref_fn = oracle_mod.bfs if which.startswith("bfs") else oracle_mod.sssp
    refs = [ref_fn(csr, int(v)) for v in srcs]
    code = {"bfs": grus.CHECK_BFS, "sssp": grus.CHECK_SSSP, "bfs_multi": grus.CHECK_BFS_MULTI,
            "sssp_multi": grus.CHECK_SSSP_MULTI}[which]
    if multi:
        algo(g, srcs)  # creates the workspace
        out = torch.zeros((len(srcs), g.n), dtype=torch.int32, device="cuda")
        grus.check_stale_barrier(g, code, 150, stream=s)
        algo(g, srcs, out=out, stream=s)
        s.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        for i in range(len(srcs)):
            assert np.array_equal(got[i], refs[i])
        again, st = algo(g, srcs, stats=True)
    else:
        single(g, int(srcs[0]))  # creates the workspace
        out = torch.zeros(g.n, dtype=torch.int32, device="cuda")
        grus.check_stale_barrier(g, code, 150, stream=s)
        single(g, int(srcs[0]), out=out, stream=s)
        s.synchronize()
        assert np.array_equal(out.cpu().numpy().view(np.uint32), refs[0])
        again, st = single(g, int(srcs[1]), stats=True)
        again = again[None]
        refs = refs[1:2]
    # a synchronous call afterwards reports success and exact results
    for i in range(len(again)):
        assert np.array_equal(again[i], refs[i])
    g.free()


def test_stale_barrier_check_rejects_missing_workspace(grus):
    g = grus.Graph.rmat(8, 4, 1, symmetric=True)
    with pytest.raises(grus.GrusError):
        grus.check_stale_barrier(g, grus.CHECK_BFS, 100)
    grus.bfs(g, 0)
    with pytest.raises(grus.GrusError):
        grus.check_stale_barrier(g, 99, 100)
    with pytest.raises(grus.GrusError):
        grus.check_stale_barrier(g, grus.CHECK_BFS, 0)
    g.free()
