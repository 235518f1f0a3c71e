"""GPU: the allocation-free BFS entry point, grus_bfs_static.

It serves callers that cannot allocate device memory (a host process that
owns the whole device budget through its own pool, or loops that cannot
afford cudaMalloc's device-wide synchronisation): its scratch is a fixed
device array inside libgrus, and the caller passes device CSR arrays and a
device output.  This file checks, through the C ABI, that two calls in a row
give exactly the depths of the allocating entry point grus_bfs and of the
oracle (bit-exact, the bar of every BFS test here), for a symmetric graph
(direction-optimising) and a directed one (push only), that an asynchronous
call followed by a synchronous one gives exact depths for both, and that
oversized graphs are refused.
It is collected last so that a run stopping at the first failure has run
every other test first; it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_fn(grus):
    fn = grus.lib.grus_bfs_static
    fn.argtypes = [C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int, C.c_uint32,
                   C.c_void_p, C.POINTER(grus.Stats), C.c_void_p]
    fn.restype = C.c_int
    return fn


@pytest.mark.parametrize("symmetric", [True, False])
def test_static_bfs_matches_grus_bfs_twice(grus, oracle_mod, symmetric):
    torch = pytest.importorskip("torch")
    fn = _static_fn(grus)
    g = grus.Graph.rmat(16, 16, 1, symmetric=symmetric)
    offs, cols, _ = g.copy_csr()
    csr = oracle_mod.CSR(offs, cols)
    info = g.info()
    assert info.n <= (1 << 20) and info.m <= (1 << 25)
    out = torch.empty(info.n, dtype=torch.int32, device="cuda")
    for src in (g.max_degree_vertex, 4242):  # two calls in a row on the shared scratch
        ref, ref_st = grus.bfs(g, src, stats=True)
        out.fill_(-1)
        st = grus.Stats()
        rc = fn(info.n, info.m, info.offsets, info.cols, int(symmetric), src, out.data_ptr(),
                C.byref(st), None)
        assert rc == 0, grus.lib.grus_last_error()
        got = out.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, ref)
        assert np.array_equal(got, oracle_mod.bfs(csr, src))
        assert st.vertices_reached == ref_st["vertices_reached"]
        assert st.edges_reached == ref_st["edges_reached"]
    g.free()


def test_static_bfs_async_then_sync(grus, oracle_mod):
    """Without stats the call is asynchronous on the stream; a call with
    stats queued right behind it on the same stream (and the same shared
    scratch) reports success, and both give exact depths."""
    torch = pytest.importorskip("torch")
    fn = _static_fn(grus)
    g = grus.Graph.rmat(14, 8, 3, symmetric=True)
    offs, cols, _ = g.copy_csr()
    csr = oracle_mod.CSR(offs, cols)
    info = g.info()
    out = torch.empty(info.n, dtype=torch.int32, device="cuda")
    out2 = torch.empty(info.n, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    rc = fn(info.n, info.m, info.offsets, info.cols, 1, 7, out.data_ptr(), None, s.cuda_stream)
    assert rc == 0
    st = grus.Stats()
    rc = fn(info.n, info.m, info.offsets, info.cols, 1, 11, out2.data_ptr(), C.byref(st),
            s.cuda_stream)
    assert rc == 0, grus.lib.grus_last_error()
    s.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint32), oracle_mod.bfs(csr, 7))
    assert np.array_equal(out2.cpu().numpy().view(np.uint32), oracle_mod.bfs(csr, 11))
    assert np.array_equal(out.cpu().numpy().view(np.uint32), grus.bfs(g, 7))


def test_static_bfs_rejects_oversized_and_bad_args(grus):
    torch = pytest.importorskip("torch")
    fn = _static_fn(grus)
    g = grus.Graph.rmat(10, 4, 1)
    info = g.info()
    out = torch.empty(info.n, dtype=torch.int32, device="cuda")
    assert fn((1 << 20) + 1, info.m, info.offsets, info.cols, 1, 0, out.data_ptr(), None, None) == grus.EOVERFLOW
    assert fn(info.n, (1 << 25) + 1, info.offsets, info.cols, 1, 0, out.data_ptr(), None, None) == grus.EOVERFLOW
    assert fn(info.n, info.m, info.offsets, info.cols, 1, info.n, out.data_ptr(), None, None) == grus.EINVAL
    host = np.empty(info.n, np.uint32)
    assert fn(info.n, info.m, info.offsets, info.cols, 1, 0, host.ctypes.data, None, None) == grus.EINVAL
