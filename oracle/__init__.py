"""CPU oracle for the Grus traversal path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this package, and only as the checker or the timed CPU baseline.  The product
(grus_framework_gb300, libgrus.so, the mgg headers) never uses it.

ctypes binding of oracle/_build/libgrus_oracle.so (built by oracle/build.py);
see grus_oracle.h for what each function restates and where it is pinned.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

INFINIT = 4294967294
GEN_SYMMETRIC, GEN_WEIGHTED, GEN_RELABEL = 1, 2, 4

_lib = None
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_PU32 = C.POINTER(C.c_uint32)


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not path.exists():
            _build.build_oracle()
        L = C.CDLL(str(path))
        L.orc_rmat_csr.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_uint32,
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(_PU32), C.POINTER(_PU32), C.POINTER(_PU32)]
        L.orc_grid_csr.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(_PU32), C.POINTER(_PU32), C.POINTER(_PU32)]
        L.orc_read_gr.argtypes = [C.c_char_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                  C.POINTER(_PU32), C.POINTER(_PU32), C.POINTER(_PU32)]
        L.orc_write_gr.argtypes = [C.c_char_p, C.c_uint64, C.c_uint64, _u32p, _u32p, C.c_void_p]
        L.orc_rmat_edge.argtypes = [C.c_int, C.c_uint64, C.c_uint64, _PU32, _PU32]
        L.orc_relabel.argtypes = [C.c_int, C.c_uint64, C.c_uint32]
        L.orc_relabel.restype = C.c_uint32
        L.orc_edge_weight.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        L.orc_edge_weight.restype = C.c_uint32
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_csr_to_csc.argtypes = [C.c_uint64, _u32p, _u32p, C.c_void_p, _u32p, _u32p, C.c_void_p]
        L.orc_max_degree_vertex.argtypes = [C.c_uint64, _u32p]
        L.orc_max_degree_vertex.restype = C.c_uint32
        L.orc_bfs.argtypes = [C.c_uint64, _u32p, _u32p, C.c_uint32, _u32p]
        L.orc_sssp.argtypes = [C.c_uint64, _u32p, _u32p, _u32p, C.c_uint32, _u32p]
        L.orc_cc.argtypes = [C.c_uint64, _u32p, _u32p, _u32p]
        L.orc_pagerank.argtypes = [C.c_uint64, _u32p, _u32p, C.c_double, C.c_int, _f64p]
        L.orc_delta_pagerank.argtypes = [C.c_uint64, _u32p, _u32p, _f32p, _PU32]
        L.orc_reached_edges.argtypes = [C.c_uint64, _u32p, _u32p]
        L.orc_reached_edges.restype = C.c_uint64
        L.orc_bfs_multi.argtypes = [C.c_uint64, _u32p, _u32p, _u32p, C.c_int, _u32p]
        L.orc_omp_bfs.argtypes = [C.c_uint64, _u32p, _u32p, C.c_uint32, _u32p, C.c_int]
        L.orc_omp_bfs.restype = C.c_double
        L.orc_omp_sssp.argtypes = [C.c_uint64, _u32p, _u32p, _u32p, C.c_uint32, _u32p, C.c_int]
        L.orc_omp_sssp.restype = C.c_double
        L.orc_omp_cc.argtypes = [C.c_uint64, _u32p, _u32p, _u32p, C.c_int]
        L.orc_omp_cc.restype = C.c_double
        L.orc_omp_pagerank.argtypes = [C.c_uint64, _u32p, _u32p, _u32p, C.c_float, C.c_int, _f32p, C.c_int]
        L.orc_omp_pagerank.restype = C.c_double
        L.orc_omp_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed: {rc}")


def _take(ptr, count):
    """Copy a malloc'ed uint32 array into numpy and free it."""
    if not ptr:
        return None
    arr = np.ctypeslib.as_array(ptr, shape=(max(int(count), 1),))[: int(count)].copy()
    lib().orc_free(C.cast(ptr, C.c_void_p))
    return arr


class CSR:
    """Host CSR (uint32 offsets/cols/weights) as plain numpy arrays."""

    def __init__(self, offs, cols, wts=None):
        self.offs = np.ascontiguousarray(offs, dtype=np.uint32)
        self.cols = np.ascontiguousarray(cols, dtype=np.uint32)
        self.wts = None if wts is None else np.ascontiguousarray(wts, dtype=np.uint32)

    @property
    def n(self):
        return len(self.offs) - 1

    @property
    def m(self):
        return len(self.cols)

    def degrees(self):
        return np.diff(self.offs.astype(np.int64)).astype(np.uint32)


def _gen(fn, *args):
    n, m = C.c_uint64(), C.c_uint64()
    o, c, w = _PU32(), _PU32(), _PU32()
    _check(fn(*args, C.byref(n), C.byref(m), C.byref(o), C.byref(c), C.byref(w)), fn.__name__)
    return CSR(_take(o, n.value + 1), _take(c, m.value), _take(w, m.value) if w else None)


def rmat(scale, edge_factor, seed, flags):
    return _gen(lib().orc_rmat_csr, scale, edge_factor, seed, flags)


def grid(rows, cols, seed=0, flags=0):
    return _gen(lib().orc_grid_csr, rows, cols, seed, flags)


def rmat_edge(scale, seed, i):
    u, v = C.c_uint32(), C.c_uint32()
    lib().orc_rmat_edge(scale, seed, i, C.byref(u), C.byref(v))
    return u.value, v.value


def relabel(scale, seed, x):
    return lib().orc_relabel(scale, seed, x)


def edge_weight(seed, u, v):
    return lib().orc_edge_weight(seed, u, v)


def read_gr(path):
    n, m = C.c_uint64(), C.c_uint64()
    o, c, w = _PU32(), _PU32(), _PU32()
    rc = lib().orc_read_gr(str(path).encode(), C.byref(n), C.byref(m), C.byref(o), C.byref(c), C.byref(w))
    if rc != 0:
        return rc
    return CSR(_take(o, n.value + 1), _take(c, m.value), _take(w, m.value))


def write_gr(path, g: CSR, weights=True):
    w = g.wts if (weights and g.wts is not None) else None
    wp = w.ctypes.data_as(C.c_void_p) if w is not None else None
    _check(lib().orc_write_gr(str(path).encode(), g.n, g.m, g.offs, g.cols, wp), "write_gr")


def csr_to_csc(g: CSR):
    n = g.n
    to = np.zeros(n + 1, np.uint32)
    tc = np.zeros(max(g.m, 1), np.uint32)
    tw = np.zeros(max(g.m, 1), np.uint32) if g.wts is not None else None
    lib().orc_csr_to_csc(n, g.offs, g.cols if g.m else np.zeros(1, np.uint32),
                         g.wts.ctypes.data_as(C.c_void_p) if g.wts is not None else None,
                         to, tc, tw.ctypes.data_as(C.c_void_p) if tw is not None else None)
    return CSR(to, tc[: g.m], None if tw is None else tw[: g.m])


def _cols(g):
    return g.cols if g.m else np.zeros(1, np.uint32)


def max_degree_vertex(g: CSR):
    return lib().orc_max_degree_vertex(g.n, g.offs)


def bfs(g: CSR, src):
    d = np.empty(g.n, np.uint32)
    _check(lib().orc_bfs(g.n, g.offs, _cols(g), src, d), "bfs")
    return d


def sssp(g: CSR, src):
    d = np.empty(g.n, np.uint32)
    w = g.wts if g.wts is not None else np.ones(max(g.m, 1), np.uint32)
    _check(lib().orc_sssp(g.n, g.offs, _cols(g), w, src, d), "sssp")
    return d


def cc(g: CSR):
    lab = np.empty(g.n, np.uint32)
    _check(lib().orc_cc(g.n, g.offs, _cols(g), lab), "cc")
    return lab


def pagerank(g: CSR, damping=0.85, iters=20):
    r = np.empty(g.n, np.float64)
    _check(lib().orc_pagerank(g.n, g.offs, _cols(g), damping, iters, r), "pagerank")
    return r


def delta_pagerank(g: CSR):
    r = np.empty(g.n, np.float32)
    it = C.c_uint32()
    _check(lib().orc_delta_pagerank(g.n, g.offs, _cols(g), r, C.byref(it)), "delta_pagerank")
    return r, it.value


def reached_edges(g: CSR, depth):
    return lib().orc_reached_edges(g.n, g.offs, np.ascontiguousarray(depth, np.uint32))


def bfs_multi(g: CSR, srcs):
    srcs = np.ascontiguousarray(srcs, np.uint32)
    out = np.empty(len(srcs) * g.n, np.uint32)
    _check(lib().orc_bfs_multi(g.n, g.offs, _cols(g), srcs, len(srcs), out), "bfs_multi")
    return out.reshape(len(srcs), g.n)


# ---- timed OpenMP baselines ------------------------------------------------
def omp_threads():
    return lib().orc_omp_max_threads()


def omp_bfs(g: CSR, src, threads=0):
    d = np.empty(g.n, np.uint32)
    t = lib().orc_omp_bfs(g.n, g.offs, _cols(g), src, d, threads)
    return d, t


def omp_sssp(g: CSR, src, threads=0):
    d = np.empty(g.n, np.uint32)
    w = g.wts if g.wts is not None else np.ones(max(g.m, 1), np.uint32)
    t = lib().orc_omp_sssp(g.n, g.offs, _cols(g), w, src, d, threads)
    return d, t


def omp_cc(g: CSR, threads=0):
    lab = np.empty(g.n, np.uint32)
    t = lib().orc_omp_cc(g.n, g.offs, _cols(g), lab, threads)
    return lab, t


def omp_pagerank(csc: CSR, outdeg, damping=0.85, iters=20, threads=0):
    r = np.empty(csc.n, np.float32)
    t = lib().orc_omp_pagerank(csc.n, csc.offs, _cols(csc), np.ascontiguousarray(outdeg, np.uint32),
                               damping, iters, r, threads)
    return r, t
