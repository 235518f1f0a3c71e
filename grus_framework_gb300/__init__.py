"""grus_framework_gb300 -- GB300-native frontier-traversal core (Grus drop-in).

Python host side over the C ABI in include/grus.h (libgrus.so, hand-written
sm_103a CUDA).  There is no CPU fallback: the first call into the package
loads the library and raises ImportError if it has not been built
(``__graft_entry__.build()`` or ``python -m grus_framework_gb300.build``).

The names follow the reference's interface: a graph is loaded from a Galois
``.gr`` file (graph_loader::Load, include/graph_loader.cuh:160-166) or built
from CSR arrays, and the per-application operators (BFS, SSSP, CC, PageRank)
run over it on the device.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libgrus.so"

INFINIT = 4294967294
OK, ENOENT, EIO, ENOMEM, EBUSY, ENODEV, EINVAL, EOVERFLOW, ETIMEDOUT, ECUDA = (
    0, -2, -5, -12, -16, -19, -22, -75, -110, -1000)
MEM_DEVICE, MEM_MANAGED = 0, 1
GRAPH_SYMMETRIC, GRAPH_WEIGHTED = 1, 2
GEN_SYMMETRIC, GEN_WEIGHTED, GEN_RELABEL = 1, 2, 4
ALGO_BFS, ALGO_SSSP = 0, 1


class GrusError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        msg = f"{what}: {_strerror(status)} ({status})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


class Stats(C.Structure):
    _fields_ = [
        ("levels", C.c_uint32),
        ("bottom_up_levels", C.c_uint32),
        ("direction_switches", C.c_uint32),
        ("kernel_launches", C.c_uint32),
        ("vertices_reached", C.c_uint64),
        ("edges_reached", C.c_uint64),
        ("edges_relaxed", C.c_uint64),
        ("device_ms", C.c_float),
        ("reserved0", C.c_uint32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("reserved")}


class GraphInfo(C.Structure):
    _fields_ = [
        ("n", C.c_uint64), ("m", C.c_uint64),
        ("max_degree_vertex", C.c_uint32), ("max_degree", C.c_uint32),
        ("flags", C.c_uint32), ("mem_mode", C.c_int32),
        ("offsets", C.c_void_p), ("cols", C.c_void_p), ("weights", C.c_void_p),
        ("t_offsets", C.c_void_p), ("t_cols", C.c_void_p), ("t_weights", C.c_void_p),
        ("budget_bytes", C.c_uint64),
    ]


class LevelTrace(C.Structure):
    _fields_ = [("end_ns", C.c_uint64), ("edges", C.c_uint64), ("vertices", C.c_uint32),
                ("pull", C.c_uint32)]


class Query(C.Structure):
    _fields_ = [("graph", C.c_uint32), ("algo", C.c_uint32), ("src", C.c_uint32),
                ("reserved", C.c_uint32), ("out_offset", C.c_uint64)]


class BatchConfig(C.Structure):
    _fields_ = [("cluster_size", C.c_uint32), ("workers", C.c_uint32),
                ("huge_degree", C.c_uint32), ("sssp_delta", C.c_uint32),
                ("group_sources", C.c_uint32), ("big_edges", C.c_uint32),
                ("launch_entries", C.c_uint32)]


class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("cluster_size", C.c_uint32),
                ("hbm_reserve_bytes", C.c_uint64), ("sssp_delta", C.c_uint32),
                ("big_edges", C.c_uint32), ("bfs_pack_min", C.c_uint32)]


class Completion(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("status", C.c_int32), ("reserved", C.c_uint32),
                ("latency_us", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("pending", C.c_uint64), ("rejected", C.c_uint64), ("slots", C.c_uint32),
                ("slots_ready", C.c_uint32), ("big_launches", C.c_uint64),
                ("big_queries", C.c_uint64), ("kernel_launches", C.c_uint64)]


class Telemetry(C.Structure):
    _fields_ = [("hbm_total_bytes", C.c_uint64), ("hbm_free_bytes", C.c_uint64),
                ("link_tx_kbps", C.c_uint32), ("link_rx_kbps", C.c_uint32),
                ("sm_clock_mhz", C.c_uint32), ("mem_clock_mhz", C.c_uint32),
                ("power_mw", C.c_uint32), ("temperature_c", C.c_uint32),
                ("valid", C.c_uint32), ("reserved", C.c_uint32),
                ("driver_version", C.c_char * 32)]


class Tuning(C.Structure):
    _fields_ = [
        ("alpha", C.c_float), ("beta", C.c_float), ("ctas_per_sm", C.c_uint32),
        ("huge_degree", C.c_uint32), ("bu_scan", C.c_uint32), ("timeout_ms", C.c_uint32),
        ("sssp_delta", C.c_uint32), ("bu_words", C.c_uint32), ("multi_alpha", C.c_float),
        ("depth_planes", C.c_uint32), ("tail_cluster", C.c_uint32),
    ]


def _load():
    if not LIB_PATH.exists():
        raise ImportError(
            f"libgrus.so not built at {LIB_PATH}; run __graft_entry__.build() "
            "(the package has no CPU fallback)")
    L = C.CDLL(str(LIB_PATH))
    vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
    PG = C.POINTER(vp)
    sig = {
        "grus_version": ([], C.c_char_p),
        "grus_strerror": ([i32], C.c_char_p),
        "grus_last_error": ([], C.c_char_p),
        "grus_device_init": ([i32], i32),
        "grus_convert_edgelist": ([C.c_char_p, C.c_char_p, C.c_uint32], i32),
        "grus_save_result": ([C.c_char_p, vp, C.c_uint64, C.c_uint32], i32),
        "grus_telemetry_sample": ([C.POINTER(Telemetry)], i32),
        "grus_check_wait_limit": ([C.c_uint32], i32),
        "grus_check_stale_barrier": ([vp, u32, u32, vp], i32),
        "grus_graph_from_csr": ([u64, u64, vp, vp, vp, u32, i32, u64, PG], i32),
        "grus_graph_load_gr": ([C.c_char_p, i32, i32, u64, PG], i32),
        "grus_graph_save_gr": ([vp, C.c_char_p], i32),
        "grus_graph_rmat": ([i32, i32, u64, u32, i32, u64, PG], i32),
        "grus_graph_grid2d": ([u32, u32, u64, u32, PG], i32),
        "grus_graph_get_info": ([vp, C.POINTER(GraphInfo)], i32),
        "grus_graph_copy_csr": ([vp, vp, vp, vp], i32),
        "grus_graph_build_csc": ([vp], i32),
        "grus_graph_build_index": ([vp, C.POINTER(C.c_float)], i32),
        "grus_graph_copy_csc": ([vp, vp, vp, vp], i32),
        "grus_graph_set_tuning": ([vp, C.POINTER(Tuning)], i32),
        "grus_graph_get_tuning": ([vp, C.POINTER(Tuning)], i32),
        "grus_graph_free": ([vp], i32),
        "grus_bfs": ([vp, u32, vp, C.POINTER(Stats), vp], i32),
        "grus_sssp": ([vp, u32, vp, C.POINTER(Stats), vp], i32),
        "grus_bfs_trace": ([vp, C.POINTER(LevelTrace), i32], i32),
        "grus_sssp_trace": ([vp, C.POINTER(LevelTrace), i32], i32),
        "grus_bfs_multi": ([vp, vp, i32, vp, C.POINTER(Stats), vp], i32),
        "grus_sssp_multi": ([vp, vp, i32, vp, C.POINTER(Stats), vp], i32),
        "grus_batch_create": ([C.POINTER(vp), i32, C.POINTER(BatchConfig), PG], i32),
        "grus_batch_run": ([vp, C.POINTER(Query), i32, vp, i32, C.POINTER(Stats), vp], i32),
        "grus_batch_get_info": ([vp, C.POINTER(BatchConfig)], i32),
        "grus_batch_free": ([vp], i32),
        "grus_server_create": ([C.POINTER(vp), i32, C.POINTER(ServerConfig), PG], i32),
        "grus_server_submit": ([vp, u32, u32, u32, vp, u64], i32),
        "grus_server_poll": ([vp, C.POINTER(Completion), i32, i32], i32),
        "grus_server_get_stats": ([vp, C.POINTER(ServerStats)], i32),
        "grus_server_destroy": ([vp], i32),
        "grus_autotune": ([vp, u32, u32, i32, C.POINTER(Tuning), C.POINTER(C.c_float)], i32),
        "grus_cc": ([vp, vp, C.POINTER(Stats), vp], i32),
        "grus_batch_autotune": ([C.POINTER(vp), i32, C.POINTER(Query), i32, i32,
                                 C.POINTER(BatchConfig), C.POINTER(C.c_float)], i32),
        "grus_server_autotune": ([C.POINTER(vp), i32, C.POINTER(Query), i32, i32,
                                  C.POINTER(ServerConfig), C.POINTER(C.c_float)], i32),
        "grus_pagerank": ([vp, C.c_float, i32, vp, C.POINTER(Stats), vp], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


class _LazyLib:
    """Loads libgrus.so on first use; raises ImportError if it is missing."""

    _handle = None

    def __getattr__(self, name):
        if _LazyLib._handle is None:
            _LazyLib._handle = _load()
        return getattr(_LazyLib._handle, name)


lib = _LazyLib()


def _strerror(status):
    return lib.grus_strerror(status).decode()


def _check(status, what):
    if status != 0:
        raise GrusError(status, what, lib.grus_last_error().decode())


RESULT_U32, RESULT_F32 = 0, 1
TEL_HBM, TEL_LINK, TEL_CLOCKS, TEL_POWER, TEL_TEMP, TEL_DRIVER = 1, 2, 4, 8, 16, 32
RESULT_MAGIC = b"GRUSRES1"


def convert_edgelist(in_path, out_path, symmetric=False, weighted=False) -> None:
    """Edge list or Matrix Market coordinate file -> Galois .gr (include/grus.h
    grus_convert_edgelist)."""
    flags = (GEN_SYMMETRIC if symmetric else 0) | (GEN_WEIGHTED if weighted else 0)
    _check(lib.grus_convert_edgelist(str(in_path).encode(), str(out_path).encode(), flags),
           "grus_convert_edgelist")


def save_result(path, values) -> None:
    """Binary dump of a uint32/int32 or float32 result (numpy array or CUDA tensor)."""
    dt = getattr(values, "dtype", None)
    is_f32 = str(dt) in ("float32", "torch.float32")
    n = values.numel() if hasattr(values, "numel") else int(values.size)
    if not is_f32 and str(dt) not in ("uint32", "int32", "torch.int32"):
        raise TypeError("results are 4-byte integers or float32")
    if hasattr(values, "ctypes"):
        values = np.ascontiguousarray(values)
    _check(lib.grus_save_result(str(path).encode(), _ptr(values), n,
                                RESULT_F32 if is_f32 else RESULT_U32), "grus_save_result")


def load_result(path) -> np.ndarray:
    """Reads a file written by save_result."""
    raw = Path(path).read_bytes()
    if raw[:8] != RESULT_MAGIC:
        raise ValueError("not a result file")
    typ, size = np.frombuffer(raw, np.uint32, 2, 8)
    n = int(np.frombuffer(raw, np.uint64, 1, 16)[0])
    return np.frombuffer(raw, np.float32 if typ == RESULT_F32 else np.uint32, n, 24).copy()


def telemetry() -> dict:
    """Device memory, host-link throughput, clocks, power and temperature of
    the current device (fields present when the matching TEL_* bit is set)."""
    t = Telemetry()
    _check(lib.grus_telemetry_sample(C.byref(t)), "grus_telemetry_sample")
    d = {k: getattr(t, k) for k, _ in t._fields_ if k != "reserved"}
    d["driver_version"] = t.driver_version.decode(errors="replace")
    return d


def check_wait_limit(timeout_ms: int = 100) -> int:
    """Runs the bounded-wait diagnostic (include/grus.h grus_check_wait_limit);
    returns its status code (ETIMEDOUT when the wait ended by its limit)."""
    return lib.grus_check_wait_limit(timeout_ms)


CHECK_BFS, CHECK_SSSP, CHECK_BFS_MULTI, CHECK_SSSP_MULTI, CHECK_PAGERANK = 0, 1, 2, 3, 4


def check_stale_barrier(g: "Graph", which: int, timeout_ms: int = 100, stream=None) -> None:
    """Queues, without waiting, a one-CTA wait that times out on the control
    block of `g`'s workspace for `which` (CHECK_*), leaving it as a launch that
    timed out at a grid barrier leaves it (include/grus.h
    grus_check_stale_barrier).  The next call on that workspace must still
    run correctly."""
    _check(lib.grus_check_stale_barrier(g._handle(), which, timeout_ms, _stream(stream)),
           "grus_check_stale_barrier")


def version() -> str:
    return lib.grus_version().decode()


def device_init(device: int = 0) -> None:
    _check(lib.grus_device_init(device), "grus_device_init")


def _ptr(buf):
    """Address of a numpy array, torch tensor or raw integer pointer."""
    if buf is None:
        return None
    if isinstance(buf, int):
        return buf
    if isinstance(buf, np.ndarray):
        if not buf.flags["C_CONTIGUOUS"]:
            raise ValueError("buffer must be C-contiguous")
        return buf.ctypes.data
    if hasattr(buf, "data_ptr"):
        if not buf.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return buf.data_ptr()
    raise TypeError(f"unsupported buffer type {type(buf)!r}")


def _stream(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return getattr(stream, "cuda_stream", None)


class Graph:
    """A device-resident CSR graph (uint32 offsets, columns and weights)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    # ---- construction -----------------------------------------------------
    @classmethod
    def rmat(cls, scale, edge_factor=16, seed=1, symmetric=True, weighted=False,
             relabel=True, managed=False, budget_bytes=0):
        flags = ((GEN_SYMMETRIC if symmetric else 0) | (GEN_WEIGHTED if weighted else 0)
                 | (GEN_RELABEL if relabel else 0))
        h = C.c_void_p()
        _check(lib.grus_graph_rmat(scale, edge_factor, seed, flags,
                                   MEM_MANAGED if managed else MEM_DEVICE, budget_bytes,
                                   C.byref(h)), "grus_graph_rmat")
        return cls(h.value)

    @classmethod
    def grid2d(cls, rows, cols, seed=0, weighted=False):
        h = C.c_void_p()
        _check(lib.grus_graph_grid2d(rows, cols, seed, GEN_WEIGHTED if weighted else 0,
                                     C.byref(h)), "grus_graph_grid2d")
        return cls(h.value)

    @classmethod
    def from_csr(cls, offsets, cols, weights=None, symmetric=False, managed=False,
                 budget_bytes=0):
        offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
        cols = np.ascontiguousarray(cols, dtype=np.uint32)
        if cols.size == 0:
            cols = np.zeros(1, np.uint32)[:0]
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.uint32)
        n = offsets.size - 1
        m = int(offsets[-1]) if n >= 0 else 0
        h = C.c_void_p()
        _check(lib.grus_graph_from_csr(n, m, _ptr(offsets), _ptr(cols) if m else None,
                                       _ptr(w) if w is not None else None,
                                       GRAPH_SYMMETRIC if symmetric else 0,
                                       MEM_MANAGED if managed else MEM_DEVICE, budget_bytes,
                                       C.byref(h)), "grus_graph_from_csr")
        return cls(h.value)

    @classmethod
    def load_gr(cls, path, need_weights=False, managed=False, budget_bytes=0):
        h = C.c_void_p()
        _check(lib.grus_graph_load_gr(str(path).encode(), int(bool(need_weights)),
                                      MEM_MANAGED if managed else MEM_DEVICE, budget_bytes,
                                      C.byref(h)), "grus_graph_load_gr")
        return cls(h.value)

    # ---- queries ----------------------------------------------------------
    def _handle(self):
        if not self._h or not self._h.value:
            raise ValueError("graph has been freed")
        return self._h

    def info(self) -> GraphInfo:
        inf = GraphInfo()
        _check(lib.grus_graph_get_info(self._handle(), C.byref(inf)), "grus_graph_get_info")
        return inf

    @property
    def n(self):
        return self.info().n

    @property
    def m(self):
        return self.info().m

    @property
    def max_degree_vertex(self):
        return self.info().max_degree_vertex

    @property
    def weighted(self):
        return bool(self.info().flags & GRAPH_WEIGHTED)

    def copy_csr(self):
        inf = self.info()
        offs = np.empty(inf.n + 1, np.uint32)
        cols = np.empty(max(inf.m, 1), np.uint32)
        wts = np.empty(max(inf.m, 1), np.uint32) if inf.weights else None
        _check(lib.grus_graph_copy_csr(self._handle(), _ptr(offs), _ptr(cols),
                                       _ptr(wts) if wts is not None else None),
               "grus_graph_copy_csr")
        return offs, cols[: inf.m], (wts[: inf.m] if wts is not None else None)

    def copy_offsets(self):
        """The CSR offsets alone (n + 1 entries) on the host."""
        offs = np.empty(self.info().n + 1, np.uint32)
        _check(lib.grus_graph_copy_csr(self._handle(), _ptr(offs), None, None),
               "grus_graph_copy_csr")
        return offs

    def build_csc(self):
        _check(lib.grus_graph_build_csc(self._handle()), "grus_graph_build_csc")

    def build_index(self) -> float:
        """Builds the BFS pull index now (include/grus.h
        grus_graph_build_index); returns its build time in device ms."""
        ms = C.c_float()
        _check(lib.grus_graph_build_index(self._handle(), C.byref(ms)), "grus_graph_build_index")
        return ms.value

    def copy_csc(self):
        inf = self.info()
        offs = np.empty(inf.n + 1, np.uint32)
        cols = np.empty(max(inf.m, 1), np.uint32)
        wts = np.empty(max(inf.m, 1), np.uint32) if inf.t_weights else None
        _check(lib.grus_graph_copy_csc(self._handle(), _ptr(offs), _ptr(cols),
                                       _ptr(wts) if wts is not None else None),
               "grus_graph_copy_csc")
        return offs, cols[: inf.m], (wts[: inf.m] if wts is not None else None)

    def save_gr(self, path):
        _check(lib.grus_graph_save_gr(self._handle(), str(path).encode()), "grus_graph_save_gr")

    def set_tuning(self, **kw):
        """Set fields of this graph's grus_tuning (the others keep their
        values; 0 means the library default).  Unknown names raise TypeError."""
        t = Tuning()
        _check(lib.grus_graph_get_tuning(self._handle(), C.byref(t)), "grus_graph_get_tuning")
        known = {f for f, _ in t._fields_}
        for k, v in kw.items():
            if k not in known:
                raise TypeError(f"unknown tuning field {k!r}")
            setattr(t, k, v)
        _check(lib.grus_graph_set_tuning(self._handle(), C.byref(t)), "grus_graph_set_tuning")

    def get_tuning(self) -> dict:
        t = Tuning()
        _check(lib.grus_graph_get_tuning(self._handle(), C.byref(t)), "grus_graph_get_tuning")
        return {k: getattr(t, k) for k, _ in t._fields_}

    def free(self):
        if self._h and self._h.value:
            lib.grus_graph_free(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _out_array(g: Graph, out, dtype):
    if out is None:
        return np.empty(g.n, dtype)
    return out


def bfs(g: Graph, src: int, out=None, stream=None, stats: bool = False):
    """BFS depths from `src` (uint32, INFINIT for unreached).

    `out` may be a numpy array (host) or a CUDA tensor/pointer (device); with
    a device output and stats=False the call is asynchronous on `stream`.
    """
    out = _out_array(g, out, np.uint32)
    st = Stats() if stats else None
    _check(lib.grus_bfs(g._handle(), src, _ptr(out), C.byref(st) if st is not None else None,
                        _stream(stream)), "grus_bfs")
    return (out, st.as_dict()) if stats else out


def bfs_multi(g: Graph, srcs, out=None, stream=None, stats: bool = False):
    """Depths from up to 64 sources at once: a (k, n) uint32 array."""
    srcs = np.ascontiguousarray(srcs, dtype=np.uint32)
    k = int(srcs.size)
    if out is None:
        out = np.empty((k, g.n), np.uint32)
    st = Stats() if stats else None
    _check(lib.grus_bfs_multi(g._handle(), _ptr(srcs), k, _ptr(out),
                              C.byref(st) if st is not None else None, _stream(stream)),
           "grus_bfs_multi")
    return (out, st.as_dict()) if stats else out


def sssp_multi(g: Graph, srcs, out=None, stream=None, stats: bool = False):
    """Distances from up to 32 sources at once: a (k, n) uint32 array."""
    srcs = np.ascontiguousarray(srcs, dtype=np.uint32)
    k = int(srcs.size)
    if out is None:
        out = np.empty((k, g.n), np.uint32)
    st = Stats() if stats else None
    _check(lib.grus_sssp_multi(g._handle(), _ptr(srcs), k, _ptr(out),
                               C.byref(st) if st is not None else None, _stream(stream)),
           "grus_sssp_multi")
    return (out, st.as_dict()) if stats else out


def bfs_trace(g: Graph, max_levels: int = 128):
    """Per-level records of the last bfs(..., stats=True) call on `g`."""
    buf = (LevelTrace * max_levels)()
    k = lib.grus_bfs_trace(g._handle(), buf, max_levels)
    if k < 0:
        _check(k, "grus_bfs_trace")
    return [dict(end_us=buf[i].end_ns / 1e3, edges=buf[i].edges, vertices=buf[i].vertices,
                 pull=bool(buf[i].pull)) for i in range(k)]


def sssp_trace(g: Graph, max_levels: int = 256):
    """Per-level records of the last sssp(..., stats=True) call on `g`:
    relaxations, frontier entries and threshold advances so far."""
    buf = (LevelTrace * max_levels)()
    k = lib.grus_sssp_trace(g._handle(), buf, max_levels)
    if k < 0:
        _check(k, "grus_sssp_trace")
    return [dict(end_us=buf[i].end_ns / 1e3, relaxations=buf[i].edges,
                 frontier=buf[i].vertices, splits=buf[i].pull) for i in range(k)]


def sssp(g: Graph, src: int, out=None, stream=None, stats: bool = False):
    """Exact shortest-path distances from `src` over the uint32 edge weights."""
    out = _out_array(g, out, np.uint32)
    st = Stats() if stats else None
    _check(lib.grus_sssp(g._handle(), src, _ptr(out), C.byref(st) if st is not None else None,
                         _stream(stream)), "grus_sssp")
    return (out, st.as_dict()) if stats else out


def cc(g: Graph, out=None, stream=None, stats: bool = False):
    """Connected-component labels: the minimum vertex id of each component."""
    out = _out_array(g, out, np.uint32)
    st = Stats() if stats else None
    _check(lib.grus_cc(g._handle(), _ptr(out), C.byref(st) if st is not None else None,
                       _stream(stream)), "grus_cc")
    return (out, st.as_dict()) if stats else out


def pagerank(g: Graph, damping: float = 0.85, iters: int = 20, out=None, stream=None,
             stats: bool = False):
    """Pull PageRank (FP32 ranks, r0 = 1/n, no dangling redistribution)."""
    out = _out_array(g, out, np.float32)
    st = Stats() if stats else None
    _check(lib.grus_pagerank(g._handle(), damping, iters, _ptr(out),
                             C.byref(st) if st is not None else None, _stream(stream)),
           "grus_pagerank")
    return (out, st.as_dict()) if stats else out


def _graph_array(graphs):
    arr = (C.c_void_p * len(graphs))(*[g._handle().value for g in graphs])
    return arr


class Batch:
    """Many BFS / SSSP queries over several resident graphs in one call
    (include/grus.h grus_batch_*).  Queries on graphs of at least
    `big_edges` edges run first as whole-GPU launches -- SSSP packs of up to
    32 sources per graph, several graphs' packs per launch while their
    distance rows total at most `launch_entries` entries -- and the rest on
    cluster workers in one launch.  Zero arguments take the library
    defaults (grus_batch_config)."""

    def __init__(self, graphs, cluster_size=0, workers=0, huge_degree=0, sssp_delta=0,
                 group_sources=0, big_edges=0, launch_entries=0):
        self.graphs = list(graphs)
        cfg = BatchConfig(cluster_size, workers, huge_degree, sssp_delta, group_sources, big_edges,
                          launch_entries)
        h = C.c_void_p()
        _check(lib.grus_batch_create(_graph_array(self.graphs), len(self.graphs), C.byref(cfg),
                                     C.byref(h)), "grus_batch_create")
        self._h = h

    def layout(self, queries):
        """Output offsets of a list of (graph, algo, src) and the total size."""
        offs, at = [], 0
        for gi, _, _ in queries:
            offs.append(at)
            at += self.graphs[gi].n
        return offs, at

    def run(self, queries, out, offsets=None, use_graph=False, stream=None, stats=False):
        """queries: list of (graph_index, algo, src); out: device buffer
        (uint32/int32 tensor or pointer) holding every result back to back."""
        if offsets is None:
            offsets, _ = self.layout(queries)
        arr = (Query * len(queries))()
        for i, ((gi, algo, src), off) in enumerate(zip(queries, offsets)):
            arr[i] = Query(gi, algo, src, 0, off)
        st = Stats() if stats else None
        _check(lib.grus_batch_run(self._h, arr, len(queries), _ptr(out), int(bool(use_graph)),
                                  C.byref(st) if st is not None else None, _stream(stream)),
               "grus_batch_run")
        return st.as_dict() if stats else None

    def info(self):
        cfg = BatchConfig()
        _check(lib.grus_batch_get_info(self._h, C.byref(cfg)), "grus_batch_get_info")
        return {k: getattr(cfg, k) for k, _ in cfg._fields_}

    def free(self):
        if self._h and self._h.value:
            lib.grus_batch_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Server:
    """Query server over resident graphs (include/grus.h grus_server_*)."""

    def __init__(self, graphs, slots=16, cluster_size=8, hbm_reserve_bytes=0, sssp_delta=0,
                 big_edges=0, bfs_pack_min=0):
        self.graphs = list(graphs)
        cfg = ServerConfig(slots, cluster_size, hbm_reserve_bytes, sssp_delta, big_edges,
                           bfs_pack_min)
        h = C.c_void_p()
        _check(lib.grus_server_create(_graph_array(self.graphs), len(self.graphs), C.byref(cfg),
                                      C.byref(h)), "grus_server_create")
        self._h = h

    def submit(self, graph, algo, src, out, tag):
        _check(lib.grus_server_submit(self._h, graph, algo, src, _ptr(out), tag),
               "grus_server_submit")

    def poll(self, max_items=256, wait_ms=0):
        buf = (Completion * max_items)()
        k = lib.grus_server_poll(self._h, buf, max_items, wait_ms)
        if k < 0:
            _check(k, "grus_server_poll")
        return [(buf[i].tag, buf[i].status, buf[i].latency_us) for i in range(k)]

    def stats(self):
        st = ServerStats()
        _check(lib.grus_server_get_stats(self._h, C.byref(st)), "grus_server_get_stats")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if self._h and self._h.value:
            lib.grus_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _query_array(graphs, queries):
    arr = (Query * len(queries))()
    at = 0
    for i, (gi, algo, src) in enumerate(queries):
        arr[i] = Query(gi, algo, src, 0, at)
        at += graphs[gi].n
    return arr


def batch_autotune(graphs, queries, reps=2, start=None):
    """Tunes the batch engine's knobs on this query mix (include/grus.h
    grus_batch_autotune); returns (Batch keyword arguments, best device ms)."""
    cfg = BatchConfig(**(start or {}))
    ms = C.c_float()
    _check(lib.grus_batch_autotune(_graph_array(graphs), len(graphs), _query_array(graphs, queries),
                                   len(queries), reps, C.byref(cfg), C.byref(ms)),
           "grus_batch_autotune")
    return {k: getattr(cfg, k) for k, _ in cfg._fields_}, ms.value


def server_autotune(graphs, queries, reps=1, start=None):
    """Tunes the server's knobs for saturated throughput on this query mix
    (include/grus.h grus_server_autotune); returns (Server keyword arguments,
    best queries/s)."""
    cfg = ServerConfig(**(start or {}))
    qps = C.c_float()
    _check(lib.grus_server_autotune(_graph_array(graphs), len(graphs), _query_array(graphs, queries),
                                    len(queries), reps, C.byref(cfg), C.byref(qps)),
           "grus_server_autotune")
    return {k: getattr(cfg, k) for k, _ in cfg._fields_}, qps.value


def autotune(g: Graph, algo=ALGO_BFS, src=None, reps=2):
    """Tunes the persistent kernel for `g` (stored on the graph); returns
    (tuning dict, best device ms)."""
    if src is None:
        src = g.max_degree_vertex
    t = Tuning()
    ms = C.c_float()
    _check(lib.grus_autotune(g._handle(), algo, src, reps, C.byref(t), C.byref(ms)), "grus_autotune")
    return {k: getattr(t, k) for k, _ in t._fields_}, ms.value
