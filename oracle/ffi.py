"""ctypes wrapper of the oracle library (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg;
never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

ORC_PR_DELTA, ORC_PR_PULL, ORC_CC, ORC_SSSP_HOP, ORC_SSSP_W = 0, 1, 2, 3, 4

u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)


class orc_stats(C.Structure):
    _fields_ = [("rounds", C.c_uint32), ("converged", C.c_uint32), ("edges_scanned", C.c_uint64),
                ("bytes_synced", C.c_uint64), ("reference_bytes_moved", C.c_uint64),
                ("no_offload_rounds", C.c_uint32)]


# offload decision per round: every round NDP_OFFLOAD (the reference), the
# NDPEngine rule, every round NO_OFFLOAD
ORC_OFFLOAD_NDP, ORC_OFFLOAD_ENGINE, ORC_OFFLOAD_NONE = 0, 1, 2


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.OUT
        if not path.exists():
            path = _build.build()
        L = C.CDLL(os.fspath(path))
        L.orc_run.restype = C.c_int
        L.orc_run.argtypes = [C.c_int, C.c_uint32, C.c_uint64, u64p, u32p, u32p, u32p, C.c_uint32, C.c_uint32,
                              C.c_uint32, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.POINTER(orc_stats)]
        L.orc_layout_create.restype = C.c_void_p
        L.orc_layout_create.argtypes = [C.c_uint32, u64p, u32p, u32p, u32p, C.c_uint32]
        L.orc_layout_free.restype = None
        L.orc_layout_free.argtypes = [C.c_void_p]
        L.orc_run_layout.restype = C.c_int
        L.orc_run_layout.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_int,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(orc_stats)]
        L.orc_run_layout_ex.restype = C.c_int
        L.orc_run_layout_ex.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.c_uint32, C.c_double, C.c_double,
                                        C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(orc_stats)]
        L.orc_layout_slots.restype = C.c_uint32
        L.orc_layout_slots.argtypes = [C.c_uint32, u64p, u32p, u32p, C.c_uint32, C.c_uint32, u32p, C.c_uint32, u32p]
        L.orc_bfs.restype = None
        L.orc_bfs.argtypes = [C.c_uint32, u64p, u32p, C.c_uint32, u32p]
        L.orc_dijkstra.restype = None
        L.orc_dijkstra.argtypes = [C.c_uint32, u64p, u32p, u32p, C.c_uint32, u32p]
        L.orc_cc_union_find.restype = None
        L.orc_cc_union_find.argtypes = [C.c_uint32, u64p, u32p, u32p]
        L.orc_pr_jacobi_fp64.restype = C.c_uint32
        L.orc_pr_jacobi_fp64.argtypes = [C.c_uint32, u64p, u32p, C.c_double, C.c_uint32, C.c_double,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_pr_jacobi_fp64_mt.restype = C.c_uint32
        L.orc_pr_jacobi_fp64_mt.argtypes = [C.c_uint32, u64p, u32p, C.c_double, C.c_uint32, C.c_double, C.c_int,
                                            C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_rmat_seed.restype = C.c_uint64
        L.orc_rmat_seed.argtypes = [C.c_uint32, C.c_uint32]
        L.orc_gen_rmat.restype = C.c_void_p
        L.orc_gen_rmat.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_int,
                                   C.c_int, C.c_int]
        L.orc_graph_num_vertices.restype = C.c_uint32
        L.orc_graph_num_vertices.argtypes = [C.c_void_p]
        L.orc_graph_num_edges.restype = C.c_uint64
        L.orc_graph_num_edges.argtypes = [C.c_void_p]
        L.orc_graph_copy.restype = None
        L.orc_graph_copy.argtypes = [C.c_void_p, u64p, u32p, u32p]
        L.orc_graph_free.restype = None
        L.orc_graph_free.argtypes = [C.c_void_p]
        L.orc_prj_create.restype = C.c_void_p
        L.orc_prj_create.argtypes = [C.c_uint32, u64p, u32p, C.c_double, C.c_int]
        L.orc_prj_init.restype = None
        L.orc_prj_init.argtypes = [C.c_void_p]
        L.orc_prj_iterate.restype = C.c_uint32
        L.orc_prj_iterate.argtypes = [C.c_void_p, C.c_uint32, C.c_double, C.POINTER(C.c_double)]
        L.orc_prj_ranks.restype = None
        L.orc_prj_ranks.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        L.orc_prj_free.restype = None
        L.orc_prj_free.argtypes = [C.c_void_p]
        L.orc_partition_edge_balanced.restype = None
        L.orc_partition_edge_balanced.argtypes = [C.c_uint32, u64p, C.c_uint32, u32p]
        _lib = L
    return _lib


def _csr(ro, col, w=None):
    ro = np.ascontiguousarray(ro, dtype=np.uint64)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    if len(col) == 0:
        col = np.zeros(1, dtype=np.uint32)
    w = None if w is None else np.ascontiguousarray(w, dtype=np.uint32)
    return ro, col, w


def _p32(a):
    return None if a is None else a.ctypes.data_as(u32p)


def run(algo: int, ro, col, w=None, mirror=None, num_memory: int = 1, source: int = 0, max_rounds: int = 1000,
        damping: float = 0.85, tol: float = 1e-6, threads: int = 1, offload: int = ORC_OFFLOAD_NDP) -> dict:
    """Restated reference round protocol; returns props/updates/ranks/stats."""
    if offload != ORC_OFFLOAD_NDP:
        out = Layout(ro, col, w, mirror, num_memory).run(algo, source, max_rounds, damping, tol, threads, offload)
        if algo != ORC_PR_DELTA:
            del out["ranks"]
        return out
    ro, col, w = _csr(ro, col, w)
    V = len(ro) - 1
    mir = None if mirror is None else np.ascontiguousarray(mirror, dtype=np.uint32)
    dt = np.float32 if algo == ORC_PR_DELTA else np.uint32
    props = np.zeros(V, dtype=dt)
    upd = np.zeros(V, dtype=dt)
    ranks = np.zeros(V, dtype=np.float32)
    st = orc_stats()
    rc = lib().orc_run(algo, V, int(ro[-1]), ro.ctypes.data_as(u64p), col.ctypes.data_as(u32p), _p32(w), _p32(mir),
                       num_memory, source, max_rounds, damping, tol, threads, props.ctypes.data_as(C.c_void_p),
                       ranks.ctypes.data_as(C.c_void_p), upd.ctypes.data_as(C.c_void_p), C.byref(st))
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    out = {"props": props, "updates": upd, "stats": {f: getattr(st, f) for f, _ in orc_stats._fields_}}
    if algo == ORC_PR_DELTA:
        out["ranks"] = ranks
    return out


class Layout:
    """Prebuilt restated layout, so timing covers run() only."""

    def __init__(self, ro, col, w=None, mirror=None, num_memory: int = 1):
        ro, col, w = _csr(ro, col, w)
        self.V = len(ro) - 1
        self._keep = (ro, col, w)
        mir = None if mirror is None else np.ascontiguousarray(mirror, dtype=np.uint32)
        self._h = lib().orc_layout_create(self.V, ro.ctypes.data_as(u64p), col.ctypes.data_as(u32p), _p32(w),
                                          _p32(mir), num_memory)
        if not self._h:
            raise ValueError("oracle rejected the layout arguments")

    def run(self, algo: int, source: int = 0, max_rounds: int = 1000, damping: float = 0.85, tol: float = 1e-6,
            threads: int = 1, offload: int = ORC_OFFLOAD_NDP) -> dict:
        dt = np.float32 if algo == ORC_PR_DELTA else np.uint32
        props = np.zeros(self.V, dtype=dt)
        upd = np.zeros(self.V, dtype=dt)
        ranks = np.zeros(self.V, dtype=np.float32)
        st = orc_stats()
        rc = lib().orc_run_layout_ex(self._h, algo, source, max_rounds, damping, tol, threads, offload,
                                     props.ctypes.data_as(C.c_void_p), ranks.ctypes.data_as(C.c_void_p),
                                     upd.ctypes.data_as(C.c_void_p), C.byref(st))
        if rc != 0:
            raise ValueError("oracle rejected the run arguments")
        return {"props": props, "updates": upd, "ranks": ranks,
                "stats": {f: getattr(st, f) for f, _ in orc_stats._fields_}}

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_layout_free(self._h)
            self._h = None


def layout_slots(ro, col, mirror, num_memory: int, part: int):
    ro, col, _ = _csr(ro, col)
    V = len(ro) - 1
    mir = None if mirror is None else np.ascontiguousarray(mirror, dtype=np.uint32)
    cap = V * 2 + 1
    out = np.zeros(cap, dtype=np.uint32)
    n_owned = C.c_uint32()
    T = lib().orc_layout_slots(V, ro.ctypes.data_as(u64p), col.ctypes.data_as(u32p), _p32(mir), num_memory, part,
                               out.ctypes.data_as(u32p), cap, C.byref(n_owned))
    return out[:T].copy(), int(n_owned.value)


def bfs(ro, col, src: int) -> np.ndarray:
    ro, col, _ = _csr(ro, col)
    d = np.zeros(len(ro) - 1, dtype=np.uint32)
    lib().orc_bfs(len(ro) - 1, ro.ctypes.data_as(u64p), col.ctypes.data_as(u32p), src, d.ctypes.data_as(u32p))
    return d


def dijkstra(ro, col, w, src: int) -> np.ndarray:
    ro, col, w = _csr(ro, col, w)
    if len(w) == 0:
        w = np.zeros(1, dtype=np.uint32)
    d = np.zeros(len(ro) - 1, dtype=np.uint32)
    lib().orc_dijkstra(len(ro) - 1, ro.ctypes.data_as(u64p), col.ctypes.data_as(u32p), w.ctypes.data_as(u32p), src,
                       d.ctypes.data_as(u32p))
    return d


def cc_union_find(ro, col) -> np.ndarray:
    ro, col, _ = _csr(ro, col)
    lab = np.zeros(len(ro) - 1, dtype=np.uint32)
    lib().orc_cc_union_find(len(ro) - 1, ro.ctypes.data_as(u64p), col.ctypes.data_as(u32p), lab.ctypes.data_as(u32p))
    return lab


def pr_jacobi_fp64(ro, col, damping: float = 0.85, iters: int = 100, tol: float = 0.0):
    ro, col, _ = _csr(ro, col)
    V = len(ro) - 1
    pr = np.zeros(V, dtype=np.float64)
    res = C.c_double()
    it = lib().orc_pr_jacobi_fp64(V, ro.ctypes.data_as(u64p), col.ctypes.data_as(u32p), damping, iters, tol,
                                  pr.ctypes.data_as(C.POINTER(C.c_double)), C.byref(res))
    return pr, int(it), float(res.value)


def pr_jacobi_fp64_mt(ro, col, damping: float = 0.85, iters: int = 100, tol: float = 0.0, threads: int = 0):
    ro, col, _ = _csr(ro, col)
    V = len(ro) - 1
    pr = np.zeros(V, dtype=np.float64)
    res = C.c_double()
    it = lib().orc_pr_jacobi_fp64_mt(V, ro.ctypes.data_as(u64p), col.ctypes.data_as(u32p), damping, iters, tol,
                                     threads or (os.cpu_count() or 1), pr.ctypes.data_as(C.POINTER(C.c_double)),
                                     C.byref(res))
    return pr, int(it), float(res.value)


def rmat_seed(scale: int, edge_factor: int) -> int:
    return int(lib().orc_rmat_seed(scale, edge_factor))


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed=None,
             symmetrize: bool = False, weighted: bool = False, threads: int = 0):
    """The restated seeded RMAT generator: (row_offsets u64, col u32, weights
    u32 or None), identical to the product generator's CSR for the same
    arguments."""
    if seed is None:
        seed = rmat_seed(scale, edge_factor)
    h = lib().orc_gen_rmat(scale, edge_factor, a, b, c, seed, int(symmetrize), int(weighted), threads)
    if not h:
        raise ValueError("oracle generator rejected the arguments")
    try:
        V = lib().orc_graph_num_vertices(h)
        E = lib().orc_graph_num_edges(h)
        ro = np.empty(V + 1, dtype=np.uint64)
        col = np.empty(max(E, 1), dtype=np.uint32)
        w = np.empty(max(E, 1), dtype=np.uint32) if weighted else None
        lib().orc_graph_copy(h, ro.ctypes.data_as(u64p), col.ctypes.data_as(u32p), _p32(w))
    finally:
        lib().orc_graph_free(h)
    return ro, col[:E], (w[:E] if w is not None else None)


def partition_edge_balanced(ro, num_memory: int) -> np.ndarray:
    ro = np.ascontiguousarray(ro, dtype=np.uint64)
    part = np.empty(len(ro) - 1, dtype=np.uint32)
    lib().orc_partition_edge_balanced(len(ro) - 1, ro.ctypes.data_as(u64p), num_memory, part.ctypes.data_as(u32p))
    return part


def csr_checksum(ro, col, w=None) -> str:
    """Order-sensitive 64-bit digest of a CSR (hex), computed with numpy so
    that both benchmark arms can state which graph they ran."""
    m = np.uint64(0x9E3779B97F4A7C15)
    with np.errstate(over="ignore"):
        acc = np.uint64(len(ro) - 1) * m
        for arr in (ro, col, w):
            if arr is None:
                continue
            a = np.ascontiguousarray(arr).astype(np.uint64, copy=False)
            idx = np.arange(1, len(a) + 1, dtype=np.uint64)
            acc = acc * np.uint64(31) + np.sum((a + np.uint64(1)) * (idx * m | np.uint64(1)), dtype=np.uint64)
    return f"{int(acc):016x}"


class PrJacobi:
    """FP32-Kahan Jacobi PageRank (FP64 residual) on the host: the graph is
    transposed once, then iterations run in bounded samples."""

    def __init__(self, ro, col, damping: float = 0.85, threads: int = 0):
        ro, col, _ = _csr(ro, col)
        self.V = len(ro) - 1
        self._keep = (ro, col)
        self._h = lib().orc_prj_create(self.V, ro.ctypes.data_as(u64p), col.ctypes.data_as(u32p), damping,
                                       threads or (os.cpu_count() or 1))

    def init(self) -> None:
        lib().orc_prj_init(self._h)

    def iterate(self, iters: int, tol: float = 0.0):
        """Runs up to `iters` iterations (stopping once the residual / V <
        tol when tol > 0); returns (iterations, last residual / V)."""
        r = C.c_double()
        it = lib().orc_prj_iterate(self._h, iters, tol, C.byref(r))
        return int(it), float(r.value)

    def ranks(self) -> np.ndarray:
        out = np.empty(self.V, dtype=np.float32)
        lib().orc_prj_ranks(self._h, out.ctypes.data_as(C.POINTER(C.c_float)))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_prj_free(self._h)
            self._h = None
