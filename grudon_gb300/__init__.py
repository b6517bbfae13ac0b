"""grudon_gb300: GB300-native per-round graph operator of Grudon.

Python mirror of the C ABI (include/grudon_gpu.h).  The compute path is the
in-tree CUDA library libgrudon_gpu.so; importing works without a GPU (the
host graph tools run on the CPU), but every device call raises GrdError when
no CUDA device is present — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _ffi
from ._ffi import (GRD_CC, GRD_DIR_AUTO, GRD_DIR_PULL, GRD_DIR_PUSH, GRD_FMT_AUTO, GRD_FMT_BITVEC,
                   GRD_FMT_LIST, GRD_PR_DELTA, GRD_PR_PULL, GRD_ROUND_PULL_BITVEC, GRD_ROUND_PULL_LIST,
                   GRD_ROUND_PUSH_BITVEC, GRD_ROUND_PUSH_LIST, GRD_RUN_STRICT, GRD_SSSP_HOP, GRD_SSSP_W,
                   GRD_POLICY_FIXED, GRD_POLICY_LEARNED, GRD_ROUND_NO_OFFLOAD, GRD_OFFLOAD_NDP,
                   GRD_OFFLOAD_ENGINE, GRD_OFFLOAD_NONE)

__all__ = [
    "GrdError", "Graph", "Context", "lib", "device_count", "rmat_seed",
    "GRD_PR_DELTA", "GRD_PR_PULL", "GRD_CC", "GRD_SSSP_HOP", "GRD_SSSP_W",
    "GRD_DIR_AUTO", "GRD_DIR_PUSH", "GRD_DIR_PULL", "GRD_FMT_AUTO", "GRD_FMT_BITVEC", "GRD_FMT_LIST",
    "GRD_ROUND_PUSH_BITVEC", "GRD_ROUND_PUSH_LIST", "GRD_ROUND_PULL_BITVEC", "GRD_ROUND_PULL_LIST",
    "GRD_POLICY_FIXED", "GRD_POLICY_LEARNED", "GRD_RUN_STRICT", "ALGO_NAMES", "GRD_ROUND_NO_OFFLOAD",
    "GRD_OFFLOAD_NDP", "GRD_OFFLOAD_ENGINE", "GRD_OFFLOAD_NONE",
]

ALGO_NAMES = {"pr": GRD_PR_DELTA, "pr_delta": GRD_PR_DELTA, "pr_pull": GRD_PR_PULL, "cc": GRD_CC,
              "sssp": GRD_SSSP_HOP, "sssp_hop": GRD_SSSP_HOP, "sssp_w": GRD_SSSP_W}


class GrdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ffi.ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    return _ffi.load()


def device_count() -> int:
    return int(lib().grd_device_count())


def rmat_seed(scale: int, edge_factor: int) -> int:
    return int(lib().grd_rmat_seed(scale, edge_factor))


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


class Graph:
    """Host CSR owned by the library (generators / readers) or copied in."""

    def __init__(self, handle):
        self._h = handle

    # -- constructors --------------------------------------------------------
    @staticmethod
    def _make(fn, *args) -> "Graph":
        out = C.POINTER(_ffi.grd_host_graph)()
        rc = fn(*args, C.byref(out))
        if rc != 0:
            raise GrdError(rc, f"{fn.__name__} failed")
        return Graph(out)

    @classmethod
    def rmat(cls, scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: Optional[int] = None, symmetrize: bool = False, weighted: bool = False,
             threads: int = 0) -> "Graph":
        if seed is None:
            seed = rmat_seed(scale, edge_factor)
        return cls._make(lib().grd_gen_rmat, scale, edge_factor, a, b, c, seed, int(symmetrize),
                         int(weighted), threads)

    @classmethod
    def er(cls, num_vertices: int, edge_factor: int, seed: int, symmetrize: bool = False,
           weighted: bool = False, threads: int = 0) -> "Graph":
        return cls._make(lib().grd_gen_er, num_vertices, edge_factor, seed, int(symmetrize), int(weighted),
                         threads)

    @classmethod
    def grid(cls, k: int, seed: int = 1, weighted: bool = True, threads: int = 0) -> "Graph":
        return cls._make(lib().grd_gen_grid, k, seed, int(weighted), threads)

    @classmethod
    def from_csr(cls, row_offsets, col_indices, weights=None) -> "Graph":
        ro = np.ascontiguousarray(row_offsets, dtype=np.uint64)
        ci = _u32(col_indices)
        w = None if weights is None else _u32(weights)
        csr = _ffi.grd_csr(len(ro) - 1, len(ci), ro.ctypes.data_as(_ffi.u64p), ci.ctypes.data_as(_ffi.u32p),
                           w.ctypes.data_as(_ffi.u32p) if w is not None else None)
        return cls._make(lib().grd_graph_from_csr, C.byref(csr))

    @classmethod
    def from_edges(cls, num_vertices: int, src, dst, weights=None) -> "Graph":
        """Edges in any order; rows are sorted by destination (stable for weights)."""
        src = np.asarray(src, dtype=np.int64)
        dst = np.asarray(dst, dtype=np.int64)
        order = np.lexsort((dst, src))
        ro = np.zeros(num_vertices + 1, dtype=np.uint64)
        np.add.at(ro, src + 1, 1)
        ro = np.cumsum(ro).astype(np.uint64)
        w = None if weights is None else np.asarray(weights)[order]
        return cls.from_csr(ro, dst[order], w)

    @classmethod
    def read_gr(cls, path: str) -> "Graph":
        return cls._make(lib().grd_read_gr, path.encode())

    @classmethod
    def read_mtx(cls, path: str) -> "Graph":
        return cls._make(lib().grd_read_mtx, path.encode())

    # -- accessors -------------------------------------------------------------
    @property
    def num_vertices(self) -> int:
        return int(self._h.contents.num_vertices)

    @property
    def num_edges(self) -> int:
        return int(self._h.contents.num_edges)

    @property
    def seed(self) -> int:
        return int(self._h.contents.seed)

    @property
    def row_offsets(self) -> np.ndarray:
        return np.ctypeslib.as_array(self._h.contents.row_offsets, shape=(self.num_vertices + 1,))

    @property
    def col_indices(self) -> np.ndarray:
        if self.num_edges == 0:
            return np.zeros(0, dtype=np.uint32)
        return np.ctypeslib.as_array(self._h.contents.col_indices, shape=(self.num_edges,))

    @property
    def weights(self) -> Optional[np.ndarray]:
        if not self._h.contents.weights:
            return None
        if self.num_edges == 0:
            return np.zeros(0, dtype=np.uint32)
        return np.ctypeslib.as_array(self._h.contents.weights, shape=(self.num_edges,))

    def csr_struct(self) -> _ffi.grd_csr:
        h = self._h.contents
        return _ffi.grd_csr(h.num_vertices, h.num_edges, h.row_offsets, h.col_indices, h.weights)

    def out_degrees(self) -> np.ndarray:
        return np.diff(self.row_offsets).astype(np.uint32)

    def write_gr(self, path: str) -> None:
        rc = lib().grd_write_gr(self._h, path.encode())
        if rc != 0:
            raise GrdError(rc, f"cannot write {path}")

    def write_mtx(self, path: str) -> None:
        rc = lib().grd_write_mtx(self._h, path.encode())
        if rc != 0:
            raise GrdError(rc, f"cannot write {path}")

    def partition_edge_balanced(self, num_memory: int) -> np.ndarray:
        part = np.zeros(self.num_vertices, dtype=np.uint32)
        rc = lib().grd_partition_edge_balanced(self._h, num_memory, part.ctypes.data_as(_ffi.u32p))
        if rc != 0:
            raise GrdError(rc, "partitioning failed")
        return part

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                lib().grd_graph_free(h)
            except Exception:
                pass
            self._h = None


def layout_preview(graph: Graph, mirror_part, num_memory: int, part: int):
    """Slot -> gid order of one memory partition, built on the host (no GPU)."""
    mp = None if mirror_part is None else _u32(mirror_part)
    cap = 2 * graph.num_vertices + 1
    out = np.zeros(cap, dtype=np.uint32)
    no, npx = C.c_uint32(), C.c_uint32()
    csr = graph.csr_struct()
    rc = lib().grd_layout_preview(C.byref(csr), None if mp is None else mp.ctypes.data_as(_ffi.u32p), num_memory,
                                  part, out.ctypes.data_as(C.c_void_p), cap, C.byref(no), C.byref(npx))
    if rc != 0:
        raise GrdError(rc, lib().grd_create_error().decode())
    return out[: no.value + npx.value].copy(), int(no.value)


def write_partition_file(part, path: str) -> None:
    p = _u32(part)
    rc = lib().grd_write_partition_file(p.ctypes.data_as(_ffi.u32p), len(p), path.encode())
    if rc != 0:
        raise GrdError(rc, f"cannot write {path}")


def read_partition_file(path: str, n: int, num_memory: int) -> np.ndarray:
    p = np.zeros(n, dtype=np.uint32)
    rc = lib().grd_read_partition_file(path.encode(), n, num_memory, p.ctypes.data_as(_ffi.u32p))
    if rc != 0:
        raise GrdError(rc, f"cannot read partition file {path}")
    return p


class Context:
    """One partitioned graph resident on one GPU (grd_ctx)."""

    def __init__(self, graph: Graph, mirror_part=None, num_memory: int = 1, device: int = 0,
                 device_layout: bool = False):
        """device_layout=True builds the partition layout on the GPU from the
        uploaded CSR (grd_ctx_create_ex with GRD_CREATE_DEVICE_LAYOUT)."""
        self._lib = lib()
        self._ctx = C.c_void_p()
        self._graph = graph  # keeps host arrays alive for the create call
        self.num_vertices = graph.num_vertices
        mp = None
        if mirror_part is not None:
            self._mp = _u32(mirror_part)
            if len(self._mp) != graph.num_vertices:
                raise ValueError("mirror_part must have one entry per vertex")
            mp = self._mp.ctypes.data_as(_ffi.u32p)
        csr = graph.csr_struct()
        flags = _ffi.GRD_CREATE_DEVICE_LAYOUT if device_layout else 0
        rc = self._lib.grd_ctx_create_ex(C.byref(csr), mp, 1, num_memory, device, flags, C.byref(self._ctx))
        if rc != 0:
            raise GrdError(rc, self._lib.grd_create_error().decode())
        self.algo = None
        self.device_layout = device_layout

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise GrdError(rc, self._lib.grd_last_error(self._ctx).decode())

    def set_algo(self, algo, source: int = 0, max_rounds: int = 1000, damping: float = 0.85,
                 tolerance: Optional[float] = None, direction: int = GRD_DIR_AUTO,
                 frontier_format: int = GRD_FMT_AUTO, dense_div: int = 0, pull_div: int = 0,
                 push_blocks_per_sm: int = 0, policy: int = _ffi.GRD_POLICY_FIXED,
                 offload: int = GRD_OFFLOAD_NDP) -> None:
        """policy=GRD_POLICY_LEARNED picks each round's mode with the model
        given to set_policy (the fixed rule while none is set).  offload:
        GRD_OFFLOAD_NDP (every round in the memory partitions, the
        reference's choice), GRD_OFFLOAD_ENGINE (the NDPEngine rule per
        round) or GRD_OFFLOAD_NONE (every round pushed by the compute
        partition over the shipped adjacency)."""
        if isinstance(algo, str):
            algo = ALGO_NAMES[algo]
        if tolerance is None:
            tolerance = 1e-7 if algo == GRD_PR_PULL else 1e-6
        p = _ffi.grd_params(source, max_rounds, damping, tolerance, direction, frontier_format, dense_div, pull_div,
                            push_blocks_per_sm, policy, offload)
        self._check(self._lib.grd_set_algo(self._ctx, algo, C.byref(p)))
        self.algo = algo

    def verify(self) -> dict:
        """The reference's verify() checks on the device for the algorithm
        last run (grd_verify): CC/SSSP edge invariants, PageRank top ranks."""
        r = _ffi.grd_verify_result()
        self._check(self._lib.grd_verify(self._ctx, C.byref(r)))
        n = r.num_top
        return {"errors": r.errors, "edges_checked": r.edges_checked, "count": r.count, "max_value": r.max_value,
                "top_ids": list(r.top_ids[:n]), "top_values": list(r.top_values[:n])}

    def set_policy(self, model) -> None:
        """Uploads a learned round-policy model (a grd_policy_model, or None
        to clear it)."""
        self._check(self._lib.grd_set_policy(self._ctx, C.byref(model) if model is not None else None))

    def init(self) -> None:
        self._check(self._lib.grd_init(self._ctx))

    def init_sources(self, sources) -> None:
        """SSSP init with several sources at distance 0."""
        s = _u32(sources)
        self._check(self._lib.grd_init_sources(self._ctx, s.ctypes.data_as(_ffi.u32p), len(s)))

    def sync_fwd(self) -> None:
        self._check(self._lib.grd_sync_fwd(self._ctx))

    def edge_map(self) -> None:
        self._check(self._lib.grd_edge_map(self._ctx))

    def sync_bwd(self) -> None:
        self._check(self._lib.grd_sync_bwd(self._ctx))

    def aggregate(self) -> None:
        self._check(self._lib.grd_aggregate(self._ctx))

    def update(self) -> int:
        f = C.c_uint64()
        self._check(self._lib.grd_update(self._ctx, C.byref(f)))
        return int(f.value)

    def round(self) -> int:
        """One round through the per-stage API; returns |frontier|."""
        self.sync_fwd()
        self.edge_map()
        self.sync_bwd()
        self.aggregate()
        return self.update()

    @staticmethod
    def _stats_dict(s) -> dict:
        out = {}
        for f, _ in _ffi.grd_stats._fields_:
            v = getattr(s, f)
            out[f] = list(v) if isinstance(v, C.Array) else v
        return out

    def run(self, strict: bool = False, host_loop: bool = False, wait: bool = True) -> dict:
        """Runs to convergence (or the round cap).  By default the rounds run
        as one device-driven CUDA-graph launch; host_loop=True drives them
        from the host instead.  wait=False queues the launch and returns at
        once (GRD_RUN_ASYNC): call wait() for the finished statistics, so
        that the runs of several contexts overlap on the GPU."""
        s = _ffi.grd_stats()
        flags = ((GRD_RUN_STRICT if strict else 0) | (_ffi.GRD_RUN_HOST_LOOP if host_loop else 0) |
                 (0 if wait else _ffi.GRD_RUN_ASYNC))
        self._check(self._lib.grd_run(self._ctx, flags, C.byref(s)))
        return self._stats_dict(s)

    def wait(self) -> dict:
        """Completes a run started with wait=False; returns its statistics."""
        s = _ffi.grd_stats()
        self._check(self._lib.grd_wait(self._ctx, C.byref(s)))
        return self._stats_dict(s)

    def stats(self) -> dict:
        s = _ffi.grd_stats()
        self._check(self._lib.grd_get_stats(self._ctx, C.byref(s)))
        return self._stats_dict(s)

    def set_profiling(self, enable: bool = True) -> None:
        self._check(self._lib.grd_set_profiling(self._ctx, int(enable)))

    def round_log(self) -> list:
        """Per-round records of profiled host-loop runs since grd_init."""
        n = C.c_size_t()
        self._check(self._lib.grd_get_round_log(self._ctx, None, 0, C.byref(n)))
        recs = (_ffi.grd_round_rec * max(1, n.value))()
        self._check(self._lib.grd_get_round_log(self._ctx, recs, n.value, C.byref(n)))
        out = []
        for r in recs[: n.value]:
            d = {f: getattr(r, f) for f, _ in _ffi.grd_round_rec._fields_}
            d["ms"] = list(d["ms"])
            out.append(d)
        return out

    def upload(self) -> int:
        b = C.c_uint64()
        self._check(self._lib.grd_upload(self._ctx, C.byref(b)))
        return int(b.value)

    def ingest(self, graph: Graph, mirror_part=None) -> int:
        """Re-uploads a CSR of the same shape into a device-layout ctx and
        rebuilds the layout on the GPU; returns the host->device bytes."""
        mp = None
        if mirror_part is not None:
            keep = _u32(mirror_part)
            mp = keep.ctypes.data_as(_ffi.u32p)
        csr = graph.csr_struct()
        b = C.c_uint64()
        self._check(self._lib.grd_ingest(self._ctx, C.byref(csr), mp, C.byref(b)))
        return int(b.value)

    def read_layout(self, name: str) -> np.ndarray:
        """One resident layout array (grd_read_layout): slot_gid, row_off,
        col, wgt, outdeg, own_slot, hubs, in_off, in_src, in_wgt, in_hubs,
        in_meds; hub lists come back as (n, 3) arrays of (slot, e0, e1)."""
        which = _ffi.LAYOUT_ARRAYS[name]
        n = C.c_size_t()
        self._check(self._lib.grd_read_layout(self._ctx, which, None, 0, C.byref(n)))
        out = np.empty(n.value // 4, dtype=np.uint32)
        self._check(self._lib.grd_read_layout(self._ctx, which, out.ctypes.data_as(C.c_void_p), out.nbytes,
                                              C.byref(n)))
        return out.reshape(-1, 3) if name in ("hubs", "in_hubs", "in_meds") else out

    def _read(self, fn, dtype, n, out=None):
        """out: a caller's array to fill (for example a view of pinned host
        memory, which the copy reaches at the link's full speed); a new array
        otherwise."""
        if out is None:
            out = np.empty(n, dtype=dtype)
        elif out.dtype != dtype or out.size < n or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"out must be a contiguous {np.dtype(dtype).name} array of at least {n} elements")
        self._check(fn(self._ctx, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def read_props(self, out=None, wait: bool = True) -> np.ndarray:
        """wait=False queues the copy into `out` on the ctx stream and returns
        at once (grd_read_props_async): `out` holds the values after
        synchronize(), or wait() for a run(wait=False) queued before it;
        give pinned memory for a truly queued copy."""
        dt = np.float32 if self.algo in (GRD_PR_DELTA, GRD_PR_PULL) else np.uint32
        if wait:
            return self._read(self._lib.grd_read_props, dt, self.num_vertices, out)
        if out is None:
            raise ValueError("read_props(wait=False) needs the caller's out array")
        return self._read(self._lib.grd_read_props_async, dt, self.num_vertices, out)

    def sssp_multi(self, sources) -> tuple:
        """Distances from up to 64 sources at once (grd_sssp_multi): returns
        (dist[n, V] uint32, stats).  The ctx's algorithm must be SSSP (hop or
        weighted) and init() must have run."""
        src = _u32(sources)
        out = np.empty((len(src), self.num_vertices), dtype=np.uint32)
        s = _ffi.grd_stats()
        self._check(self._lib.grd_sssp_multi(self._ctx, src.ctypes.data_as(C.c_void_p), len(src),
                                             out.ctypes.data_as(C.c_void_p), C.byref(s)))
        return out, self._stats_dict(s)

    def read_ranks(self, out=None, wait: bool = True) -> np.ndarray:
        """PageRank values; wait=False queues the copy like read_props."""
        if out is None:
            if not wait:
                raise ValueError("read_ranks(wait=False) needs the caller's out array")
            out = np.empty(self.num_vertices, dtype=np.float32)
        elif out.dtype != np.float32 or out.size < self.num_vertices or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"out must be a contiguous float32 array of at least {self.num_vertices} elements")
        fn = self._lib.grd_read_ranks if wait else self._lib.grd_read_ranks_async
        self._check(fn(self._ctx, out.ctypes.data_as(C.c_void_p), out.size))
        return out

    def read_updates(self, out=None) -> np.ndarray:
        dt = np.float32 if self.algo in (GRD_PR_DELTA, GRD_PR_PULL) else np.uint32
        return self._read(self._lib.grd_read_updates, dt, self.num_vertices, out)

    def read_frontier(self) -> np.ndarray:
        words = (self.num_vertices + 31) // 32
        out = np.empty(words, dtype=np.uint32)
        self._check(self._lib.grd_read_frontier(self._ctx, out.ctypes.data_as(C.c_void_p), words))
        bits = np.unpackbits(out.view(np.uint8), bitorder="little")[: self.num_vertices]
        return bits.astype(bool)

    def layout_info(self, part: int) -> tuple:
        no, npx, ne = C.c_uint32(), C.c_uint32(), C.c_uint64()
        self._check(self._lib.grd_layout_info(self._ctx, part, C.byref(no), C.byref(npx), C.byref(ne)))
        return int(no.value), int(npx.value), int(ne.value)

    def layout_slots(self, part: int) -> np.ndarray:
        no, npx, _ = self.layout_info(part)
        out = np.empty(no + npx, dtype=np.uint32)
        self._check(self._lib.grd_layout_slots(self._ctx, part, out.ctypes.data_as(C.c_void_p), out.size))
        return out

    def device_props_ptr(self) -> int:
        p = C.c_void_p()
        self._check(self._lib.grd_device_props(self._ctx, C.byref(p)))
        return int(p.value or 0)

    def stream(self) -> int:
        return int(self._lib.grd_stream(self._ctx) or 0)

    def synchronize(self) -> None:
        self._check(self._lib.grd_synchronize(self._ctx))

    def close(self) -> None:
        if getattr(self, "_ctx", None) and self._ctx.value:
            self._lib.grd_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
