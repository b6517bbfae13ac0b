"""ctypes declarations of include/grudon_gpu.h (the C ABI)."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libgrudon_gpu.so"

GRD_OK = 0
GRD_E_INVALID = -1
GRD_E_OOM = -2
GRD_E_CUDA = -3
GRD_E_TIMEOUT = -4
GRD_E_ROUND_CAP = -5
GRD_E_IO = -6

GRD_PR_DELTA = 0
GRD_PR_PULL = 1
GRD_CC = 2
GRD_SSSP_HOP = 3
GRD_SSSP_W = 4

GRD_DIR_AUTO, GRD_DIR_PUSH, GRD_DIR_PULL = 0, 1, 2
GRD_FMT_AUTO, GRD_FMT_BITVEC, GRD_FMT_LIST = 0, 1, 2
GRD_ROUND_PUSH_BITVEC, GRD_ROUND_PUSH_LIST, GRD_ROUND_PULL_BITVEC, GRD_ROUND_PULL_LIST = 0, 1, 2, 3
GRD_ROUND_NO_OFFLOAD = 5
GRD_OFFLOAD_NDP, GRD_OFFLOAD_ENGINE, GRD_OFFLOAD_NONE = 0, 1, 2
GRD_CREATE_DEVICE_LAYOUT = 1
LAYOUT_ARRAYS = {"slot_gid": 0, "row_off": 1, "col": 2, "wgt": 3, "outdeg": 4, "own_slot": 5, "hubs": 6,
                 "in_off": 7, "in_src": 8, "in_wgt": 9, "in_hubs": 10, "in_meds": 11}
GRD_RUN_STRICT = 1
GRD_RUN_HOST_LOOP = 2
GRD_RUN_ASYNC = 4

ERROR_NAMES = {
    GRD_E_INVALID: "GRD_E_INVALID", GRD_E_OOM: "GRD_E_OOM", GRD_E_CUDA: "GRD_E_CUDA",
    GRD_E_TIMEOUT: "GRD_E_TIMEOUT", GRD_E_ROUND_CAP: "GRD_E_ROUND_CAP", GRD_E_IO: "GRD_E_IO",
}

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
f32p = C.POINTER(C.c_float)


class grd_csr(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_edges", C.c_uint64),
                ("row_offsets", u64p), ("col_indices", u32p), ("weights", u32p)]


class grd_params(C.Structure):
    _fields_ = [("source", C.c_uint32), ("max_rounds", C.c_uint32), ("damping", C.c_double),
                ("tolerance", C.c_double), ("direction", C.c_int), ("frontier_format", C.c_int),
                ("dense_div", C.c_uint32), ("pull_div", C.c_uint32), ("push_blocks_per_sm", C.c_uint32),
                ("policy", C.c_int), ("offload", C.c_int)]


class grd_stats(C.Structure):
    _fields_ = [("rounds", C.c_uint32), ("converged", C.c_uint32), ("edges_scanned", C.c_uint64),
                ("bytes_synced", C.c_uint64), ("reference_bytes_moved", C.c_uint64),
                ("last_residual", C.c_double), ("push_rounds", C.c_uint32), ("pull_rounds", C.c_uint32),
                ("actives_total", C.c_uint64), ("kernel_launches", C.c_uint64), ("stage_ms", C.c_double * 5),
                ("device_loop", C.c_uint32), ("push_actives", C.c_uint64), ("lbs_ms", C.c_double),
                ("lbs_edges", C.c_uint64), ("lbs_actives", C.c_uint64), ("lbs_launches", C.c_uint64),
                ("no_offload_rounds", C.c_uint32), ("pull_ms", C.c_double), ("pull_launches", C.c_uint64)]


GRD_POLICY_FIXED, GRD_POLICY_LEARNED = 0, 1
GRD_POLICY_IN, GRD_POLICY_HID, GRD_POLICY_OUT = 8, 64, 4
GRD_POLICY_NPARAM = (GRD_POLICY_HID * GRD_POLICY_IN + GRD_POLICY_HID + GRD_POLICY_HID * GRD_POLICY_HID +
                     GRD_POLICY_HID + GRD_POLICY_OUT * GRD_POLICY_HID + GRD_POLICY_OUT)


class grd_policy_model(C.Structure):
    _fields_ = [("mean", C.c_float * GRD_POLICY_IN), ("scale", C.c_float * GRD_POLICY_IN),
                ("w1", C.c_uint16 * (GRD_POLICY_HID * GRD_POLICY_IN)), ("b1", C.c_float * GRD_POLICY_HID),
                ("w2", C.c_uint16 * (GRD_POLICY_HID * GRD_POLICY_HID)), ("b2", C.c_float * GRD_POLICY_HID),
                ("w3", C.c_uint16 * (GRD_POLICY_OUT * GRD_POLICY_HID)), ("b3", C.c_float * GRD_POLICY_OUT),
                ("lo", C.c_float * GRD_POLICY_IN), ("hi", C.c_float * GRD_POLICY_IN)]


class grd_policy_train_cfg(C.Structure):
    _fields_ = [("steps", C.c_uint32), ("lr", C.c_float), ("weight_decay", C.c_float), ("seed", C.c_uint64),
                ("device", C.c_int)]


GRD_VERIFY_TOPK = 20


class grd_verify_result(C.Structure):
    _fields_ = [("errors", C.c_uint64), ("edges_checked", C.c_uint64), ("count", C.c_uint64),
                ("max_value", C.c_uint64), ("num_top", C.c_uint32), ("top_ids", C.c_uint32 * GRD_VERIFY_TOPK),
                ("top_values", C.c_float * GRD_VERIFY_TOPK)]


class grd_round_rec(C.Structure):
    _fields_ = [("round", C.c_uint32), ("mode", C.c_int32), ("frontier_in", C.c_uint64), ("actives", C.c_uint64),
                ("edges", C.c_uint64), ("frontier_out", C.c_uint64), ("ms", C.c_double * 5),
                ("frontier_edges_in", C.c_uint64), ("max_degree_in", C.c_uint64), ("unvisited_in", C.c_uint64)]


class grd_host_graph(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("num_edges", C.c_uint64), ("row_offsets", u64p),
                ("col_indices", u32p), ("weights", u32p), ("seed", C.c_uint64)]


# name -> (restype, argtypes); every symbol here is declared in include/grudon_gpu.h
SIGNATURES = {
    "grd_version": (C.c_char_p, []),
    "grd_device_count": (C.c_int, []),
    "grd_ctx_create": (C.c_int, [C.POINTER(grd_csr), u32p, C.c_uint32, C.c_uint32, C.c_int, C.POINTER(C.c_void_p)]),
    "grd_ctx_destroy": (None, [C.c_void_p]),
    "grd_last_error": (C.c_char_p, [C.c_void_p]),
    "grd_create_error": (C.c_char_p, []),
    "grd_upload": (C.c_int, [C.c_void_p, u64p]),
    "grd_ctx_create_ex": (C.c_int, [C.POINTER(grd_csr), u32p, C.c_uint32, C.c_uint32, C.c_int, C.c_uint32,
                                    C.POINTER(C.c_void_p)]),
    "grd_ingest": (C.c_int, [C.c_void_p, C.POINTER(grd_csr), u32p, u64p]),
    "grd_wait": (C.c_int, [C.c_void_p, C.POINTER(grd_stats)]),
    "grd_read_layout": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "grd_set_algo": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(grd_params)]),
    "grd_init": (C.c_int, [C.c_void_p]),
    "grd_init_sources": (C.c_int, [C.c_void_p, u32p, C.c_size_t]),
    "grd_sync_fwd": (C.c_int, [C.c_void_p]),
    "grd_edge_map": (C.c_int, [C.c_void_p]),
    "grd_sync_bwd": (C.c_int, [C.c_void_p]),
    "grd_aggregate": (C.c_int, [C.c_void_p]),
    "grd_update": (C.c_int, [C.c_void_p, u64p]),
    "grd_aggregate_values": (C.c_int, [C.c_void_p, u32p, u32p, C.c_size_t]),
    "grd_aggregate_values_noalloc": (C.c_int, [C.c_void_p, u32p, u32p, C.c_size_t]),
    "grd_set_policy": (C.c_int, [C.c_void_p, C.POINTER(grd_policy_model)]),
    "grd_policy_features": (C.c_int, [u64p, u64p, u64p, u64p, u32p, C.c_uint32, C.c_uint64, C.c_size_t, f32p]),
    "grd_policy_train": (C.c_int, [f32p, f32p, u8p, C.c_size_t, C.POINTER(grd_policy_train_cfg),
                                   C.POINTER(grd_policy_model), f32p]),
    "grd_policy_grad": (C.c_int, [C.POINTER(grd_policy_model), f32p, f32p, u8p, C.c_size_t, C.c_int, f32p, f32p]),
    "grd_policy_predict": (C.c_int, [C.POINTER(grd_policy_model), f32p, C.c_size_t, C.c_uint32, C.c_int, f32p,
                                     C.POINTER(C.c_int32)]),
    "grd_policy_error": (C.c_char_p, []),
    "grd_verify": (C.c_int, [C.c_void_p, C.POINTER(grd_verify_result)]),
    "grd_policy_load": (C.c_int, [C.c_char_p, C.POINTER(grd_policy_model)]),
    "grd_policy_save": (C.c_int, [C.c_char_p, C.POINTER(grd_policy_model)]),
    "grd_run": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(grd_stats)]),
    "grd_get_stats": (C.c_int, [C.c_void_p, C.POINTER(grd_stats)]),
    "grd_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "grd_get_round_log": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "grd_read_props": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "grd_read_props_async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "grd_read_ranks": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "grd_read_ranks_async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "grd_sssp_multi": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "grd_read_updates": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "grd_read_frontier": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "grd_layout_info": (C.c_int, [C.c_void_p, C.c_uint32, u32p, u32p, u64p]),
    "grd_layout_slots": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_size_t]),
    "grd_layout_preview": (C.c_int, [C.POINTER(grd_csr), u32p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_size_t,
                                     u32p, u32p]),
    "grd_device_props": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "grd_device_ranks": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "grd_stream": (C.c_void_p, [C.c_void_p]),
    "grd_synchronize": (C.c_int, [C.c_void_p]),
    "grd_gen_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                               C.c_int, C.c_int, C.c_int, C.POINTER(C.POINTER(grd_host_graph))]),
    "grd_gen_er": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint64, C.c_int, C.c_int, C.c_int,
                             C.POINTER(C.POINTER(grd_host_graph))]),
    "grd_gen_grid": (C.c_int, [C.c_uint32, C.c_uint64, C.c_int, C.c_int, C.POINTER(C.POINTER(grd_host_graph))]),
    "grd_graph_from_csr": (C.c_int, [C.POINTER(grd_csr), C.POINTER(C.POINTER(grd_host_graph))]),
    "grd_graph_free": (None, [C.POINTER(grd_host_graph)]),
    "grd_rmat_seed": (C.c_uint64, [C.c_uint32, C.c_uint32]),
    "grd_write_gr": (C.c_int, [C.POINTER(grd_host_graph), C.c_char_p]),
    "grd_read_gr": (C.c_int, [C.c_char_p, C.POINTER(C.POINTER(grd_host_graph))]),
    "grd_write_mtx": (C.c_int, [C.POINTER(grd_host_graph), C.c_char_p]),
    "grd_read_mtx": (C.c_int, [C.c_char_p, C.POINTER(C.POINTER(grd_host_graph))]),
    "grd_partition_edge_balanced": (C.c_int, [C.POINTER(grd_host_graph), C.c_uint32, u32p]),
    "grd_write_partition_file": (C.c_int, [u32p, C.c_uint32, C.c_char_p]),
    "grd_read_partition_file": (C.c_int, [C.c_char_p, C.c_uint32, C.c_uint32, u32p]),
}

_lib = None


def load() -> C.CDLL:
    """Loads the in-tree CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the CUDA extension is required; there is no CPU fallback)")
    lib = C.CDLL(os.fspath(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
