"""ctypes binding of libgas (include/gas.h).

The library is built in-tree by :mod:`graphreduce_gb300.build`.  Loading it
never falls back to anything: if it is missing or fails to load, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

from .build import LIB

_lock = threading.Lock()
_lib = None

c_i32 = C.c_int32
c_i64 = C.c_int64
c_u64 = C.c_uint64
c_size = C.c_size_t
c_dbl = C.c_double
c_vp = C.c_void_p
P_i32 = C.POINTER(C.c_int32)


class GasError(RuntimeError):
    """A libgas call returned a status other than GAS_OK."""

    def __init__(self, status: int, where: str, detail: str):
        self.status = status
        super().__init__(f"{where}: status {status} ({STATUS_NAMES.get(status, '?')}): {detail}")


STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error",
                4: "iteration cap reached", 5: "I/O error", 6: "call out of order",
                7: "unsupported", 8: "device-side error", 9: "too large"}

GAS_PROG_USER, GAS_PROG_BFS, GAS_PROG_SSSP, GAS_PROG_CC, GAS_PROG_PAGERANK = range(5)
(GAS_SCHED_AUTO, GAS_SCHED_GENERIC, GAS_SCHED_PUSH, GAS_SCHED_PULL,
 GAS_SCHED_ORDERED, GAS_SCHED_LEARNED) = range(6)
GAS_SCHED_FEATURES = 16
GAS_WARM_FEATURES = 4
GAS_TRACE_CAP = 4096
P_f32 = C.POINTER(C.c_float)


class RunStats(C.Structure):
    _fields_ = [("iterations", c_i32), ("push_iters", c_i32), ("pull_iters", c_i32),
                ("kernel_launches", c_i32), ("edges_processed", c_i64),
                ("residual", c_dbl), ("graph_launches", c_i32), ("pad", c_i32)]


class KernelProfile(C.Structure):
    _fields_ = [("push_ms", c_dbl), ("pull_ms", c_dbl), ("pagerank_ms", c_dbl),
                ("push_bytes", c_i64), ("pull_bytes", c_i64), ("pagerank_bytes", c_i64),
                ("push_launches", c_i32), ("pull_launches", c_i32),
                ("pagerank_launches", c_i32), ("pad", c_i32)]


class TraceRecord(C.Structure):
    _fields_ = [("iteration", c_i32), ("mode", c_i32), ("n_queue", c_i32),
                ("n_edges_out", c_i32), ("hist", c_i32 * 8), ("t_start_ns", c_i64),
                ("t_end_ns", c_i64)]


class Counters(C.Structure):
    _fields_ = [("n_active", c_i32), ("n_edges", c_i32), ("n_scatter_edges", c_i32),
                ("error", c_i32), ("iteration", c_i32), ("cond", c_i32),
                ("n_changed", c_i32), ("max_iter", c_i32), ("mode", c_i32),
                ("n_push", c_i32), ("n_pull", c_i32), ("pull_div", c_i32),
                ("sched", c_i32), ("push_chunk_log2", c_i32), ("q_heavy", c_i32),
                ("q_heavy_edges", c_i32), ("seen_edges", c_i32), ("prev_changed", c_i32),
                ("pad", c_i32 * 2)]


GAS_BATCH_MAX_LANES = 32


class BatchJob(C.Structure):
    _fields_ = [("bfs_lanes", c_i32), ("bfs_sources", c_vp), ("ppr_lanes", c_i32),
                ("ppr_seeds", c_vp), ("damping", c_dbl), ("tol", c_dbl),
                ("max_bfs_levels", c_i32), ("max_ppr_iterations", c_i32),
                ("piece_edges", c_i32), ("sssp_lanes", c_i32), ("sssp_sources", c_vp),
                ("max_sssp_iterations", c_i32)]


class BatchStats(C.Structure):
    _fields_ = [("bfs_iterations", c_i32), ("ppr_iterations", c_i32), ("bfs_edges", c_i64),
                ("ppr_residual", c_dbl), ("piece_edges", c_i32), ("kernel_launches", c_i32),
                ("graph_launches", c_i32), ("sssp_iterations", c_i32),
                ("ppr_lane_residual", c_dbl * GAS_BATCH_MAX_LANES), ("sssp_edges", c_i64),
                ("sssp_lane_iterations", c_i32 * GAS_BATCH_MAX_LANES)]


# name -> (restype, argtypes); restype "status" means gas_status_t checked.
_SIGS = {
    "gas_status_string": (C.c_char_p, [c_i32]),
    "gas_last_error": (C.c_char_p, []),
    "gas_version": (C.c_char_p, []),
    "gas_edge_list_create": ("status", [c_i32, c_i64, c_vp, c_vp, c_vp, C.POINTER(c_vp)]),
    "gas_edge_list_destroy": (None, [c_vp]),
    "gas_edge_list_num_vertices": (c_i32, [c_vp]),
    "gas_edge_list_num_edges": (c_i64, [c_vp]),
    "gas_edge_list_srcs": (c_vp, [c_vp]),
    "gas_edge_list_dsts": (c_vp, [c_vp]),
    "gas_edge_list_weights": (c_vp, [c_vp]),
    "gas_rmat": ("status", [c_i32, c_i32, c_dbl, c_dbl, c_dbl, c_u64, c_i32, C.POINTER(c_vp)]),
    "gas_erdos_renyi": ("status", [c_i32, c_i64, c_u64, c_i32, C.POINTER(c_vp)]),
    "gas_edge_list_append_grid_islands": ("status", [c_vp, c_i32, c_i32]),
    "gas_edge_list_set_uniform_weights": ("status", [c_vp, c_i32, c_i32, c_u64]),
    "gas_edge_list_max_out_degree_vertex": ("status", [c_vp, P_i32, P_i32]),
    "gas_edge_list_sample_sources": ("status", [c_vp, c_i32, c_u64, c_vp]),
    "gas_gr_write": ("status", [C.c_char_p, c_vp]),
    "gas_gr_read": ("status", [C.c_char_p, C.POINTER(c_vp)]),
    "gas_mtx_read": ("status", [C.c_char_p, C.POINTER(c_vp)]),
    "gas_snap_read": ("status", [C.c_char_p, C.POINTER(c_vp)]),
    "gas_mtx_write": ("status", [C.c_char_p, c_vp]),
    "gas_graph_read": ("status", [C.c_char_p, C.POINTER(c_vp)]),
    "gas_edge_list_to_csr": ("status", [c_i32, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "gas_engine_create": ("status", [c_i32, C.POINTER(c_vp)]),
    "gas_engine_create_user": ("status", [c_size, c_size, c_size, C.POINTER(c_vp)]),
    "gas_engine_destroy": (None, [c_vp]),
    "gas_engine_set_graph": ("status", [c_vp, c_i32, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp]),
    "gas_engine_set_active": ("status", [c_vp, c_i32, c_i32, c_vp]),
    "gas_engine_count_active": ("status", [c_vp, P_i32]),
    "gas_engine_gather": ("status", [c_vp, c_i32, c_vp]),
    "gas_engine_apply": ("status", [c_vp, c_vp]),
    "gas_engine_scatter_activate": ("status", [c_vp, c_i32, c_vp]),
    "gas_engine_next_iter": ("status", [c_vp, P_i32, c_vp]),
    "gas_engine_get_results": ("status", [c_vp, c_vp]),
    "gas_engine_run": ("status", [c_vp, P_i32, c_vp]),
    "gas_engine_set_iteration": ("status", [c_vp, c_i32]),
    "gas_engine_vertex_data_device": ("status", [c_vp, C.POINTER(c_vp)]),
    "gas_engine_upload_vertex_data": ("status", [c_vp, c_vp, c_vp]),
    "gas_engine_download_vertex_data": ("status", [c_vp, c_vp, c_vp]),
    "gas_engine_download_vertex_data_async": ("status", [c_vp, c_vp, c_vp]),
    "gas_engine_run_schedule": ("status", [c_vp, c_i32, c_i32, C.POINTER(RunStats), c_vp]),
    "gas_engine_run_user": ("status", [c_vp, c_vp, c_vp, c_i32, c_i32, C.POINTER(RunStats),
                                       c_vp]),
    "gas_engine_pagerank_precision": ("status", [c_vp, c_dbl, c_dbl, c_i32, c_vp,
                                                 C.POINTER(RunStats), c_vp]),
    "gas_pagerank_step_noalloc": ("status", [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp,
                                             c_dbl, c_vp, c_vp]),
    "gas_engine_set_profiling": ("status", [c_vp, c_i32]),
    "gas_engine_get_profile": ("status", [c_vp, C.POINTER(KernelProfile), c_i32]),
    "gas_mlp_create": ("status", [c_i32, c_i32, c_u64, C.POINTER(c_vp)]),
    "gas_mlp_destroy": (None, [c_vp]),
    "gas_mlp_num_params": (c_i64, [c_vp]),
    "gas_mlp_get_params": ("status", [c_vp, c_vp]),
    "gas_mlp_set_params": ("status", [c_vp, c_vp]),
    "gas_mlp_gradients": ("status", [c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp]),
    "gas_mlp_train_step": ("status", [c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, C.c_float, c_vp,
                                      c_vp]),
    "gas_mlp_forward": ("status", [c_vp, c_vp, c_i32, c_vp, c_vp]),
    "gas_engine_set_trace": ("status", [c_vp, c_i32]),
    "gas_engine_get_trace": ("status", [c_vp, c_vp, c_i32, P_i32]),
    "gas_schedule_features": (None, [c_vp, c_i32, c_i64, c_i32, c_vp]),
    "gas_engine_set_schedule_model": ("status", [c_vp, c_vp]),
    "gas_engine_pagerank_warm_start": ("status", [c_vp, c_vp, c_dbl, c_vp, c_vp]),
    "gas_engine_pagerank_precision_from": ("status", [c_vp, c_dbl, c_dbl, c_i32, c_vp, c_vp,
                                                      C.POINTER(RunStats), c_vp]),
    "gas_engine_ppr_precision": ("status", [c_vp, c_i32, c_dbl, c_dbl, c_i32, c_vp,
                                            C.POINTER(RunStats), c_vp]),
    "gas_batch_create": ("status", [C.POINTER(c_vp)]),
    "gas_batch_destroy": (None, [c_vp]),
    "gas_batch_add_graph": ("status", [c_vp, c_i32, c_i64, c_vp, c_vp, C.POINTER(c_i32)]),
    "gas_batch_add_graph_weighted": ("status", [c_vp, c_i32, c_i64, c_vp, c_vp, c_vp,
                                                C.POINTER(c_i32)]),
    "gas_batch_build": ("status", [c_vp, c_vp]),
    "gas_batch_num_graphs": (c_i32, [c_vp]),
    "gas_batch_num_vertices": (c_i32, [c_vp]),
    "gas_batch_num_edges": (c_i64, [c_vp]),
    "gas_batch_vertex_offset": (c_i32, [c_vp, c_i32]),
    "gas_batch_run": ("status", [c_vp, C.POINTER(BatchJob), c_vp, c_vp, c_vp,
                                 C.POINTER(BatchStats), c_vp]),
    "gas_batch_set_profiling": ("status", [c_vp, c_i32]),
    "gas_batch_get_profile": ("status", [c_vp, C.POINTER(KernelProfile), c_i32]),
    "gas_batch_tune": ("status", [c_vp, c_i32, c_dbl, c_i32, C.POINTER(c_i32),
                                  C.POINTER(C.c_float), c_vp]),
    "gas_engine_set_edge_placement": ("status", [c_vp, c_i32]),
    "gas_engine_download_graph": ("status", [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "gas_engine_prepare_scatter": ("status", [c_vp, C.POINTER(c_vp), c_vp]),
    "gas_engine_view_get": ("status", [c_vp, c_vp]),
    "gas_engine_note_applied": ("status", [c_vp, c_i32]),
    "gas_engine_read_counters": ("status", [c_vp, C.POINTER(Counters), c_vp]),
}


def lib_path() -> Path:
    return Path(os.environ.get("GAS_LIB", str(LIB)))


def load():
    """Loads libgas.so (building it first if it is missing) and binds every
    entry point of include/gas.h."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not path.exists():
            from .build import build
            build()
        lib = C.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = c_i32 if res == "status" else res
        _lib = lib
        return lib


def check(status: int, where: str) -> None:
    if status != 0:
        lib = load()
        detail = lib.gas_last_error().decode(errors="replace")
        raise GasError(status, where, detail)


def call(name: str, *args):
    """Calls a status-returning entry point and raises GasError on failure."""
    lib = load()
    st = getattr(lib, name)(*args)
    check(st, name)


def exported_symbols() -> list[str]:
    return sorted(_SIGS)
