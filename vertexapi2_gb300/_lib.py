"""ctypes binding of libgas_gb300.so (the C ABI in include/gas_gb300.h).

The library is built in-tree by ``vertexapi2_gb300.build`` (or
``__graft_entry__.build()``); loading never falls back to anything else:
if the shared library is missing, :func:`load` raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB

GAS_OK = 0
STATUS_NAMES = {
    0: "GAS_OK", 1: "GAS_ERR_INVALID", 2: "GAS_ERR_OOM", 3: "GAS_ERR_CUDA",
    4: "GAS_ERR_TIMEOUT", 5: "GAS_ERR_STATE", 6: "GAS_ERR_UNSUPPORTED", 7: "GAS_ERR_NO_DEVICE",
}

PROGRAM_BFS = 1
PROGRAM_SSSP = 2
PROGRAM_CC = 3
PROGRAM_PAGERANK = 4
PROGRAM_PPR = 5


class GasError(RuntimeError):
    """A C-ABI call returned a non-zero gas_status."""

    def __init__(self, status: int, where: str, message: str):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {message}")


class EdgeList(C.Structure):
    _fields_ = [("nVertices", C.c_int32), ("nEdges", C.c_int64),
                ("srcs", C.POINTER(C.c_int32)), ("dsts", C.POINTER(C.c_int32)),
                ("weights", C.POINTER(C.c_int32))]


class ServerConfig(C.Structure):
    _fields_ = [("lanes", C.c_int32), ("maxBatch", C.c_int32), ("reserveBytes", C.c_int64)]


class QueryInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("program", C.c_int32), ("graph", C.c_int32),
                ("source", C.c_int32), ("rounds", C.c_int32), ("batchSize", C.c_int32),
                ("lane", C.c_int32), ("pad", C.c_int32), ("submitNs", C.c_int64),
                ("admitNs", C.c_int64), ("doneNs", C.c_int64)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "submitted", "completed", "failed", "batches", "batchedQueries", "memoryWaits",
        "bytesInUse", "peakBytesInUse", "pending", "running", "kernelLaunches")]


_P = C.c_void_p
_I32 = C.c_int32
_PI32 = C.POINTER(C.c_int32)
_PI64 = C.POINTER(C.c_int64)

# name -> (restype, argtypes); every symbol include/gas_gb300*.h declares
SIGNATURES = {
    # engine layer
    "gas_engine_create": (_I32, [_I32, _I32, _P, C.POINTER(_P)]),
    "gas_engine_destroy": (_I32, [_P]),
    "gas_engine_set_graph": (_I32, [_P, _I32, _P, _I32, _P, _PI32, _PI32]),
    "gas_engine_get_results": (_I32, [_P]),
    "gas_engine_set_vertex_data": (_I32, [_P, _P]),
    "gas_engine_set_active": (_I32, [_P, _I32, _I32]),
    "gas_engine_count_active": (_I32, [_P, _PI32]),
    "gas_engine_gather_apply": (_I32, [_P, _I32]),
    "gas_engine_scatter_activate": (_I32, [_P, _I32]),
    "gas_engine_next_iter": (_I32, [_P, _PI32]),
    "gas_engine_run": (_I32, [_P, _I32, _PI32]),
    "gas_engine_set_iteration": (_I32, [_P, _I32]),
    "gas_engine_round_stats": (_I32, [_P, _I32, _PI64, _PI64, _PI64, _PI64, _PI32]),
    "gas_engine_last_run_ms": (_I32, [_P, C.POINTER(C.c_float)]),
    "gas_engine_save_vertex_data": (_I32, [_P]),
    "gas_engine_restore_vertex_data": (_I32, [_P]),
    "gas_engine_set_profiling": (_I32, [_P, _I32]),
    "gas_engine_set_launch_config": (_I32, [_P, _I32, _I32]),
    "gas_engine_set_dense_policy": (_I32, [_P, _I32]),
    "gas_engine_set_fused_rounds": (_I32, [_P, _I32]),
    "gas_engine_kernel_times": (_I32, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), _PI32, _PI32]),
    "gas_bfs_noalloc": (_I32, [_I32, _I32, _P, _P, _I32, _P, _P, _PI32]),
    "gas_batch_create": (_I32, [_I32, _P, C.POINTER(_P)]),
    "gas_batch_destroy": (_I32, [_P]),
    "gas_batch_set_graph": (_I32, [_P, _I32, _I32, _PI32, _PI32, _PI32]),
    "gas_batch_run": (_I32, [_P, _I32, _I32, _PI32, _PI32, _PI32]),
    "gas_batch_set_config": (_I32, [_P, _I32, _I32, _I32]),
    "gas_batch_autotune": (_I32, [_P, _I32, _I32, _PI32, _PI32]),
    "gas_batch_last_ms": (_I32, [_P, C.POINTER(C.c_float)]),
    "gas_batch_set_policy": (_I32, [_P, _I32]),
    "gas_batch_set_delta": (_I32, [_P, _I32]),
    "gas_batch_set_frontier": (_I32, [_P, _I32]),
    "gas_batch_get_delta": (_I32, [_P, _PI32]),
    "gas_batch_get_tuning": (_I32, [_P, _PI32, _PI32, _PI32, _PI32, _PI32]),
    # serving loop
    "gas_server_create": (_I32, [_I32, C.POINTER(ServerConfig), C.POINTER(_P)]),
    "gas_server_destroy": (_I32, [_P]),
    "gas_server_add_graph": (_I32, [_P, _I32, _I32, _PI32, _PI32, _PI32, _PI32]),
    "gas_server_submit": (_I32, [_P, _I32, _I32, _I32, C.POINTER(C.c_uint64)]),
    "gas_server_wait": (_I32, [_P, C.c_uint64, _I32, _P, C.c_int64, C.POINTER(QueryInfo)]),
    "gas_server_poll": (_I32, [_P, C.c_uint64, _PI32]),
    "gas_server_get_stats": (_I32, [_P, C.POINTER(ServerStats)]),
    # diagnostics
    "gas_status_string": (C.c_char_p, [_I32]),
    "gas_last_error": (C.c_char_p, []),
    "gas_device_supported": (_I32, [_I32]),
    "gas_selftest_bounded_waits": (_I32, [_I32, _PI32, _PI32, C.POINTER(C.c_float)]),
    # generators
    "gas_gen_rmat": (_I32, [_I32, _I32, C.c_double, C.c_double, C.c_double, C.c_uint64, _I32,
                            _I32, _I32, C.POINTER(EdgeList)]),
    "gas_gen_grid": (_I32, [_I32, _I32, C.c_double, C.c_uint64, _I32, _I32, C.POINTER(EdgeList)]),
    "gas_edge_list_free": (None, [C.POINTER(EdgeList)]),
    # graph files
    "gas_load_graph": (_I32, [C.c_char_p, _I32, C.POINTER(EdgeList)]),
    "gas_write_graph_mtx": (_I32, [C.c_char_p, _I32, C.c_int64, _PI32, _PI32, _PI32]),
    "gas_write_graph_gr": (_I32, [C.c_char_p, _I32, C.c_int64, _PI32, _PI32, _PI32]),
    "gas_write_vertex_values": (_I32, [C.c_char_p, _I32, _P, _I32, _I32]),
    # core layer
    "gas_core_create": (_I32, [_I32, _P, C.POINTER(_P)]),
    "gas_core_destroy": (_I32, [_P]),
    "gas_core_stream": (_I32, [_P, C.POINTER(_P)]),
    "gas_core_set_graph": (_I32, [_P, _I32, _I32, _PI32, _PI32, _P, _I32, _I32, _I32]),
    "gas_core_upload_vertex_data": (_I32, [_P, _P]),
    "gas_core_download_vertex_data": (_I32, [_P, _P]),
    "gas_core_download_edge_data": (_I32, [_P, _P]),
    "gas_core_vertex_data": (_I32, [_P, C.POINTER(_P)]),
    "gas_core_set_active": (_I32, [_P, _I32, _I32]),
    "gas_core_count_active": (_I32, [_P, _PI32]),
    "gas_core_set_iteration": (_I32, [_P, _I32]),
    "gas_core_gather_apply": (_I32, [_P, _I32, _P, _P]),
    "gas_core_scatter_activate": (_I32, [_P]),
    "gas_core_next_iter": (_I32, [_P]),
    "gas_core_run": (_I32, [_P, _I32, _I32, _P, _P, _PI32]),
    "gas_core_run_persistent": (_I32, [_P, _I32, _I32, _P, _P, _P, _PI32]),
    "gas_core_round_stats": (_I32, [_P, _I32, _PI64, _PI64, _PI64, _PI64, _PI32]),
    "gas_core_last_run_ms": (_I32, [_P, C.POINTER(C.c_float)]),
    "gas_core_sync": (_I32, [_P]),
    "gas_core_save_vertex_data": (_I32, [_P]),
    "gas_core_restore_vertex_data": (_I32, [_P]),
    "gas_core_set_profiling": (_I32, [_P, _I32]),
    "gas_core_set_dense_policy": (_I32, [_P, _I32]),
    "gas_core_set_fused_rounds": (_I32, [_P, _I32]),
    "gas_core_kernel_times": (_I32, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), _PI32, _PI32]),
    "gas_core_enable_edge_scatter": (_I32, [_P, _I32]),
    "gas_core_edge_scatter": (_I32, [_P, _P, _P]),
}

_lib = None


def load() -> C.CDLL:
    """Loads the in-tree library (raises FileNotFoundError when not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError(
            f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, where: str) -> None:
    if status != GAS_OK:
        msg = load().gas_last_error()
        raise GasError(status, where, msg.decode() if msg else "")
