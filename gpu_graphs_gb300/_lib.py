"""ctypes binding of libgbfs.so (the C ABI declared in include/gbfs.h).

The library is built in-tree by gpu_graphs_gb300/build.py.  Importing this
module without it raises ImportError: there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

# GBFS_LIBRARY names another build of the same library (e.g. to compare two builds)
LIB_PATH = Path(os.environ.get("GBFS_LIBRARY") or Path(__file__).resolve().parent / "libgbfs.so")

OK = 0
ERR_INVALID_ARG = -1
ERR_OOM = -2
ERR_CUDA = -3
ERR_TIMEOUT = -4
ERR_TOO_LARGE = -5
ERR_IO = -6
ERR_BUDGET = -7
ERR_NOT_FOUND = -8
ERR_SHUTDOWN = -9

SYMMETRIZE = 1
DEDUP = 2
DROP_SELF_LOOPS = 4
UNDIRECTED = SYMMETRIZE | DEDUP | DROP_SELF_LOOPS
HUB_FIRST = 8
WIDE_ROWS = 16

DIR_OPTIMIZING = 0
DIR_TOPDOWN = 1
DIR_BOTTOMUP = 2


class Stats(C.Structure):
    _fields_ = [
        ("ms", C.c_float),
        ("levels", C.c_int32),
        ("td_levels", C.c_int32),
        ("bu_levels", C.c_int32),
        ("launches", C.c_int32),
        ("vertices_reached", C.c_int64),
        ("edges_in_component", C.c_int64),
        ("edges_traversed", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Params(C.Structure):
    _fields_ = [
        ("threads_per_block", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("alpha", C.c_int32),
        ("beta", C.c_int32),
        ("big_degree", C.c_int32),
        ("direction", C.c_int32),
        ("per_level_launch", C.c_int32),
        ("timeout_ms", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class GraphInfo(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("max_degree", C.c_int32),
        ("m", C.c_int64),
        ("nonisolated", C.c_int64),
        ("device_bytes", C.c_int64),
        ("wide", C.c_int32),
        ("reserved", C.c_int32),
    ]


class LevelTrace(C.Structure):
    _fields_ = [
        ("level", C.c_int32),
        ("direction", C.c_int32),
        ("frontier_vertices", C.c_int64),
        ("frontier_edges", C.c_int64),
        ("t_us", C.c_double),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("mem_budget_bytes", C.c_int64),
        ("num_slots", C.c_int32),
        ("max_lanes", C.c_int32),
        ("batch_window_us", C.c_int32),
        ("timeout_ms", C.c_int32),
        ("window_pct", C.c_int32),
    ]


class QueryInfo(C.Structure):
    _fields_ = [
        ("latency_ms", C.c_double),
        ("queue_ms", C.c_double),
        ("batch_lanes", C.c_int32),
        ("status", C.c_int32),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("completed", C.c_int64),
        ("launches", C.c_int64),
        ("rejected", C.c_int64),
        ("p50_ms", C.c_double),
        ("p99_ms", C.c_double),
        ("mean_ms", C.c_double),
        ("max_ms", C.c_double),
        ("mean_batch_lanes", C.c_double),
        ("resident_bytes", C.c_int64),
        ("peak_bytes", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
PI32 = C.POINTER(C.c_int32)
PI64 = C.POINTER(C.c_int64)

# name -> (restype, argtypes)
SIGNATURES = {
    "gbfs_strerror": (C.c_char_p, [C.c_int]),
    "gbfs_last_error": (C.c_char_p, []),
    "gbfs_version": (C.c_char_p, []),
    "gbfs_graph_from_edges": (C.c_int, [I32, I64, P, P, C.c_uint32, C.POINTER(P)]),
    "gbfs_graph_from_csr": (C.c_int, [I32, I64, P, P, C.POINTER(P)]),
    "gbfs_graph_destroy": (None, [P]),
    "gbfs_graph_get_info": (C.c_int, [P, C.POINTER(GraphInfo)]),
    "gbfs_graph_get_csr": (C.c_int, [P, P, P]),
    "gbfs_graph_get_csr64": (C.c_int, [P, P, P]),
    "gbfs_default_params": (C.c_int, [C.POINTER(Params)]),
    "gbfs_get_params": (C.c_int, [P, C.POINTER(Params)]),
    "gbfs_set_params": (C.c_int, [P, C.POINTER(Params)]),
    "gbfs_autotune": (C.c_int, [P, P, I32, C.POINTER(Params)]),
    "gbfs_bfs": (C.c_int, [P, I32, P, C.POINTER(Stats)]),
    "gbfs_bfs_parents": (C.c_int, [P, I32, P, P, C.POINTER(Stats)]),
    "gbfs_bfs_multiroot": (C.c_int, [P, P, I32, P, C.POINTER(Stats)]),
    "gbfs_bfs_many": (C.c_int, [P, P, I32, P, P]),
    "gbfs_graph_stream": (C.c_void_p, [P]),
    "gbfs_last_trace": (C.c_int, [P, P, I32]),
    "gbfs_bfs_multi": (C.c_int, [P, P, I32, P, C.POINTER(Stats)]),
    "gbfs_graphset_from_edges": (C.c_int, [I32, P, P, P, P, C.c_uint32, C.POINTER(P)]),
    "gbfs_graphset_from_graphs": (C.c_int, [I32, P, C.POINTER(P)]),
    "gbfs_graphset_destroy": (None, [P]),
    "gbfs_graphset_vertex_offsets": (C.c_int, [P, P]),
    "gbfs_bfs_batch": (C.c_int, [P, P, P, C.POINTER(Stats)]),
    "gbfs_bfs_batch_graphs": (C.c_int, [P, P, I32, P, C.POINTER(Stats)]),
    "gbfs_exclusive_scan_i32": (C.c_int, [P, P, I64, P]),
    "gbfs_exclusive_scan_i32_noalloc": (C.c_int, [P, P, I64, P]),
    "gbfs_read_edge_list": (C.c_int, [C.c_char_p, I32, PI32, PI64, C.POINTER(PI32), C.POINTER(PI32)]),
    "gbfs_free": (None, [P]),
    "gbfs_graph_save": (C.c_int, [P, C.c_char_p]),
    "gbfs_graph_load": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "gbfs_gen_er": (I64, [I32, I64, C.c_uint64, P, P, I64]),
    "gbfs_gen_rmat": (I64, [I32, I32, C.c_double, C.c_double, C.c_double, C.c_uint64, P, P, I64]),
    "gbfs_gen_grid": (I64, [I32, C.c_double, C.c_double, I32, C.c_uint64, P, P, I64]),
    "gbfs_gen_grid_capacity": (I64, [I32, C.c_double]),
    "gbfs_selftest_wait_timeout": (C.c_int, [I32]),
    "gbfs_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(P)]),
    "gbfs_server_destroy": (None, [P]),
    "gbfs_server_add_graph": (C.c_int, [P, P, PI32]),
    "gbfs_server_remove_graph": (C.c_int, [P, I32]),
    "gbfs_server_submit": (C.c_int, [P, I32, I32, P, PI64]),
    "gbfs_server_wait": (C.c_int, [P, I64, I32, C.POINTER(QueryInfo)]),
    "gbfs_server_get_stats": (C.c_int, [P, C.POINTER(ServerStats)]),
    "gbfs_server_reset_stats": (None, [P]),
}



def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()' or python gpu_graphs_gb300/build.py)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


class GbfsError(RuntimeError):
    """A non-zero status from libgbfs.so."""

    def __init__(self, code: int, where: str = ""):
        self.code = code
        detail = lib.gbfs_last_error().decode(errors="replace")
        msg = f"{where}: {lib.gbfs_strerror(code).decode()} ({code})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


def check(rc: int, where: str = "") -> int:
    if rc != OK:
        raise GbfsError(rc, where)
    return rc
