"""gpu_graphs_gb300 -- GB300-native BFS engine (Python side).

Everything here is a thin layer over libgbfs.so (include/gbfs.h): graphs
live in HBM behind opaque handles and every traversal runs in hand-written
sm_103a kernels.  Arrays may be numpy (host) or torch CUDA tensors
(device); outputs default to numpy.

Two layers:
  * Graph / GraphSet / Server -- the engine API.
  * csr / gpuBFS -- the reference's host interface (1D Partition/include/
    csr.h:9-23 and gpuBFS.cuh:9-54): same class names, constructor
    arguments and public members (row_offset, col_idx, num_nodes,
    num_edges; host_distance, exec_time, total_edges_traversed, iteration).
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from typing import Iterable, Sequence

import numpy as np

# The server runs its slots' searches on many streams at once; CUDA's
# default of 8 hardware work queues per process serialises most of them.
# Effective only when this import comes before the process's first CUDA call.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import _lib
from ._lib import (DEDUP, DIR_BOTTOMUP, DIR_OPTIMIZING, DIR_TOPDOWN, DROP_SELF_LOOPS, HUB_FIRST, SYMMETRIZE,
                   UNDIRECTED, WIDE_ROWS, GbfsError, Params, Stats, check, lib)

__all__ = [
    "Graph", "GraphSet", "Server", "GbfsError", "Params", "Stats", "csr", "gpuBFS",
    "read_edge_list", "gen_er", "gen_rmat", "gen_grid", "exclusive_scan", "default_params",
    "SYMMETRIZE", "DEDUP", "DROP_SELF_LOOPS", "UNDIRECTED", "HUB_FIRST", "WIDE_ROWS", "DIR_OPTIMIZING", "DIR_TOPDOWN",
    "DIR_BOTTOMUP", "library_path",
]


def library_path() -> str:
    return str(_lib.LIB_PATH)


def _is_torch_cuda(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


def _ptr_i32(x, name: str = "array"):
    """(pointer, keepalive) for an int32 host array or CUDA tensor."""
    if _is_torch_cuda(x):
        import torch
        if x.dtype != torch.int32 or not x.is_contiguous():
            raise ValueError(f"{name} must be a contiguous int32 CUDA tensor")
        return C.c_void_p(x.data_ptr()), x
    a = np.ascontiguousarray(x, dtype=np.int32)
    return C.c_void_p(a.ctypes.data), a


def default_params() -> Params:
    p = Params()
    check(lib.gbfs_default_params(C.byref(p)), "gbfs_default_params")
    return p


class Graph:
    """A CSR graph resident in HBM (wraps gbfs_graph*)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        info = _lib.GraphInfo()
        check(lib.gbfs_graph_get_info(self._h, C.byref(info)), "gbfs_graph_get_info")
        self.n = info.n
        self.m = info.m
        self.max_degree = info.max_degree
        self.nonisolated = info.nonisolated
        self.wide = bool(info.wide)  # 64-bit row offsets

    # ---- construction ----
    @classmethod
    def from_edges(cls, n: int, src, dst, flags: int = UNDIRECTED) -> "Graph":
        ps, ks = _ptr_i32(src, "src")
        pd, kd = _ptr_i32(dst, "dst")
        m = len(ks) if not _is_torch_cuda(ks) else ks.numel()
        if (len(kd) if not _is_torch_cuda(kd) else kd.numel()) != m:
            raise ValueError("src and dst differ in length")
        h = C.c_void_p()
        check(lib.gbfs_graph_from_edges(int(n), int(m), ps, pd, int(flags), C.byref(h)), "gbfs_graph_from_edges")
        return cls(h)

    @classmethod
    def from_csr(cls, row_offset, col_idx) -> "Graph":
        pr, kr = _ptr_i32(row_offset, "row_offset")
        pc, kc = _ptr_i32(col_idx, "col_idx")
        n = (len(kr) if not _is_torch_cuda(kr) else kr.numel()) - 1
        m = len(kc) if not _is_torch_cuda(kc) else kc.numel()
        h = C.c_void_p()
        check(lib.gbfs_graph_from_csr(int(n), int(m), pr, pc, C.byref(h)), "gbfs_graph_from_csr")
        return cls(h)

    @classmethod
    def load(cls, path: str) -> "Graph":
        h = C.c_void_p()
        check(lib.gbfs_graph_load(str(path).encode(), C.byref(h)), "gbfs_graph_load")
        return cls(h)

    def save(self, path: str) -> None:
        check(lib.gbfs_graph_save(self._h, str(path).encode()), "gbfs_graph_save")

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.gbfs_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def info(self) -> dict:
        info = _lib.GraphInfo()
        check(lib.gbfs_graph_get_info(self._h, C.byref(info)), "gbfs_graph_get_info")
        return {k: getattr(info, k) for k, _ in info._fields_}

    def csr(self) -> tuple[np.ndarray, np.ndarray]:
        """(row offsets, column ids); the offsets are int64 on a wide graph."""
        row = np.empty(self.n + 1, np.int64 if self.wide else np.int32)
        col = np.empty(max(self.m, 1), np.int32)
        fn = lib.gbfs_graph_get_csr64 if self.wide else lib.gbfs_graph_get_csr
        check(fn(self._h, C.c_void_p(row.ctypes.data), C.c_void_p(col.ctypes.data)), "gbfs_graph_get_csr")
        return row, col[: self.m]

    def row_offsets(self) -> np.ndarray:
        """The n + 1 row offsets alone, as int64."""
        row = np.empty(self.n + 1, np.int64)
        check(lib.gbfs_graph_get_csr64(self._h, C.c_void_p(row.ctypes.data), None), "gbfs_graph_get_csr64")
        return row

    # ---- parameters ----
    @property
    def params(self) -> Params:
        p = Params()
        check(lib.gbfs_get_params(self._h, C.byref(p)), "gbfs_get_params")
        return p

    def set_params(self, p: Params | None = None, **kw) -> None:
        q = Params.from_buffer_copy(p) if p is not None else self.params
        for k, v in kw.items():
            setattr(q, k, int(v))
        check(lib.gbfs_set_params(self._h, C.byref(q)), "gbfs_set_params")

    def autotune(self, sources: Sequence[int]) -> Params:
        s = np.ascontiguousarray(sources, np.int32)
        p = Params()
        check(lib.gbfs_autotune(self._h, C.c_void_p(s.ctypes.data), len(s), C.byref(p)), "gbfs_autotune")
        return p

    # ---- traversal ----
    def bfs(self, source: int, out=None, stats: bool = False):
        """Levels from `source` (int32, -1 unreachable); out: host array or CUDA tensor."""
        if out is None:
            out = np.empty(self.n, np.int32)
        po, ko = _ptr_i32(out, "out") if _is_torch_cuda(out) else (C.c_void_p(out.ctypes.data), out)
        st = Stats()
        check(lib.gbfs_bfs(self._h, int(source), po, C.byref(st)), "gbfs_bfs")
        return (out, st) if stats else out

    def bfs_parents(self, source: int, levels=None, parents=None, stats: bool = False):
        """Levels and canonical BFS-tree parents (smallest neighbour one level
        closer; -1 for the source and unreached vertices).  levels/parents:
        host arrays or CUDA tensors of n int32.  Returns (levels, parents[, stats])."""
        if levels is None:
            levels = np.empty(self.n, np.int32)
        if parents is None:
            parents = np.empty(self.n, np.int32)
        for name, a in (("levels", levels), ("parents", parents)):
            if not _is_torch_cuda(a) and (a.dtype != np.int32 or not a.flags.c_contiguous or a.size != self.n):
                raise ValueError(f"{name} must be a contiguous int32 array of n entries")
        pl = _ptr_i32(levels, "levels")[0] if _is_torch_cuda(levels) else C.c_void_p(levels.ctypes.data)
        pp = _ptr_i32(parents, "parents")[0] if _is_torch_cuda(parents) else C.c_void_p(parents.ctypes.data)
        st = Stats()
        check(lib.gbfs_bfs_parents(self._h, int(source), pl, pp, C.byref(st)), "gbfs_bfs_parents")
        return (levels, parents, st) if stats else (levels, parents)

    def bfs_many(self, sources: Sequence[int], out=None, keep: bool = True):
        """One launch per source, back to back on the graph's stream.

        out: (k, n) host array or CUDA tensor; keep=False discards levels.
        Returns (levels or None, list of Stats)."""
        s = np.ascontiguousarray(sources, np.int32)
        k = len(s)
        if out is None and keep:
            out = np.empty((k, self.n), np.int32)
        po = None if out is None else (C.c_void_p(out.data_ptr()) if _is_torch_cuda(out)
                                       else C.c_void_p(out.ctypes.data))
        sts = (Stats * k)()
        check(lib.gbfs_bfs_many(self._h, C.c_void_p(s.ctypes.data), k, po, C.cast(sts, C.c_void_p)),
              "gbfs_bfs_many")
        return out, list(sts)

    def last_trace(self) -> list[dict]:
        """Per-level trace of the last traversal: level, direction, frontier
        size and edges, and the step's end time in us after initialisation."""
        cap = 16384 + 3
        rows = (_lib.LevelTrace * cap)()
        k = lib.gbfs_last_trace(self._h, C.cast(rows, C.c_void_p), cap)
        if k < 0:
            raise GbfsError(k, "gbfs_last_trace")
        dirs = {-3: "exit", -2: "end", -1: "init", 0: "td", 1: "bu", 2: "td+split", 4: "relaxed"}
        return [{"level": r.level, "dir": dirs.get(r.direction, str(r.direction)), "frontier": r.frontier_vertices,
                 "edges": r.frontier_edges, "t_us": round(r.t_us, 2)} for r in rows[:k]]

    @property
    def stream(self) -> int:
        """The cudaStream_t (as an integer) this graph's work runs on."""
        return int(lib.gbfs_graph_stream(self._h) or 0)

    def bfs_multiroot(self, sources: Sequence[int], out=None, stats: bool = False):
        s = np.ascontiguousarray(sources, np.int32)
        if out is None:
            out = np.empty(self.n, np.int32)
        po = C.c_void_p(out.data_ptr()) if _is_torch_cuda(out) else C.c_void_p(out.ctypes.data)
        st = Stats()
        check(lib.gbfs_bfs_multiroot(self._h, C.c_void_p(s.ctypes.data), len(s), po, C.byref(st)),
              "gbfs_bfs_multiroot")
        return (out, st) if stats else out

    def bfs_multi(self, sources: Sequence[int], out=None, stats: bool = False):
        """One level array per source, 64 sources per launch: shape (k, n)."""
        s = np.ascontiguousarray(sources, np.int32)
        if out is None:
            out = np.empty((len(s), self.n), np.int32)
        po = C.c_void_p(out.data_ptr()) if _is_torch_cuda(out) else C.c_void_p(out.ctypes.data)
        st = Stats()
        check(lib.gbfs_bfs_multi(self._h, C.c_void_p(s.ctypes.data), len(s), po, C.byref(st)), "gbfs_bfs_multi")
        return (out, st) if stats else out


class GraphSet:
    """Many small graphs as one disjoint-union CSR; one fused BFS launch."""

    def __init__(self, handle: C.c_void_p, sizes: list[int]):
        self._h = handle
        self.sizes = sizes
        off = np.empty(len(sizes) + 1, np.int64)
        check(lib.gbfs_graphset_vertex_offsets(self._h, C.c_void_p(off.ctypes.data)), "gbfs_graphset_vertex_offsets")
        self.offsets = off

    @classmethod
    def from_edges(cls, graphs: Sequence[tuple[int, np.ndarray, np.ndarray]], flags: int = UNDIRECTED):
        count = len(graphs)
        ns = np.array([g[0] for g in graphs], np.int32)
        keep = [(np.ascontiguousarray(g[1], np.int32), np.ascontiguousarray(g[2], np.int32)) for g in graphs]
        ms = np.array([len(k[0]) for k in keep], np.int64)
        sp = (C.c_void_p * count)(*[k[0].ctypes.data for k in keep])
        dp = (C.c_void_p * count)(*[k[1].ctypes.data for k in keep])
        h = C.c_void_p()
        check(lib.gbfs_graphset_from_edges(count, C.c_void_p(ns.ctypes.data), C.c_void_p(ms.ctypes.data),
                                           C.cast(sp, C.c_void_p), C.cast(dp, C.c_void_p), int(flags), C.byref(h)),
              "gbfs_graphset_from_edges")
        return cls(h, [int(x) for x in ns])

    @classmethod
    def from_graphs(cls, graphs: Sequence[Graph]):
        arr = (C.c_void_p * len(graphs))(*[g.handle.value for g in graphs])
        h = C.c_void_p()
        check(lib.gbfs_graphset_from_graphs(len(graphs), C.cast(arr, C.c_void_p), C.byref(h)),
              "gbfs_graphset_from_graphs")
        return cls(h, [g.n for g in graphs])

    def bfs(self, sources: Sequence[int], stats: bool = False):
        s = np.ascontiguousarray(sources, np.int32)
        outs = [np.empty(n, np.int32) for n in self.sizes]
        ptrs = (C.c_void_p * len(outs))(*[o.ctypes.data for o in outs])
        st = Stats()
        check(lib.gbfs_bfs_batch(self._h, C.c_void_p(s.ctypes.data), C.cast(ptrs, C.c_void_p), C.byref(st)),
              "gbfs_bfs_batch")
        return (outs, st) if stats else outs

    def close(self):
        if getattr(self, "_h", None):
            lib.gbfs_graphset_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bfs_batch_graphs(graphs: Sequence[Graph], sources: Sequence[int], stats: bool = False):
    s = np.ascontiguousarray(sources, np.int32)
    arr = (C.c_void_p * len(graphs))(*[g.handle.value for g in graphs])
    outs = [np.empty(g.n, np.int32) for g in graphs]
    ptrs = (C.c_void_p * len(outs))(*[o.ctypes.data for o in outs])
    st = Stats()
    check(lib.gbfs_bfs_batch_graphs(C.cast(arr, C.c_void_p), C.c_void_p(s.ctypes.data), len(graphs),
                                    C.cast(ptrs, C.c_void_p), C.byref(st)), "gbfs_bfs_batch_graphs")
    return (outs, st) if stats else outs


# ---- primitives, files, generators ---------------------------------------------------

def exclusive_scan(x, stream: int = 0):
    """Exclusive prefix sum of a CUDA int32 tensor into a new int64 tensor."""
    import torch
    if not _is_torch_cuda(x) or x.dtype != torch.int32:
        raise ValueError("x must be an int32 CUDA tensor")
    x = x.contiguous()
    out = torch.empty(x.numel(), dtype=torch.int64, device=x.device)
    check(lib.gbfs_exclusive_scan_i32(C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr()), x.numel(),
                                      C.c_void_p(stream)), "gbfs_exclusive_scan_i32")
    return out


def read_edge_list(path: str, one_based: bool = True) -> tuple[int, np.ndarray, np.ndarray]:
    """Parse the reference's text format ("n", "m", then "from to" pairs)."""
    n = C.c_int32()
    m = C.c_int64()
    ps = _lib.PI32()
    pd = _lib.PI32()
    check(lib.gbfs_read_edge_list(str(path).encode(), int(one_based), C.byref(n), C.byref(m), C.byref(ps),
                                  C.byref(pd)), "gbfs_read_edge_list")
    try:
        src = np.ctypeslib.as_array(ps, shape=(max(m.value, 1),))[: m.value].copy()
        dst = np.ctypeslib.as_array(pd, shape=(max(m.value, 1),))[: m.value].copy()
    finally:
        lib.gbfs_free(C.cast(ps, C.c_void_p))
        lib.gbfs_free(C.cast(pd, C.c_void_p))
    return n.value, src, dst


def _gen_call(fn, cap: int, *args):
    src = np.empty(max(cap, 1), np.int32)
    dst = np.empty(max(cap, 1), np.int32)
    r = fn(*args, C.c_void_p(src.ctypes.data), C.c_void_p(dst.ctypes.data), cap)
    if r < 0:
        raise GbfsError(int(r), fn.__name__)
    return src[:r], dst[:r]


def gen_er(n: int, pairs: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    return _gen_call(lib.gbfs_gen_er, pairs, int(n), int(pairs), int(seed))


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    cap = (1 << scale) * edge_factor
    return _gen_call(lib.gbfs_gen_rmat, cap, int(scale), int(edge_factor), float(a), float(b), float(c), int(seed))


def gen_grid(side: int, drop: float = 0.1, extra: float = 0.001, radius: int = 8,
             seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    cap = int(lib.gbfs_gen_grid_capacity(int(side), float(extra)))
    if cap < 0:
        raise GbfsError(cap, "gbfs_gen_grid_capacity")
    return _gen_call(lib.gbfs_gen_grid, cap, int(side), float(drop), float(extra), int(radius), int(seed))


# ---- the reference's host interface -----------------------------------------------------

class csr:
    """Mirror of the reference's ``csr`` (1D Partition/include/csr.h:9-23).

    ``csr(filename)`` parses the text format (``n``, ``m``, then 1-based
    ``from to`` pairs, as 2D Partition/src/csc.cpp:14-25 and the migration
    loader read it), builds the CSR on the GPU with edges kept as stored
    (directed, duplicates and self-loops kept) and exposes the public
    members ``row_offset``, ``col_idx``, ``num_nodes``, ``num_edges``.
    Where the reference prints "Error: Unable to open file" and leaves a
    half-built object (csr.cpp:8-12), this prints the same line and raises.
    """

    def __init__(self, filename: str, flags: int = 0):
        try:
            n, src, dst = read_edge_list(filename, one_based=True)
        except GbfsError as e:
            if e.code == _lib.ERR_IO and "Unable to open" in str(e):
                print(f"Error: Unable to open file {filename}", file=sys.stderr)
            raise
        self.graph = Graph.from_edges(n, src, dst, flags)
        self.row_offset, self.col_idx = self.graph.csr()
        self.num_nodes = self.graph.n
        self.num_edges = self.graph.m


class gpuBFS:
    """Mirror of the reference's ``gpuBFS`` (1D Partition/include/gpuBFS.cuh:9-54).

    ``gpuBFS(graph, source)`` does all the work in the constructor, like
    1D Partition/src/gpuBFS.cu:13-116, and leaves ``host_distance`` (int32
    levels, -1 unreachable), ``exec_time`` (ms of device time),
    ``total_edges_traversed`` (discovered vertices) and ``iteration``
    (number of levels).  Errors raise GbfsError instead of exit(1).
    """

    def __init__(self, graph, source: int):
        g = graph.graph if isinstance(graph, csr) else graph
        self.host_distance, st = g.bfs(int(source), stats=True)
        self.exec_time = float(st.ms)
        self.total_edges_traversed = int(st.edges_traversed)
        self.iteration = int(st.levels)
        self.stats = st


from .server import Server  # noqa: E402  (needs Graph)
