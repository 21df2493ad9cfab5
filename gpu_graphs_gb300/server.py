"""Serving loop over HBM-resident graphs (wraps gbfs_server_* of libgbfs.so)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib


class Server:
    """Continuous-batching BFS server.

    Graphs are admitted against an HBM budget; queries are queued per graph
    and served by ``num_slots`` slots of four units (streams) each.  On most
    graphs a slot packs up to ``max_lanes`` queued sources into one
    multi-source launch; a graph's queries wait up to ``batch_window_us``,
    or ``window_pct`` percent of its recent launch time if that is longer,
    for a fuller batch.  On graphs of out-degree <= 16 (grids, meshes, road
    networks) every free unit runs one query as a single-source search and
    takes the next as soon as it ends.  Result copies are fastest into
    pinned host buffers.
    """

    def __init__(self, mem_budget_bytes: int, num_slots: int = 4, max_lanes: int = 64,
                 batch_window_us: int = 200, timeout_ms: int = 2000, window_pct: int = 0):
        cfg = _lib.ServerConfig(int(mem_budget_bytes), int(num_slots), int(max_lanes), int(batch_window_us),
                                int(timeout_ms), int(window_pct))
        self._h = C.c_void_p()
        check(lib.gbfs_server_create(C.byref(cfg), C.byref(self._h)), "gbfs_server_create")
        self._graphs = {}
        self._outs = {}

    def add_graph(self, g) -> int:
        gid = C.c_int32()
        check(lib.gbfs_server_add_graph(self._h, g.handle, C.byref(gid)), "gbfs_server_add_graph")
        self._graphs[gid.value] = g
        return gid.value

    def remove_graph(self, gid: int) -> None:
        check(lib.gbfs_server_remove_graph(self._h, int(gid)), "gbfs_server_remove_graph")
        self._graphs.pop(gid, None)

    def submit(self, gid: int, source: int, out: np.ndarray | None = None) -> int:
        g = self._graphs.get(gid)
        if out is None:
            out = np.empty(g.n if g is not None else 1, np.int32)
        t = C.c_int64()
        check(lib.gbfs_server_submit(self._h, int(gid), int(source), C.c_void_p(out.ctypes.data), C.byref(t)),
              "gbfs_server_submit")
        self._outs[t.value] = out
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        """(levels, QueryInfo) of a ticket.  If several threads wait on one
        ticket, all of them see its status; the levels array goes to one."""
        info = _lib.QueryInfo()
        rc = lib.gbfs_server_wait(self._h, int(ticket), int(timeout_ms), C.byref(info))
        check(rc, "gbfs_server_wait")
        return self._outs.pop(ticket, None), info

    def stats(self) -> dict:
        st = _lib.ServerStats()
        check(lib.gbfs_server_get_stats(self._h, C.byref(st)), "gbfs_server_get_stats")
        return st.as_dict()

    def reset_stats(self) -> None:
        lib.gbfs_server_reset_stats(self._h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.gbfs_server_destroy(self._h)
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
