"""CPU oracle for the gbfs engine -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg and
reference arm may import this package, and only as the checker or the
timed CPU baseline; the engine never calls it.

  * liboracle.so -- oracle.c, a plain-C restatement of the reference's CPU
    path (CSR build of 2D Partition/src/csc.cpp, level-synchronous BFS of
    2D Partition/src/cpuBFS.cpp, queue BFS of the migration cpuBFS.cpp),
    linked with the seeded workload generators (the engine's host-only
    gen.cpp compiled a second time), so the CPU reference arm of bench.py
    builds its graphs without loading the engine.
  * _ref/ref_c9, _ref/ref_c10 -- the reference's own CPU BFS compiled from
    its unmodified sources by oracle/Makefile, only when
    GBFS_REFERENCE_ROOT names a checkout of the reference project; used to
    pin the restatement and to make tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
# a checkout of the reference project, or None (then _ref/ is not built)
REFERENCE_ROOT = Path(os.environ["GBFS_REFERENCE_ROOT"]) if os.environ.get("GBFS_REFERENCE_ROOT") else None
GEN_SRC = HERE.parent / "gpu_graphs_gb300" / "csrc" / "gen.cpp"

SYMMETRIZE, DEDUP, DROP_SELF_LOOPS = 1, 2, 4
UNDIRECTED = 7


def reference_present() -> bool:
    return REFERENCE_ROOT is not None and REFERENCE_ROOT.exists()


def build(ref: bool = False) -> None:
    """make liboracle.so (and the reference binaries when asked and possible)."""
    targets = ["all"] + (["ref"] if ref and reference_present() else [])
    extra = [f"REF={REFERENCE_ROOT}"] if reference_present() else []
    subprocess.run(["make", "-s", "-C", str(HERE), *targets, *extra], check=True, stdout=subprocess.DEVNULL)


def _stale() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    deps = (HERE / "oracle.c", HERE / "oracle.h", GEN_SRC, HERE.parent / "include" / "gbfs.h")
    return any(p.stat().st_mtime > t for p in deps if p.exists())


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if _stale():
            build()
        L = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        L.oracle_csr_build.restype = C.c_int64
        L.oracle_csr_build.argtypes = [C.c_int32, C.c_int64, P, P, C.c_uint32, P, P]
        L.oracle_bfs_levelsync.restype = C.c_int64
        L.oracle_bfs_levelsync.argtypes = [C.c_int32, P, P, C.c_int32, P, P]
        L.oracle_bfs_queue.restype = C.c_int
        L.oracle_bfs_queue.argtypes = [C.c_int32, P, P, C.c_int32, P]
        L.oracle_bfs_queue_clock.restype = C.c_int
        L.oracle_bfs_queue_clock.argtypes = [C.c_int32, P, P, C.c_int32, P, P, P]
        L.gbfs_gen_er.restype = C.c_int64
        L.gbfs_gen_er.argtypes = [C.c_int32, C.c_int64, C.c_uint64, P, P, C.c_int64]
        L.gbfs_gen_rmat.restype = C.c_int64
        L.gbfs_gen_rmat.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_uint64, P, P,
                                    C.c_int64]
        L.gbfs_gen_grid.restype = C.c_int64
        L.gbfs_gen_grid.argtypes = [C.c_int32, C.c_double, C.c_double, C.c_int32, C.c_uint64, P, P, C.c_int64]
        L.gbfs_gen_grid_capacity.restype = C.c_int64
        L.gbfs_gen_grid_capacity.argtypes = [C.c_int32, C.c_double]
        L.oracle_exclusive_scan_i32.restype = None
        L.oracle_exclusive_scan_i32.argtypes = [P, P, C.c_int64]
        L.oracle_component_edges.restype = C.c_int64
        L.oracle_component_edges.argtypes = [C.c_int32, P, P]
        L.oracle_bfs_min_parents.restype = None
        L.oracle_bfs_min_parents.argtypes = [C.c_int32, P, P, P, P]
        _lib = L
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class CSR:
    """Host CSR built by the oracle (row_offset int64, col_idx int32)."""

    def __init__(self, n: int, row_offset: np.ndarray, col_idx: np.ndarray):
        self.n = n
        self.row_offset = row_offset
        self.col_idx = col_idx

    @property
    def m(self) -> int:
        return int(self.row_offset[-1])

    def degrees(self) -> np.ndarray:
        return np.diff(self.row_offset)


def csr_build(n: int, src, dst, flags: int = 0) -> CSR:
    s = np.ascontiguousarray(src, np.int32)
    d = np.ascontiguousarray(dst, np.int32)
    m = len(s)
    row = np.zeros(n + 1, np.int64)
    cap = 2 * m if flags & SYMMETRIZE else m
    col = np.empty(max(cap, 1), np.int32)
    r = lib().oracle_csr_build(n, m, _p(s), _p(d), flags, _p(row), _p(col))
    if r < 0:
        raise ValueError("edge endpoint outside [0, n)")
    return CSR(n, row, col[:r].copy())


def bfs_levelsync(g: CSR, source: int, with_pred: bool = False):
    level = np.empty(g.n, np.int32)
    pred = np.empty(g.n, np.int32) if with_pred else None
    r = lib().oracle_bfs_levelsync(g.n, _p(g.row_offset), _p(g.col_idx), source, _p(level),
                                   _p(pred) if with_pred else None)
    if r < 0:
        raise ValueError("bad source")
    return (level, pred, int(r)) if with_pred else level


def bfs_queue(g: CSR, source: int) -> np.ndarray:
    level = np.empty(g.n, np.int32)
    if lib().oracle_bfs_queue(g.n, _p(g.row_offset), _p(g.col_idx), source, _p(level)) != 0:
        raise ValueError("bad source")
    return level


def bfs_queue_clock(g: CSR, source: int) -> tuple[np.ndarray, float, int]:
    """Queue BFS timed the reference's way (clock() around it, in ms); also
    the reference's edge count (discovered vertices).  Single-threaded use
    only: clock() counts the whole process's CPU time."""
    level = np.empty(g.n, np.int32)
    ms = C.c_double()
    disc = C.c_int64()
    if lib().oracle_bfs_queue_clock(g.n, _p(g.row_offset), _p(g.col_idx), source, _p(level), C.byref(ms),
                                    C.byref(disc)) != 0:
        raise ValueError("bad source")
    return level, float(ms.value), int(disc.value)


# ---- seeded workload generators (the same code as the engine's, host only) -------------

def _gen_call(fn, cap: int, *args) -> tuple[np.ndarray, np.ndarray]:
    src = np.empty(max(cap, 1), np.int32)
    dst = np.empty(max(cap, 1), np.int32)
    r = fn(*args, _p(src), _p(dst), cap)
    if r < 0:
        raise ValueError(f"{fn.__name__} failed ({r})")
    return src[:r], dst[:r]


def gen_er(n: int, pairs: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    return _gen_call(lib().gbfs_gen_er, pairs, int(n), int(pairs), int(seed))


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    return _gen_call(lib().gbfs_gen_rmat, (1 << scale) * edge_factor, int(scale), int(edge_factor), float(a),
                     float(b), float(c), int(seed))


def gen_grid(side: int, drop: float = 0.1, extra: float = 0.001, radius: int = 8,
             seed: int = 1) -> tuple[np.ndarray, np.ndarray]:
    cap = int(lib().gbfs_gen_grid_capacity(int(side), float(extra)))
    if cap < 0:
        raise ValueError("gbfs_gen_grid_capacity failed")
    return _gen_call(lib().gbfs_gen_grid, cap, int(side), float(drop), float(extra), int(radius), int(seed))


def exclusive_scan(x) -> np.ndarray:
    a = np.ascontiguousarray(x, np.int32)
    out = np.empty(len(a), np.int64)
    lib().oracle_exclusive_scan_i32(_p(a), _p(out), len(a))
    return out


def min_parents(g: CSR, level: np.ndarray) -> np.ndarray:
    lv = np.ascontiguousarray(level, np.int32)
    out = np.empty(g.n, np.int32)
    lib().oracle_bfs_min_parents(g.n, _p(g.row_offset), _p(g.col_idx), _p(lv), _p(out))
    return out


def bfs_levelsync_pred(g: CSR, source: int):
    """Levels and the reference's order-dependent predecessors (C9 restatement)."""
    level = np.empty(g.n, np.int32)
    pred = np.empty(g.n, np.int32)
    if lib().oracle_bfs_levelsync(g.n, _p(g.row_offset), _p(g.col_idx), source, _p(level), _p(pred)) < 0:
        raise ValueError("bad source")
    return level, pred


def component_edges(g: CSR, level: np.ndarray) -> int:
    lv = np.ascontiguousarray(level, np.int32)
    return int(lib().oracle_component_edges(g.n, _p(g.row_offset), _p(lv)))


# ---- the reference's own binaries (this container only) ----------------------------------

def ref_available() -> bool:
    return (REF_DIR / "ref_c9").exists() and (REF_DIR / "ref_c10").exists()


def write_csr_bin(path: str, n: int, row: np.ndarray, col: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(np.int32(n).tobytes())
        f.write(np.int64(len(col)).tobytes())
        f.write(np.ascontiguousarray(row, np.int32).tobytes())
        f.write(np.ascontiguousarray(col, np.int32).tobytes())


def ref_bfs(which: str, source: int, *, text: str | None = None, csr: CSR | None = None,
            reps: int = 1) -> tuple[np.ndarray, dict]:
    """Run the reference's cpuBFS (which = 'c9' or 'c10') from a text file or
    an injected CSR; returns (levels, {"exec_ms", "wall_ms", ...})."""
    exe = REF_DIR / f"ref_{which}"
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "levels.bin")
        if text is not None:
            cmd = [str(exe), "text", text, str(source), out, str(reps)]
        else:
            gpath = os.path.join(td, "g.csr")
            write_csr_bin(gpath, csr.n, csr.row_offset, csr.col_idx)
            cmd = [str(exe), "csr", gpath, str(source), out, str(reps)]
        r = subprocess.run(cmd, capture_output=True, text=True, check=True)
        info = dict(kv.split("=") for kv in r.stdout.split())
        lv = np.fromfile(out, dtype=np.int32)
    return lv, {k: float(v) for k, v in info.items()}
