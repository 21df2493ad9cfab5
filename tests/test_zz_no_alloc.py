"""The allocation-free scan entry point, checked through the C ABI.

gbfs_exclusive_scan_i32_noalloc serves callers that cannot let the library
allocate device memory while they run (pre-reserved HBM pools, loops that
must avoid the driver's allocation locks).  It must give exactly what the
pooled gbfs_exclusive_scan_i32 gives, call after call, although every call
reuses the same built-in scratch array.  This file sorts last so that a run
stopping at the first failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def header_max_n() -> int:
    text = (ROOT / "include" / "gbfs.h").read_text()
    m = re.search(r"#define\s+GBFS_SCAN_NOALLOC_MAX_N\s+\(1LL\s*<<\s*(\d+)\)", text)
    assert m, "GBFS_SCAN_NOALLOC_MAX_N not found in include/gbfs.h"
    return 1 << int(m.group(1))


def bind(gb):
    lib = C.CDLL(gb.library_path())
    for name in ("gbfs_exclusive_scan_i32", "gbfs_exclusive_scan_i32_noalloc"):
        fn = getattr(lib, name)
        fn.restype = C.c_int
        fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    return lib


def test_noalloc_scan_matches_pooled_scan(gb):
    torch = pytest.importorskip("torch")
    lib = bind(gb)
    max_n = header_max_n()
    rng = np.random.default_rng(7)
    # two calls in a row on the shared scratch (large then small), then the
    # largest size the scratch takes
    for n in (3_000_001, 777, max_n):
        x = torch.from_numpy(rng.integers(-5, 1000, size=n, dtype=np.int32)).cuda()
        want = torch.empty(n, dtype=torch.int64, device="cuda")
        got = torch.full((n,), -1, dtype=torch.int64, device="cuda")
        assert lib.gbfs_exclusive_scan_i32(C.c_void_p(x.data_ptr()), C.c_void_p(want.data_ptr()), n, None) == 0
        assert lib.gbfs_exclusive_scan_i32_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(got.data_ptr()), n,
                                                   None) == 0
        assert torch.equal(got, want)
        if n < max_n:  # and against an independent host computation
            xh = x.cpu().numpy().astype(np.int64)
            ref = np.concatenate([[0], np.cumsum(xh)[:-1]])
            assert np.array_equal(got.cpu().numpy(), ref)
    # limits: empty input is a no-op, beyond the scratch is refused
    assert lib.gbfs_exclusive_scan_i32_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(got.data_ptr()), 0, None) == 0
    assert lib.gbfs_exclusive_scan_i32_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(got.data_ptr()), max_n + 1,
                                               None) == gb._lib.ERR_TOO_LARGE


def test_noalloc_scan_on_a_side_stream(gb):
    """Two calls in a row on a non-default stream, against numpy."""
    torch = pytest.importorskip("torch")
    lib = bind(gb)
    side = torch.cuda.Stream()
    rng = np.random.default_rng(11)
    for n in (1_048_577, 4099):
        xh = rng.integers(-1000, 1000, size=n, dtype=np.int32)
        with torch.cuda.stream(side):
            x = torch.from_numpy(xh).cuda(non_blocking=False)
            got = torch.full((n,), -7, dtype=torch.int64, device="cuda")
        side.synchronize()
        assert lib.gbfs_exclusive_scan_i32_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(got.data_ptr()), n,
                                                   C.c_void_p(side.cuda_stream)) == 0
        side.synchronize()
        ref = np.concatenate([[0], np.cumsum(xh.astype(np.int64))[:-1]])
        assert np.array_equal(got.cpu().numpy(), ref)


_FRESH = r"""
import ctypes as C, sys
import numpy as np, torch
sys.path.insert(0, {root!r})
import gpu_graphs_gb300 as gb
lib = C.CDLL(gb.library_path())
fn = lib.gbfs_exclusive_scan_i32_noalloc
fn.restype = C.c_int
fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
n = 5_000_000
x = torch.from_numpy(np.arange(n, dtype=np.int32) % 97).cuda()
out = torch.empty(n, dtype=torch.int64, device="cuda")
torch.cuda.synchronize()
assert fn(C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr()), n, None) == 0  # first call in the process
free0 = torch.cuda.mem_get_info()[0]
for _ in range(3):
    assert fn(C.c_void_p(x.data_ptr()), C.c_void_p(out.data_ptr()), n, None) == 0
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info()[0]
ref = np.concatenate([[0], np.cumsum(np.arange(n, dtype=np.int64) % 97)[:-1]])
assert np.array_equal(out.cpu().numpy(), ref)
print("FREE", free0, free1)
"""


def test_noalloc_scan_allocates_nothing_in_a_fresh_process():
    """First in its process, then three more calls: the device's free memory
    does not move (a cudaMalloc would take at least one 2 MB page)."""
    pytest.importorskip("torch")
    r = subprocess.run([sys.executable, "-c", _FRESH.format(root=str(ROOT))], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("FREE")][-1]
    _, f0, f1 = line.split()
    assert int(f0) == int(f1)
