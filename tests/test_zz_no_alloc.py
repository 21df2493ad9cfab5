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
    # limits: empty input is a no-op, beyond the scratch is refused
    assert lib.gbfs_exclusive_scan_i32_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(got.data_ptr()), 0, None) == 0
    assert lib.gbfs_exclusive_scan_i32_noalloc(C.c_void_p(x.data_ptr()), C.c_void_p(got.data_ptr()), max_n + 1,
                                               None) == gb._lib.ERR_TOO_LARGE
