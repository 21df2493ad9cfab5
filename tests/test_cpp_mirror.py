"""The C++ mirror of the reference's csr / gpuBFS classes (include/gbfs_graphbfs.hpp)."""
from __future__ import annotations

import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden


def build_driver(tmp_path, gb) -> str:
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "graphbfs"
    libdir = str(ROOT / "gpu_graphs_gb300")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "graphbfs_main.cpp"),
                    "-L", libdir, "-lgbfs", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return str(exe)


def write_fixture(tmp_path, name):
    d = load_golden(name)
    p = tmp_path / f"{name}.txt"
    p.write_text("\n".join([str(int(d["n"])), str(len(d["src"]))] + [f"{a + 1} {b + 1}" for a, b in zip(d["src"], d["dst"])]))
    return p, d


def test_header_compiles_and_reports_errors(gb, tmp_path):
    exe = build_driver(tmp_path, gb)
    r = subprocess.run([exe, str(tmp_path / "missing.txt"), "0"], capture_output=True, text=True)
    assert r.returncode == 2
    assert "Error: Unable to open file" in r.stderr
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stderr


@pytest.mark.gpu
def test_driver_matches_reference_levels(gb, tmp_path):
    exe = build_driver(tmp_path, gb)
    for name in ("ref_test4", "ref_tree", "ref_test2"):
        p, d = write_fixture(tmp_path, name)
        for s, want in zip(d["sources"][:3], d["levels"][:3]):
            r = subprocess.run([exe, str(p), str(int(s))], capture_output=True, text=True, check=True)
            lines = r.stdout.splitlines()
            assert lines[0].startswith("GPU BFS Time:")
            got = np.array([int(x) for x in lines[1:]], np.int32)
            assert np.array_equal(got, want)
