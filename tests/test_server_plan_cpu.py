"""CPU: the serving loop's scheduling rule under simulated load.

tests/cpp/srv_plan_sim.cpp includes gpu_graphs_gb300/csrc/server_plan.h (the
rule server.cu runs) and drives it with simulated launches and Poisson or
closed-loop arrivals over single-source and batch graphs, 1-6 slots, fixed
and launch-time-scaled batch windows, slots whose workspaces hold only some
graphs, and a shutdown part-way: no unit double-booked, no slot over its CTA
share or taking a graph larger than its workspace, batches only on whole
slots, per-graph FIFO, no query left waiting beside a slot that could take
it, and every query served.
"""
from __future__ import annotations

import shutil
import subprocess

import pytest

from conftest import ROOT


def test_scheduling_rule_simulation(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "srv_plan_sim"
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", str(ROOT / "gpu_graphs_gb300" / "csrc"),
                    str(ROOT / "tests" / "cpp" / "srv_plan_sim.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok "), r.stdout
    stats = dict(kv.split("=") for kv in r.stdout.split()[1:])
    # every kind of decision was exercised
    for k in ("batches", "whole", "unit", "drains"):
        assert int(stats[k]) > 0, (k, r.stdout)
