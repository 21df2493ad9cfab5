"""bench.py's reference arm (the reference's CPU BFS on the host cores) keeps
the JSON-line contract: one line, the same metric and unit as the GPU arm,
a cpu_baseline describing the run and an e2e object with no transfers."""
from __future__ import annotations

import json
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--scale", "12",
                        "--steps", "2", "--warmup", "1", "--cpu-threads", "2"],
                       capture_output=True, text=True, timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "single-source GTEPS" and d["unit"] == "GTEPS"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] == 2 and cb["value"] == d["value"]
    assert cb["sample"] and cb["host"]
    st = cb["single_thread"]
    assert st["cores"] == 1 and st["value"] > 0 and st["exec_time_ms_per_source"] >= 0
    assert st["reference_teps_convention"].startswith("discovered vertices")
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert d["config"]["vertices"] == 1 << 12
    # the config names the workload only (engine settings live elsewhere on the GPU arm)
    assert set(d["config"]) == {"workload", "graph", "vertices", "directed_edges", "sources_per_step", "l2"}


def test_reference_arm_loads_only_the_oracle():
    """The CPU reference arm builds its graph with the oracle's copy of the
    generators and never maps the engine library."""
    code = ("import sys, io, contextlib; sys.path.insert(0, %r); import bench; "
            "sys.argv = ['bench.py', '--impl', 'reference', '--scale', '10', '--steps', '1', '--warmup', '1', "
            "'--cpu-threads', '1', '--sources', '2']; "
            "f = io.StringIO(); contextlib.redirect_stdout(f).__enter__(); bench.main(); "
            "m = open('/proc/self/maps').read(); sys.stderr.write('MAPS ' + str('libgbfs' in m) + ' ' + "
            "str('liboracle' in m) + ' ' + str('gpu_graphs_gb300' in sys.modules))") % str(ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    assert "MAPS False True False" in r.stderr
