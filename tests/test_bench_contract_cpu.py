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
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert d["config"]["vertices"] == 1 << 12
