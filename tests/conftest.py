"""Shared test setup: repo root on sys.path, the `gpu` marker, golden data."""
from __future__ import annotations

import os
import sys
from pathlib import Path

# the server's concurrent searches need more than CUDA's default 8 hardware
# work queues; set before any test makes the first CUDA call
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def load_golden(name: str) -> dict:
    z = np.load(GOLDEN / f"{name}.npz", allow_pickle=False)
    return {k: z[k] for k in z.files}


def golden_names(prefix: str = "") -> list[str]:
    return sorted(p.stem for p in GOLDEN.glob(f"{prefix}*.npz"))


def synthetic_edges(d: dict):
    """Regenerate a synthetic golden graph's edges with the library generators."""
    import ast
    import gpu_graphs_gb300 as gb
    kind = str(d["kind"])
    args = ast.literal_eval(str(d["args"]))
    if kind == "er":
        src, dst = gb.gen_er(args["n"], args["pairs"], args["seed"])
    elif kind == "rmat":
        src, dst = gb.gen_rmat(args["scale"], args["edge_factor"], seed=args["seed"])
    else:
        src, dst = gb.gen_grid(args["side"], args["drop"], args["extra"], args["radius"], args["seed"])
    return int(d["n"]), src, dst


@pytest.fixture(scope="session")
def gb():
    import gpu_graphs_gb300
    return gpu_graphs_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle
