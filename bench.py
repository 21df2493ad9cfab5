#!/usr/bin/env python3
"""Single-source BFS throughput (GTEPS) of the GB300 engine.

Workload (the scale-22 RMAT configuration): RMAT/Kronecker graph, scale 22
(4,194,304 vertices), edge factor 16, a/b/c/d = .57/.19/.19/.05, ids
permuted by the seed, symmetrised, deduplicated, self-loops removed, int32
CSR (128,305,036 directed edges); 64 sources with degree > 0 drawn from a
seeded RNG, run one at a time (one persistent launch each).  A step is the
64 traversals.  GTEPS = undirected edges in the traversed component / s,
summed over the sources (Graph500 convention).

  value       device time (CUDA events on the engine's stream) of K steps,
              level arrays written to HBM, graph resident
  e2e         the same through the C ABI with pinned HOST output buffers:
              every step's 64 level arrays are copied device -> host inside
              the timed region
  roofline    algorithmic bytes per launch (4*E_c + 8*V_c + 4*n) / mean
              launch time, against the measured HBM copy bandwidth
  cpu_baseline the oracle's restatement of the reference's CPU BFS (queue BFS
              of the migration path) on the host cores, one source per thread

--impl reference times that CPU path alone (the reference's own code cannot
be compiled on the GPU host: its sources are not shipped there).
Multi-GPU (--gpus N under torchrun): independent replicas, no collective on
the data path; value sums all ranks' edges over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

RMAT = dict(edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1)
SOURCE_SEED = 1


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gbfs", "reference"], default="gbfs")
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--sources", type=int, default=64)
    ap.add_argument("--cpu-threads", type=int, default=0, help="0 = all host cores")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--autotune", action="store_true", help="autotune parameters before timing")
    ap.add_argument("--params", type=str, default="", help="k=v,... overrides of the traversal parameters")
    ap.add_argument("--layout", choices=["hub-first", "sorted"], default="hub-first",
                    help="CSR row order: sorted ids, or highest-degree neighbour first")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max/sum over ranks (replicas only; nothing on the data path)."""

    def __init__(self, world: int, backend: str):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            td.init_process_group(backend=backend)
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def reduce(self, x: float, op: str) -> float:
        if self.world == 1:
            return x
        import torch
        dev = "cuda" if self.td.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX if op == "max" else self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


def workload(scale: int):
    import gpu_graphs_gb300 as gb
    src, dst = gb.gen_rmat(scale, RMAT["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], RMAT["seed"])
    return 1 << scale, src, dst


def pick_sources(deg: np.ndarray, k: int) -> np.ndarray:
    rng = np.random.default_rng(SOURCE_SEED)
    return rng.choice(np.flatnonzero(deg > 0), k, replace=False).astype(np.int32)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), p[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def cpu_bfs_sample(n: int, row: np.ndarray, col: np.ndarray, sources, threads: int):
    """Oracle queue BFS (the reference's CPU algorithm), one source per thread."""
    import oracle
    g = oracle.CSR(n, row.astype(np.int64), col)
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        levels = list(ex.map(lambda s: oracle.bfs_queue(g, int(s)), sources))
    wall = time.perf_counter() - t0
    edges = sum(oracle.component_edges(g, lv) for lv in levels) / 2
    return wall, edges, levels


def run_reference(args, rank: int, world: int) -> None:
    """--impl reference: the reference's CPU BFS (oracle port) on the host cores."""
    if rank != 0:
        return
    import oracle
    n, src, dst = workload(args.scale)
    g = oracle.csr_build(n, src, dst, oracle.UNDIRECTED)
    deg = g.degrees()
    sources = pick_sources(deg, args.sources)
    threads = args.cpu_threads or (os.cpu_count() or 1)
    per_step = min(threads, len(sources))
    row32 = g.row_offset.astype(np.int32)

    def step(i):
        sel = [sources[(i * per_step + j) % len(sources)] for j in range(per_step)]
        return cpu_bfs_sample(n, row32, g.col_idx, sel, per_step)

    for i in range(args.warmup):
        step(i)
    wall = edges = 0.0
    for i in range(args.steps):
        w, e, _ = step(args.warmup + i)
        wall += w
        edges += e
    gteps = edges / wall / 1e9
    line = {
        "impl": "reference", "metric": "single-source GTEPS", "value": round(gteps, 4), "unit": "GTEPS",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * wall / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": config_block(args, n, int(g.m)),
        "cpu_baseline": {"value": round(gteps, 4), "unit": "GTEPS", "cores": per_step, "kind": "port",
                         "sample": f"{per_step} of the {len(sources)} sources per step, one per thread, "
                                   "oracle restatement of the reference's queue BFS"},
        "e2e": {"value": round(gteps, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_block(args, n: int, m: int) -> dict:
    return {"workload": f"rmat-scale{args.scale}-ef16-64src", "graph": "RMAT a=.57 b=.19 c=.19 d=.05, ids permuted",
            "vertices": n, "directed_edges": m, "sources_per_step": args.sources,
            "l2": "inputs larger than L2 (CSR ~0.5 GB vs 129 MB L2)"}


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    torch.cuda.set_device(local)
    dist = Dist(world, "nccl")
    import gpu_graphs_gb300 as gb

    n, src, dst = workload(args.scale)
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | (gb.HUB_FIRST if args.layout == "hub-first" else 0))
    del src, dst
    row, col = g.csr()
    deg = np.diff(row)
    sources = pick_sources(deg, args.sources)
    if args.params:
        g.set_params(**{k: int(v) for k, v in (kv.split("=") for kv in args.params.split(","))})
    if args.autotune:
        g.autotune(sources[:4])
    params = g.params.as_dict()

    k = len(sources)
    out = torch.empty((k, n), dtype=torch.int32, device="cuda")
    stream = torch.cuda.ExternalStream(g.stream)

    # parity spot check against the oracle (outside the timed region)
    import oracle
    og = oracle.CSR(n, row.astype(np.int64), col)
    g.bfs_many(sources[:2], out=out[:2])
    parity = all(np.array_equal(out[i].cpu().numpy(), oracle.bfs_queue(og, int(s))) for i, s in enumerate(sources[:2]))

    for _ in range(args.warmup):
        g.bfs_many(sources, out=out)
    torch.cuda.synchronize()
    dist.barrier()
    launch_ms, launch_ec, edges_c, verts, lvls = [], [], 0, 0, []
    with ClockSampler(local) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            _, sts = g.bfs_many(sources, out=out)
            launch_ms += [s.ms for s in sts]
            launch_ec += [s.edges_in_component for s in sts]
            edges_c += sum(s.edges_in_component for s in sts)
            verts += sum(s.vertices_reached for s in sts)
            lvls += [(s.levels, s.td_levels, s.bu_levels) for s in sts]
        ev1.record(stream)
        torch.cuda.synchronize()
    dist.barrier()
    ms = ev0.elapsed_time(ev1)
    ms_max = dist.reduce(ms, "max")
    und_edges = edges_c / 2
    total_edges = dist.reduce(und_edges, "sum")
    value = total_edges / (ms_max / 1e3) / 1e9

    # roofline of the persistent kernel: algorithmic bytes / mean launch time
    launches = args.steps * k
    b_alg = 4 * edges_c + 8 * verts + 4 * n * launches
    peak, peak_kind = measured_peak()
    achieved = (b_alg / launches) / (np.mean(launch_ms) / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                "bytes_per_launch": int(b_alg / launches), "mean_launch_us": round(1e3 * float(np.mean(launch_ms)), 2),
                "traffic": None}
    gteps_each = [(e / 2) / (t / 1e3) / 1e9 for e, t in zip(launch_ec, launch_ms)]

    # e2e through the C ABI with pinned host output buffers
    e2e = None
    if not args.no_e2e:
        host = torch.empty((k, n), dtype=torch.int32, pin_memory=True)
        hv = host.numpy()
        g.bfs_many(sources, out=hv)
        torch.cuda.synchronize()
        dist.barrier()
        steps_e2e = max(1, min(args.steps, 3))
        t0 = time.perf_counter()
        for _ in range(steps_e2e):
            g.bfs_many(sources, out=hv)
        t1 = time.perf_counter()
        dist.barrier()
        wall = dist.reduce(t1 - t0, "max")
        e2e = {"value": round(dist.reduce(und_edges / args.steps * steps_e2e, "sum") / wall / 1e9, 3),
               "unit": "GTEPS", "h2d_bytes_per_step": 4 * k, "d2h_bytes_per_step": 4 * k * n,
               "steps": steps_e2e}
        del host, hv

    cpu = None
    if not args.no_cpu and rank == 0:
        threads = args.cpu_threads or (os.cpu_count() or 1)
        sel = sources[: min(threads, k)]
        wall, e, lv = cpu_bfs_sample(n, row, col, sel, len(sel))
        cpu = {"value": round(e / wall / 1e9, 4), "unit": "GTEPS", "cores": len(sel), "kind": "port",
               "sample": f"{len(sel)} of the {k} sources, one per thread, oracle restatement of the "
                         f"reference's queue BFS ({wall:.2f} s)"}

    if rank == 0:
        line = {
            "metric": "single-source GTEPS", "value": round(value, 3), "unit": "GTEPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic", "config": config_block(args, n, g.m) | {"parallelism": f"replicas{world}",
                                                                            "layout": args.layout, "params": params},
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clk.summary(), "parity_spot_check": parity,
            "per_source_gteps": {"min": round(min(gteps_each), 2), "median": round(statistics.median(gteps_each), 2),
                                 "max": round(max(gteps_each), 2)},
            "levels_td_bu": sorted(set(lvls))[:8],
        }
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
