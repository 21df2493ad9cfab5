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
              of the migration path) on the host cores, one source per
              thread; with a single-thread figure timed as the reference
              times itself (clock() around the search) and its own TEPS
              convention (discovered vertices / s)

Extra objects on the same line (rank 0, skipped with --no-extra): config1
(the reference's CPU-runnable ER case on GPU and CPU, levels checked against
the reference binaries' stored output), e2e_from_edge_list (host edge list
-> CSR build -> 64 searches -> host levels), grid (7000 x 7000, persistent
vs one launch per level), batched (64-lane multi-source on RMAT-20; 512
small graphs in one launch), primitives (CSR build, exclusive scan),
graph500 (RMAT scales 26 and 27 at edge factor 16, the latter with 64-bit
row offsets; --no-large skips them) and serving (32 resident graphs,
Poisson arrivals; --no-serving skips it).  The
batched and serving objects carry a cpu_parallel throughput: the same
queries through the oracle's queue BFS, one query per host core at a time.

--impl reference times that CPU path alone, on the same graph, sources and
config, loading only the oracle library (whose copy of the seeded
generators builds the graph).  The reference's own compiled CPU code is not
used there: its sources are not available on the GPU host.
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
# The server runs its slots' searches on up to 24 streams at once; CUDA's
# default of 8 hardware work queues per process lets only about four of
# them progress together (set before the first CUDA call of the process).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

RMAT = dict(edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1)
SOURCE_SEED = 1


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
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
    ap.add_argument("--no-extra", action="store_true", help="skip the grid and batched measurements")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving sweep (32 resident graphs)")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the RMAT scale-26 and scale-27 graphs (the latter with 64-bit row offsets)")
    ap.add_argument("--grid-side", type=int, default=7000)
    ap.add_argument("--grid-only", action="store_true",
                    help="only --steps persistent searches on the --grid-side grid (a profiling workload)")
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


def workload(scale: int, gen=None):
    """The RMAT edge list.  gen: a module with gen_rmat (the engine package on
    the GPU arm; the oracle, which links the same generator code, on the CPU
    reference arm so that arm never loads the engine)."""
    if gen is None:
        import gpu_graphs_gb300 as gen
    src, dst = gen.gen_rmat(scale, RMAT["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], RMAT["seed"])
    return 1 << scale, src, dst


def pick_sources(deg: np.ndarray, k: int) -> np.ndarray:
    rng = np.random.default_rng(SOURCE_SEED)
    return rng.choice(np.flatnonzero(deg > 0), k, replace=False).astype(np.int32)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms in the background.

    Started before the warm-up (nvidia-smi takes a moment to start); each
    sample is stamped on arrival and summary() keeps those inside the window
    set by mark_start() / mark_end() around the timed steps."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[tuple[float, str]] = []
        self.t0 = None
        self.t1 = None

    def mark_start(self):
        self.t0 = time.perf_counter()

    def mark_end(self):
        self.t1 = time.perf_counter()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

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
        # a sample printed within 100 ms after the window still describes it
        lo = self.t0 if self.t0 is not None else float("-inf")
        hi = self.t1 + 0.1 if self.t1 is not None else float("inf")
        for t, ln in self.lines:
            if not lo <= t <= hi:
                continue
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


def log(msg: str) -> None:
    print(f"[bench] {msg}", file=sys.stderr, flush=True)


KERNEL_SOURCES = ("bfs.cu", "bfs.cuh", "bfs_args.cuh", "common.cuh", "blockq.cuh")


def kernel_source_hash() -> str:
    """sha256 (16 hex digits) of the single-source kernel's source files."""
    import hashlib
    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        h.update((ROOT / "gpu_graphs_gb300" / "csrc" / name).read_bytes())
    return h.hexdigest()[:16]


def profiled_traffic() -> tuple[int | None, str]:
    """DRAM bytes per k_bfs launch from the committed ncu summary, only when
    the summary was taken of the kernel source being built (its stamped
    source hash equals kernel_source_hash()); else (None, why)."""
    p = ROOT / "profiles" / "k_bfs_rmat22.md"
    if not p.exists():
        return None, "no profile"
    traffic, stamp = None, None
    for ln in p.read_text().splitlines():
        if ln.startswith("traffic_bytes_per_launch ="):
            traffic = int(ln.split("=")[1])
        if ln.startswith("kernel_source_sha256_16 ="):
            stamp = ln.split("=")[1].strip()
    if traffic is None:
        return None, "profile has no traffic line"
    if stamp != kernel_source_hash():
        return None, f"profile taken of other kernel sources ({stamp} != {kernel_source_hash()})"
    return traffic, f"ncu dram__bytes_read+write per launch, profiles/k_bfs_rmat22.md (sources {stamp})"


def measured_peak() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def cpu_bfs_sample(g, sources, threads: int):
    """Oracle queue BFS (the reference's CPU algorithm), one source per thread.
    g: an oracle CSR.  Returns (wall s, undirected component edges, levels)."""
    import oracle
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        levels = list(ex.map(lambda s: oracle.bfs_queue(g, int(s)), sources))
    wall = time.perf_counter() - t0
    edges = sum(oracle.component_edges(g, lv) for lv in levels) / 2
    return wall, edges, levels


def cpu_single_thread(g, sources) -> dict:
    """The reference's CPU BFS the way its driver runs it: one thread, one
    source at a time, clock() around each search (migration cpuBFS.cpp:5-6,
    51-53), plus wall time; GTEPS in the Graph500 convention and TEPS in the
    reference's own (discovered vertices per second of exec_time,
    2D Partition/src/gpuBFS.cu:514-515, counted as cpuBFS.cpp:59 does)."""
    import oracle
    wall = exec_ms = edges = disc = 0.0
    for s0 in sources:
        t0 = time.perf_counter()
        lv, ms, d = oracle.bfs_queue_clock(g, int(s0))
        wall += time.perf_counter() - t0
        exec_ms += ms
        disc += d
        edges += oracle.component_edges(g, lv) / 2
    return {"value": round(edges / wall / 1e9, 4), "unit": "GTEPS", "cores": 1, "sources": len(sources),
            "wall_ms_per_source": round(1e3 * wall / len(sources), 2),
            "exec_time_ms_per_source": round(exec_ms / len(sources), 2),
            "reference_teps": round(disc / (exec_ms / 1e3), 1) if exec_ms > 0 else None,
            "reference_teps_convention": "discovered vertices / exec_time (clock())"}


def host_cpu() -> str:
    """The host CPU's model name and logical core count (reported beside every
    CPU figure)."""
    name = ""
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                key = ln.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware") and not name:
                    name = ln.split(":", 1)[1].strip()
                if key == "cpu part" and not name:  # Arm cores list a part number only
                    name = "Arm part " + ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return f"{name or 'unknown'}, {os.cpu_count()} logical cores"


def cpu_parallel_queries(tasks, threads: int = 0) -> dict:
    """Embarrassingly parallel CPU throughput: the oracle's queue BFS (the
    reference's CPU algorithm), one query per host core at a time.  `tasks`
    is a list of (oracle CSR, source); returns queries/s and the levels."""
    import oracle
    threads = threads or (os.cpu_count() or 1)
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        levels = list(ex.map(lambda t: oracle.bfs_queue(t[0], int(t[1])), tasks))
    wall = time.perf_counter() - t0
    return {"queries_per_s": round(len(tasks) / wall, 1), "cores": threads, "queries": len(tasks),
            "seconds": round(wall, 3), "host": host_cpu()}, levels


def run_reference(args, rank: int, world: int) -> None:
    """--impl reference: the reference's CPU BFS (the oracle's restatement of
    its queue BFS) on the host cores, on the same graph, sources, metric and
    config as the GPU arm.  Loads only the oracle library: the graph comes
    from the oracle's copy of the seeded generators and its CSR build."""
    if rank != 0:
        return
    import oracle
    n, src, dst = workload(args.scale, oracle)
    g = oracle.csr_build(n, src, dst, oracle.UNDIRECTED)
    del src, dst
    sources = pick_sources(g.degrees(), args.sources)
    threads = args.cpu_threads or (os.cpu_count() or 1)
    per_step = min(threads, len(sources))

    def step(i):
        sel = [sources[(i * per_step + j) % len(sources)] for j in range(per_step)]
        return cpu_bfs_sample(g, sel, per_step)

    for i in range(args.warmup):
        step(i)
    wall = edges = 0.0
    for i in range(args.steps):
        w, e, _ = step(args.warmup + i)
        wall += w
        edges += e
    gteps = edges / wall / 1e9
    single = cpu_single_thread(g, sources[:2])
    line = {
        "impl": "reference", "metric": "single-source GTEPS", "value": round(gteps, 4), "unit": "GTEPS",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * wall / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": config_block(args, n, int(g.m)),
        "cpu_baseline": {"value": round(gteps, 4), "unit": "GTEPS", "cores": per_step, "kind": "port",
                         "host": host_cpu(),
                         "sample": f"{per_step} of the {len(sources)} sources per step, one per thread, "
                                   "oracle restatement of the reference's queue BFS",
                         "single_thread": single},
        "e2e": {"value": round(gteps, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_block(args, n: int, m: int) -> dict:
    """The workload, identical on both arms (engine settings go elsewhere)."""
    return {"workload": f"rmat-scale{args.scale}-ef16-{args.sources}src",
            "graph": "RMAT a=.57 b=.19 c=.19 d=.05, ids permuted, symmetrised, deduplicated, no self-loops",
            "vertices": n, "directed_edges": m, "sources_per_step": args.sources,
            "l2": "inputs larger than L2 (CSR ~0.5 GB vs 129 MB L2)"}


# ---- the other configurations (extra objects on the same line) --------------------

def measure_config1(torch) -> dict:
    """The reference's own CPU-runnable case: Erdos-Renyi n = 65,536 with
    262,144 distinct undirected pairs (seed 1), symmetrised, source 0, plain
    top-down BFS.  GPU: device time of one launch and the same through the
    C ABI into a host buffer; CPU: the reference's queue BFS (oracle
    restatement) on one thread, timed by clock() as the reference does.
    Levels are checked against the reference binaries' own output for this
    graph (tests/golden/syn_er16.npz) and against the oracle."""
    import gpu_graphs_gb300 as gb
    import oracle
    n = 65536
    src, dst = gb.gen_er(n, 262144, 1)
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED)
    og = oracle.csr_build(n, src, dst, oracle.UNDIRECTED)
    dev = torch.empty(n, dtype=torch.int32, device="cuda")
    res = {"workload": "ER n=65536, 262144 undirected pairs (seed 1), symmetrised, source 0",
           "vertices": n, "directed_edges": int(g.m)}
    for name, direction in (("topdown", gb.DIR_TOPDOWN), ("direction_optimising", gb.DIR_OPTIMIZING)):
        g.set_params(direction=direction)
        for _ in range(5):
            g.bfs(0, out=dev)
        runs = [g.bfs(0, out=dev, stats=True)[1] for _ in range(50)]
        ms = float(np.median([r.ms for r in runs]))
        st = runs[-1]
        host = np.empty(n, np.int32)
        t0 = time.perf_counter()
        for _ in range(50):
            g.bfs(0, out=host)
        e2e_ms = (time.perf_counter() - t0) * 1e3 / 50
        res[name] = {"gpu_ms": round(ms, 4), "gteps": round(st.edges_in_component / 2 / (ms / 1e3) / 1e9, 3),
                     "reference_teps": round(st.edges_traversed / (ms / 1e3), 1),
                     "e2e_ms_host_output": round(e2e_ms, 4), "levels": int(st.levels),
                     "levels_identical_oracle": bool(np.array_equal(host, oracle.bfs_queue(og, 0)))}
    g.set_params(direction=gb.DIR_OPTIMIZING)
    lv, exec_ms, disc = oracle.bfs_queue_clock(og, 0)
    walls = []
    for _ in range(5):
        t0 = time.perf_counter()
        oracle.bfs_queue(og, 0)
        walls.append(time.perf_counter() - t0)
    wall_ms = 1e3 * float(np.median(walls))
    ec = oracle.component_edges(og, lv) / 2
    res["cpu"] = {"kind": "port", "cores": 1, "host": host_cpu(), "exec_time_ms": round(exec_ms, 3),
                  "wall_ms": round(wall_ms, 3), "gteps": round(ec / (wall_ms / 1e3) / 1e9, 4),
                  "reference_teps": round(disc / (exec_ms / 1e3), 1) if exec_ms > 0 else None,
                  "timing": "clock() around the queue BFS (migration cpuBFS.cpp:5-6,51-53); wall = median of 5"}
    golden = ROOT / "tests" / "golden" / "syn_er16.npz"
    if golden.exists():
        z = np.load(golden)
        res["levels_identical_reference_binaries"] = bool(int(z["sources"][0]) == 0 and
                                                          np.array_equal(z["levels"][0], host))
    res["speedup_gpu_vs_cpu_wall"] = round(wall_ms / res["topdown"]["gpu_ms"], 1)
    return res


def measure_e2e_from_edge_list(scale: int, sources, torch) -> dict:
    """The whole graphBFS path through the public API: host edge list in,
    CSR built on the GPU (symmetrised, deduplicated, hub-first rows), the 64
    searches, every level array copied back into pinned host memory."""
    import gpu_graphs_gb300 as gb
    n, src, dst = workload(scale)
    host = torch.empty((len(sources), n), dtype=torch.int32, pin_memory=True).numpy()
    times = []
    for i in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | gb.HUB_FIRST)
        t1 = time.perf_counter()
        _, sts = g.bfs_many(sources, out=host)
        t2 = time.perf_counter()
        times.append((t2 - t0, t1 - t0, t2 - t1))
        edges = sum(s.edges_in_component for s in sts) / 2
        del g
    tot, build, bfs = min(times)
    return {"workload": f"RMAT scale {scale}: {len(src)} host edges in, {len(sources)} level arrays out",
            "h2d_bytes": 8 * len(src), "d2h_bytes": 4 * n * len(sources),
            "total_ms": round(tot * 1e3, 2), "csr_build_ms": round(build * 1e3, 2),
            "searches_ms": round(bfs * 1e3, 2), "gteps_incl_build": round(edges / tot / 1e9, 2)}


def measure_grid(side: int, torch) -> dict:
    """High-diameter grid: one persistent launch vs one launch per level (host
    loop, the reference's shape) vs the same launches replayed by a CUDA graph."""
    import gpu_graphs_gb300 as gb
    src, dst = gb.gen_grid(side, 0.1, 0.001, 8, seed=1)
    n = side * side
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED)
    del src, dst
    row, col = g.csr()
    deg = np.diff(row)
    source = int(pick_sources(deg, 1)[0])
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    g.bfs(source, out=out)
    ref = out.clone()
    # the clone runs on torch's stream: finish it before the engine's stream
    # writes `out` again
    torch.cuda.synchronize()
    import oracle
    o = oracle.CSR(n, row.astype(np.int64), col)
    same_oracle = bool(np.array_equal(ref.cpu().numpy(), oracle.bfs_queue(o, source)))
    del o
    runs = [g.bfs(source, out=out, stats=True)[1] for _ in range(3)]
    st = runs[-1]
    t_p = float(np.mean([r.ms for r in runs]))
    g.set_params(per_level_launch=1)
    runs_l = [g.bfs(source, out=out, stats=True)[1] for _ in range(2)]
    same = bool(torch.equal(out, ref))
    t_l = float(np.mean([r.ms for r in runs_l]))
    # the same launches per level, replayed by a CUDA graph (device-side loop)
    g.set_params(per_level_launch=2)
    g.bfs(source, out=out)
    runs_g = [g.bfs(source, out=out, stats=True)[1] for _ in range(2)]
    same = same and bool(torch.equal(out, ref))
    t_g = float(np.mean([r.ms for r in runs_g]))
    g.set_params(per_level_launch=0)
    return {"workload": f"grid {side}x{side}, 10% edges dropped, 0.1% extra edges within radius 8",
            "vertices": n, "directed_edges": int(g.m), "source": source, "levels": int(st.levels),
            "persistent_ms": round(t_p, 3), "per_level_launch_ms": round(t_l, 3),
            "per_level_graph_ms": round(t_g, 3),
            "per_level_launches": int(runs_l[-1].launches), "speedup_vs_per_level": round(t_l / t_p, 2),
            "gteps_persistent": round(st.edges_in_component / 2 / (t_p / 1e3) / 1e9, 3),
            "us_per_level_persistent": round(1e3 * t_p / max(1, st.levels), 3),
            "levels_identical": same, "levels_identical_oracle": same_oracle}


def grid_only(side: int, reps: int) -> dict:
    """`reps` persistent searches from the grid measurement's source (the
    grid kernel's first levels, then the label-correcting kernel)."""
    import gpu_graphs_gb300 as gb
    import torch
    src, dst = gb.gen_grid(side, 0.1, 0.001, 8, seed=1)
    n = side * side
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED)
    del src, dst
    row, _ = g.csr()
    source = int(pick_sources(np.diff(row), 1)[0])
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    runs = [g.bfs(source, out=out, stats=True)[1] for _ in range(max(1, reps))]
    st = runs[-1]
    ms = float(np.mean([r.ms for r in runs]))
    return {"workload": f"grid {side}x{side}, 10% edges dropped, 0.1% extra edges within radius 8",
            "vertices": n, "source": source, "levels": int(st.levels), "launches_per_search": int(st.launches),
            "searches": len(runs), "ms": round(ms, 3), "us_per_level": round(1e3 * ms / max(1, st.levels), 3)}


def measure_rmat_large(torch, scale: int, edge_factor: int = 16, nsrc: int = 8) -> dict:
    """A Graph500-size RMAT graph (the bench's a/b/c and seed): build time
    from the host edge list and device-timed searches from nsrc sources, one
    launch each.  From scale 27 on (edge factor 16) the stored edges pass
    2^31-1 and the CSR gets 64-bit row offsets; bit-exact parity at these
    sizes is in tests/test_wide_gpu.py and tests/test_fullsize_gpu.py."""
    import gpu_graphs_gb300 as gb
    src, dst = gb.gen_rmat(scale, edge_factor, RMAT["a"], RMAT["b"], RMAT["c"], RMAT["seed"])
    n = 1 << scale
    pairs = len(src)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | gb.HUB_FIRST)
    build_s = time.perf_counter() - t0
    del src, dst
    sources = pick_sources(np.diff(g.row_offsets()), nsrc)
    out = torch.empty((nsrc, n), dtype=torch.int32, device="cuda")
    g.bfs_many(sources, out=out)
    _, sts = g.bfs_many(sources, out=out)
    ms = float(sum(x.ms for x in sts))
    ec = sum(x.edges_in_component for x in sts)
    res = {"workload": f"RMAT scale {scale}, edge factor {edge_factor} ({pairs} pairs), undirected, hub-first rows",
           "vertices": n, "directed_edges": int(g.m), "row_offset_bits": 64 if g.wide else 32,
           "build_s_from_host_edges": round(build_s, 3), "sources": nsrc, "search_ms_mean": round(ms / nsrc, 3),
           "gteps": round(ec / 2 / (ms / 1e3) / 1e9, 2),
           "levels": [int(x.levels) for x in sts]}
    del out, g
    torch.cuda.empty_cache()
    return res


def many_graphs_workload(gen, count: int = 512):
    """The fused-launch configuration: `count` Erdos-Renyi graphs, n
    log-uniform in [2^8, 2^16], 4n sampled pairs each (average degree 8 once
    symmetrised), one source each drawn among its vertices of degree > 0.
    gen: a module with gen_er.  Returns ([(n, src, dst)], sources)."""
    rng = np.random.default_rng(1)
    sizes = np.exp(rng.uniform(np.log(256), np.log(65536), count)).astype(np.int64)
    graphs, srcs = [], []
    for i, ni in enumerate(sizes):
        s_, d_ = gen.gen_er(int(ni), int(4 * ni), 1000 + i)
        deg = np.bincount(np.concatenate([s_, d_]), minlength=int(ni)) - 2 * np.bincount(s_[s_ == d_], minlength=int(ni))
        graphs.append((int(ni), s_, d_))
        srcs.append(int(rng.choice(np.flatnonzero(deg > 0))))
    return graphs, srcs


def measure_batched(torch) -> dict:
    """64 sources per launch on RMAT scale 20, and 512 small ER graphs in one launch,
    each against the plain one-query-per-launch BFS on the same GPU."""
    import gpu_graphs_gb300 as gb
    res = {}
    n20 = 1 << 20
    src, dst = gb.gen_rmat(20, 16, 0.57, 0.19, 0.19, seed=1)
    g = gb.Graph.from_edges(n20, src, dst, gb.UNDIRECTED | gb.HUB_FIRST)
    del src, dst
    row, col = g.csr()
    sources = pick_sources(np.diff(row), 64)
    plain_out = torch.empty((64, n20), dtype=torch.int32, device="cuda")
    multi_out = torch.empty((64, n20), dtype=torch.int32, device="cuda")
    g.bfs_many(sources, out=plain_out)
    g.bfs_multi(sources, out=multi_out)
    t_plain = min(sum(s.ms for s in g.bfs_many(sources, out=plain_out)[1]) for _ in range(3))
    t_multi = min(g.bfs_multi(sources, out=multi_out, stats=True)[1].ms for _ in range(3))
    same = bool(torch.equal(plain_out, multi_out))
    # the plain top-down BFS (one query per launch, no bottom-up steps)
    g.set_params(direction=1)
    t_plain_td = min(sum(s.ms for s in g.bfs_many(sources, out=plain_out)[1]) for _ in range(2))
    same = same and bool(torch.equal(plain_out, multi_out))
    g.set_params(direction=0)
    res["multi_source"] = {
        "workload": "RMAT scale 20, ef 16, 64 sources per launch (uint64 lane masks)",
        "plain_ms": round(t_plain, 3), "plain": "direction-optimising single-source kernel, one launch per source",
        "plain_topdown_ms": round(t_plain_td, 3), "batched_ms": round(t_multi, 3),
        "plain_queries_per_s": round(64 / (t_plain / 1e3), 1), "batched_queries_per_s": round(64 / (t_multi / 1e3), 1),
        "speedup": round(t_plain / t_multi, 2), "speedup_vs_topdown": round(t_plain_td / t_multi, 2),
        "levels_identical": same}
    # the same 64 queries on the host cores, one per core at a time
    import oracle
    og = oracle.CSR(n20, row.astype(np.int64), col)
    cpu, lv = cpu_parallel_queries([(og, s0) for s0 in sources])
    mo = multi_out.cpu().numpy()
    cpu["levels_identical"] = all(np.array_equal(a, b) for a, b in zip(lv, mo))
    cpu["kind"] = "port"
    res["multi_source"]["cpu_parallel"] = cpu
    res["multi_source"]["speedup_vs_cpu_parallel"] = round(res["multi_source"]["batched_queries_per_s"] /
                                                           cpu["queries_per_s"], 1)
    del plain_out, multi_out, g, og, row, col, mo, lv

    graphs, srcs = many_graphs_workload(gb)
    sizes = np.array([g[0] for g in graphs], np.int64)
    gs = gb.GraphSet.from_edges(graphs)
    fused, st = gs.bfs(srcs, stats=True)
    t_fused = min(gs.bfs(srcs, stats=True)[1].ms for _ in range(3))
    handles = [gb.Graph.from_edges(ni, s_, d_) for ni, s_, d_ in graphs]
    douts = [torch.empty(h.n, dtype=torch.int32, device="cuda") for h in handles]
    for h, o, s0 in zip(handles, douts, srcs):
        h.bfs(s0, out=o)
    t_plain = min(sum(h.bfs(s0, out=o, stats=True)[1].ms for h, o, s0 in zip(handles, douts, srcs)) for _ in range(2))
    same = all(np.array_equal(f, o.cpu().numpy()) for f, o in zip(fused, douts))
    ocsr = []
    for h in handles:
        r_, c_ = h.csr()
        ocsr.append(oracle.CSR(h.n, r_.astype(np.int64), c_))
    cpu, lv = cpu_parallel_queries(list(zip(ocsr, srcs)))
    cpu["levels_identical"] = all(np.array_equal(a, b) for a, b in zip(lv, fused))
    cpu["kind"] = "port"
    res["many_graphs"] = {
        "workload": f"512 ER graphs, n log-uniform in [256, 65536] (total {int(sizes.sum())} vertices), avg degree 8, "
                    "one source each, one fused launch",
        "plain_ms": round(t_plain, 3), "fused_ms": round(t_fused, 3),
        "plain_queries_per_s": round(512 / (t_plain / 1e3), 1), "fused_queries_per_s": round(512 / (t_fused / 1e3), 1),
        "speedup": round(t_plain / t_fused, 2), "levels_identical": bool(same),
        "cpu_parallel": cpu, "speedup_vs_cpu_parallel": round(512 / (t_fused / 1e3) / cpu["queries_per_s"], 1)}
    return res


def measure_primitives(torch) -> dict:
    """The path's other kernels: the CSR build (edge list in, CSR out) against the
    oracle's CPU restatement of the reference loader on the same edges, and the
    exclusive scan against the HBM peak."""
    import gpu_graphs_gb300 as gb
    import oracle
    res = {}
    n20 = 1 << 20
    src, dst = gb.gen_rmat(20, 16, 0.57, 0.19, 0.19, seed=1)
    gb.Graph.from_edges(n20, src, dst, gb.UNDIRECTED)  # warm-up
    ts = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g = gb.Graph.from_edges(n20, src, dst, gb.UNDIRECTED)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
        m = g.m
        del g
    t0 = time.perf_counter()
    og = oracle.csr_build(n20, src, dst, oracle.UNDIRECTED)
    t_cpu = time.perf_counter() - t0
    res["csr_build"] = {
        "workload": f"RMAT scale 20, {len(src)} input edges -> symmetrised, deduped, sorted CSR ({m} directed edges)",
        "gpu_ms_host_arrays_in": round(min(ts) * 1e3, 2),
        "gpu_input_edges_per_s": round(len(src) / min(ts), 1),
        "cpu_ms": round(t_cpu * 1e3, 1), "cpu": "oracle restatement of the reference loader (csc.cpp), 1 thread",
        "identical_edge_count": bool(og.m == m)}
    del og
    nscan = 1 << 28  # 3.2 GB moved per call: the per-call status read-back is a few % of it
    x = torch.randint(-1000, 100000, (nscan,), dtype=torch.int32, device="cuda")
    gb.exclusive_scan(x)
    out = torch.empty(nscan, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    reps = 5
    e0.record(stream)
    for _ in range(reps):
        gb._lib.check(gb._lib.lib.gbfs_exclusive_scan_i32(gb._lib.C.c_void_p(x.data_ptr()),
                                                          gb._lib.C.c_void_p(out.data_ptr()), nscan,
                                                          gb._lib.C.c_void_p(stream.cuda_stream)), "scan")
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    peak, kind = measured_peak()
    gbs = 12 * nscan / (ms / 1e3) / 1e9
    res["exclusive_scan"] = {"workload": f"{nscan} int32 -> int64 exclusive prefix sum (12 B per element), "
                                         "through the C ABI (each call reads its status back)",
                             "ms": round(ms, 3), "GB_per_s": round(gbs, 1), "frac_of_hbm_peak": round(gbs / peak, 3),
                             "peak_kind": kind}
    return res


def measure_serving(torch, seconds: float = 2.0, fractions=(0.25, 0.5, 0.75, 1.0), max_queries: int = 3000,
                    num_slots: int = 6) -> dict:
    """32 resident graphs, Poisson arrivals at fractions of the measured capacity."""
    import gpu_graphs_gb300 as gb
    rng = np.random.default_rng(5)
    graphs = []
    for i in range(16):
        sc = int(rng.integers(12, 23))
        s_, d_ = gb.gen_rmat(sc, 16, 0.57, 0.19, 0.19, seed=100 + i)
        graphs.append(gb.Graph.from_edges(1 << sc, s_, d_, gb.UNDIRECTED | gb.HUB_FIRST))
    for i in range(16):
        side = int(rng.integers(64, 4097))
        s_, d_ = gb.gen_grid(side, 0.1, 0.001, 8, seed=200 + i)
        graphs.append(gb.Graph.from_edges(side * side, s_, d_, gb.UNDIRECTED))
    del s_, d_
    log("serving: 32 graphs built")
    nz = []
    for g in graphs:
        r, _ = g.csr()
        nz.append(np.flatnonzero(np.diff(r) > 0))

    def draw():
        gi = int(rng.integers(32))
        return gi, int(rng.choice(nz[gi]))

    # plain: one query per launch, back to back, device-timed
    draws = [draw() for _ in range(96)]
    plain_ms = sorted(graphs[gi].bfs(s0, stats=True)[1].ms for gi, s0 in draws)
    for g in graphs:
        g.set_params(direction=1)
    plain_td_ms = sum(graphs[gi].bfs(s0, stats=True)[1].ms for gi, s0 in draws)
    for g in graphs:
        g.set_params(direction=0)
    out = {"workload": "32 resident graphs: 16 RMAT scale U{12..22} ef 16, 16 grids side U[64, 4096]; "
                       "queries pick a graph uniformly and a source uniformly among degree>0 vertices; "
                       f"{num_slots} slots, batch window max(0.5 ms, 10% of the graph's recent launch time); "
                       "grids (degree <= 16) served as up to 4 concurrent single-source searches per slot, "
                       "each unit refilled as its search ends; "
                       "results copied into pinned host buffers",
           "plain_one_query_per_launch": {"queries_per_s": round(len(plain_ms) / (sum(plain_ms) / 1e3), 1),
                                          "p50_ms": round(plain_ms[len(plain_ms) // 2], 3),
                                          "p99_ms": round(plain_ms[int(0.99 * (len(plain_ms) - 1))], 3)},
           "plain_topdown_queries_per_s": round(len(draws) / (plain_td_ms / 1e3), 1)}
    log("serving: plain baseline done")
    # the first 32 of the same queries on the host cores, one per core at a time
    import oracle
    cpu_draws = draws[:32]
    ocsr = {}
    for gi, _ in cpu_draws:
        if gi not in ocsr:
            r_, c_ = graphs[gi].csr()
            ocsr[gi] = oracle.CSR(graphs[gi].n, r_.astype(np.int64), c_)
    cpu, lv = cpu_parallel_queries([(ocsr[gi], s0) for gi, s0 in cpu_draws])
    cpu["kind"] = "port"
    cpu["levels_identical"] = all(np.array_equal(a, graphs[gi].bfs(s0)) for a, (gi, s0) in zip(lv, cpu_draws))
    out["cpu_parallel"] = cpu
    del ocsr, lv
    log(f"serving: cpu parallel {cpu}")
    sweep = []
    # pinned result buffers (8 per graph, reused round robin: contents are not
    # checked here, the serving tests do that)
    pinned = [[torch.empty(g.n, dtype=torch.int32, pin_memory=True) for _ in range(8)] for g in graphs]
    pools = [[t.numpy() for t in ts] for ts in pinned]
    counters = [0] * 32
    cfg = dict(mem_budget_bytes=150 << 30, num_slots=num_slots, max_lanes=64, batch_window_us=500, window_pct=10)

    def submitter(srv, gids):
        def submit():
            gi, s0 = draw()
            buf = pools[gi][counters[gi] % 8]
            counters[gi] += 1
            return srv.submit(gids[gi], s0, buf)
        return submit

    # closed loop: everything queued at once -> capacity
    with gb.Server(**cfg) as srv:
        submit = submitter(srv, [srv.add_graph(g) for g in graphs])
        t0 = time.perf_counter()
        ts = [submit() for _ in range(1024)]
        for t in ts:
            srv.wait(t)
        capacity = 1024 / (time.perf_counter() - t0)
        out["capacity_queries_per_s"] = round(capacity, 1)
        out["peak_hbm_bytes"] = srv.stats()["peak_bytes"]
    log(f"serving: capacity {capacity:.0f} q/s")
    # open loop, Poisson arrivals: 10x the plain rate, then fractions of the
    # capacity; a fresh server per point (its launch-time estimates start from
    # a short warm-up at that rate, not from the closed loop's full batches)
    plain_qps = out["plain_one_query_per_launch"]["queries_per_s"]
    rates = sorted([10 * plain_qps] + [f * capacity for f in fractions])
    for rate in rates:
        with gb.Server(**cfg) as srv:
            submit = submitter(srv, [srv.add_graph(g) for g in graphs])

            def run(duration):
                tickets = []
                t0 = time.perf_counter()
                next_t = t0
                while len(tickets) < max_queries:
                    now = time.perf_counter()
                    if now - t0 >= duration:
                        break
                    if now < next_t:
                        time.sleep(min(next_t - now, 0.0005))
                        continue
                    tickets.append(submit())
                    next_t += rng.exponential(1.0 / rate)
                for t in tickets:
                    srv.wait(t)
                return len(tickets), time.perf_counter() - t0

            run(0.5)  # warm-up at this rate
            srv.reset_stats()
            nsub, wall = run(seconds)
            st = srv.stats()
            sweep.append({"offered_queries_per_s": round(rate, 1), "offered_vs_plain": round(rate / plain_qps, 2),
                          "submitted": nsub, "achieved_queries_per_s": round(nsub / wall, 1),
                          "p50_ms": round(st["p50_ms"], 3), "p99_ms": round(st["p99_ms"], 3),
                          "mean_batch_lanes": round(st["mean_batch_lanes"], 2)})
            log(f"serving: {sweep[-1]}")
    out["sweep"] = sweep
    out["capacity_vs_plain"] = round(capacity / out["plain_one_query_per_launch"]["queries_per_s"], 2)
    out["capacity_vs_plain_topdown"] = round(capacity / out["plain_topdown_queries_per_s"], 2)
    out["capacity_vs_cpu_parallel"] = round(capacity / out["cpu_parallel"]["queries_per_s"], 1)
    return out

def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    torch.cuda.set_device(local)
    if args.grid_only:
        print(json.dumps(grid_only(args.grid_side, args.steps)), flush=True)
        return
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

    # parity check against the oracle (outside the timed region): the
    # highest-degree vertex and the first 7 bench sources, bit for bit
    import oracle
    og = oracle.CSR(n, row.astype(np.int64), col)
    chk = [int(np.argmax(deg))] + [int(s) for s in sources[:7]]
    got = g.bfs_many(chk)[0]
    with cf.ThreadPoolExecutor(min(len(chk), os.cpu_count() or 1)) as ex:
        want = list(ex.map(lambda s0: oracle.bfs_queue(og, s0), chk))
    parity = {"sources": len(chk), "includes_max_degree_vertex": True,
              "levels_identical": all(np.array_equal(a, b) for a, b in zip(got, want))}
    del got, want

    launch_ms, launch_ec, edges_c, verts, lvls = [], [], 0, 0, []
    with ClockSampler(local) as clk:
        for _ in range(args.warmup):
            g.bfs_many(sources, out=out)
        torch.cuda.synchronize()
        dist.barrier()
        clk.mark_start()
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
        clk.mark_end()
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
    traffic, traffic_src = profiled_traffic() if args.scale == 22 else (None, "other workload")
    mean_s = float(np.mean(launch_ms)) / 1e3
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                "achieved_is": "algorithmic bytes per launch (4*E_c + 8*V_c + 4*n) / mean launch time",
                "bytes_per_launch": int(b_alg / launches), "mean_launch_us": round(1e6 * mean_s, 2),
                "traffic": traffic, "traffic_source": traffic_src,
                "dram_achieved": round(traffic / mean_s / 1e9, 1) if traffic else None,
                "dram_frac": round(traffic / mean_s / 1e9 / peak, 4) if traffic else None,
                "limiter": "latency and level synchronisation: bottom-up steps stop at the first parent, so "
                           "measured DRAM traffic is a fraction of the algorithmic bytes"}
    gteps_each = [(e / 2) / (t / 1e3) / 1e9 for e, t in zip(launch_ec, launch_ms)]

    # e2e through the C ABI with pinned host output buffers
    e2e = None
    if not args.no_e2e:
        host = torch.empty((k, n), dtype=torch.int32, pin_memory=True)
        hv = host.numpy()
        g.bfs_many(sources, out=hv)
        torch.cuda.synchronize()
        dist.barrier()
        steps_e2e = max(1, args.steps)
        t0 = time.perf_counter()
        for _ in range(steps_e2e):
            g.bfs_many(sources, out=hv)
        t1 = time.perf_counter()
        dist.barrier()
        wall = dist.reduce(t1 - t0, "max")
        e2e = {"value": round(dist.reduce(und_edges / args.steps * steps_e2e, "sum") / wall / 1e9, 3),
               "unit": "GTEPS", "h2d_bytes_per_step": 4 * k, "d2h_bytes_per_step": 4 * k * n,
               "steps": steps_e2e, "clock": "host perf_counter around the calls",
               "graph": "resident in HBM (built before the timed region; see e2e_from_edge_list)"}
        del host, hv

    extra = {}
    # the other configurations and the CPU baseline: single-GPU runs only
    # (a scaling run holds all N GPUs; its line needs the headline alone)
    if rank == 0 and world == 1 and not args.no_extra:
        extra["config1"] = measure_config1(torch)
        log("config1 done")
        extra["e2e_from_edge_list"] = measure_e2e_from_edge_list(args.scale, sources, torch)
        log("e2e from edge list done")
        extra["grid"] = measure_grid(args.grid_side, torch)
        log("grid done")
        extra["batched"] = measure_batched(torch)
        log("batched done")
        extra["primitives"] = measure_primitives(torch)
        log("primitives done")
        if not args.no_large:
            extra["graph500"] = {f"scale{sc}": measure_rmat_large(torch, sc) for sc in (26, 27)}
            log(f"large RMAT done: {extra['graph500']}")
    if rank == 0 and world == 1 and not args.no_serving and not args.no_extra:
        extra["serving"] = measure_serving(torch)

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        threads = args.cpu_threads or (os.cpu_count() or 1)
        sel = sources[: min(threads, k)]
        wall, e, lv = cpu_bfs_sample(og, sel, len(sel))
        cpu = {"value": round(e / wall / 1e9, 4), "unit": "GTEPS", "cores": len(sel), "kind": "port",
               "host": host_cpu(),
               "sample": f"{len(sel)} of the {k} sources, one per thread, oracle restatement of the "
                         f"reference's queue BFS ({wall:.2f} s)",
               "single_thread": cpu_single_thread(og, sources[:2])}

    if rank == 0:
        line = {
            "metric": "single-source GTEPS", "value": round(value, 3), "unit": "GTEPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic", "config": config_block(args, n, g.m),
            "engine": {"parallelism": f"replicas{world}", "layout": args.layout, "params": params},
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clk.summary(), "parity_check": parity,
            "per_source_gteps": {"min": round(min(gteps_each), 2), "median": round(statistics.median(gteps_each), 2),
                                 "max": round(max(gteps_each), 2)},
            "levels_td_bu": sorted(set(lvls))[:8],
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
