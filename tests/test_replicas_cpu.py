"""The multi-GPU path of bench.py is replicas only: a barrier and max/sum
reductions over ranks, no collective on the data path.  Checked here with
two gloo ranks on the CPU (127.0.0.1 rendezvous)."""
from __future__ import annotations

import os
import socket

import pytest

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import sys
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench.Dist(world, "gloo")
    d.barrier()
    t_max = d.reduce(1.5 + rank, "max")        # slowest rank's time
    e_sum = d.reduce(100.0 * (rank + 1), "sum")  # all ranks' edges
    assert bench.dist_env() == (rank, world, rank)
    # the reference arm prints only on rank 0; other ranks return at once
    ret = bench.run_reference(type("A", (), {})(), rank, world) if rank != 0 else None
    d.close()
    q.put((rank, t_max, e_sum, ret))


def test_two_gloo_ranks_reduce_like_the_bench():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t_max, e_sum, ret in res:
        assert t_max == 2.5
        assert e_sum == 300.0
        assert ret is None
