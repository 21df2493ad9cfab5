"""GPU parity at the benchmark configurations themselves, bit for bit.

  * RMAT scale 22, the bench's own sources: the highest-degree vertex and
    the first eight of the 64 bench sources, one launch each;
  * RMAT scale 20 with the 64 bench sources in ONE multi-source launch
    (uint64 lane masks), every lane against the oracle;
  * the 512 small Erdos-Renyi graphs (n log-uniform in [2^8, 2^16], average
    degree 8) in ONE fused launch, every graph against the oracle;
  * a serving mix with large grids (sides 1024 and 1536, thousands of
    levels) and an RMAT scale-18 graph next to small graphs: every query's
    levels in the mix equal the same query alone and the oracle.

The oracle's queue BFS (a restatement of the reference's CPU BFS) runs in a
thread pool; ctypes releases the GIL for each call.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_levels(orc, g, sources):
    with cf.ThreadPoolExecutor(min(len(sources), os.cpu_count() or 1)) as ex:
        return list(ex.map(lambda s: orc.bfs_queue(g, int(s)), sources))


@pytest.fixture(scope="module")
def bench():
    import bench as b
    return b


def test_rmat22_bench_sources(gb, orc, bench):
    n, src, dst = bench.workload(22)
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | gb.HUB_FIRST)
    del src, dst
    row, col = g.csr()
    deg = np.diff(row)
    sources = bench.pick_sources(deg, 64)
    chk = [int(np.argmax(deg))] + [int(s) for s in sources[:8]]
    got, sts = g.bfs_many(chk)
    og = orc.CSR(n, row.astype(np.int64), col)
    want = _oracle_levels(orc, og, chk)
    for i, s in enumerate(chk):
        assert np.array_equal(got[i], want[i]), (i, s)
        assert sts[i].vertices_reached == int((want[i] >= 0).sum())
        assert sts[i].bu_levels > 0  # the direction-optimising path ran
    # the hub's search reaches the giant component
    assert sts[0].vertices_reached > n // 2


def test_rmat20_64_lanes_one_launch(gb, orc, bench):
    n = 1 << 20
    src, dst = gb.gen_rmat(20, 16, 0.57, 0.19, 0.19, seed=1)
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | gb.HUB_FIRST)
    del src, dst
    row, col = g.csr()
    sources = bench.pick_sources(np.diff(row), 64)
    got, st = g.bfs_multi(sources, stats=True)
    assert st.launches == 1
    og = orc.CSR(n, row.astype(np.int64), col)
    want = _oracle_levels(orc, og, sources)
    reached = 0
    for i, s in enumerate(sources):
        assert np.array_equal(got[i], want[i]), (i, int(s))
        reached += int((want[i] >= 0).sum())
    assert st.vertices_reached == reached


def test_512_graphs_one_fused_launch(gb, orc, bench):
    graphs, srcs = bench.many_graphs_workload(gb)
    assert len(graphs) == 512
    total = sum(ni for ni, _, _ in graphs)
    assert 4_000_000 < total < 8_000_000
    gs = gb.GraphSet.from_edges(graphs)
    outs, st = gs.bfs(srcs, stats=True)
    assert st.launches == 1

    def check(i):
        ni, s_, d_ = graphs[i]
        want = orc.bfs_queue(orc.csr_build(ni, s_, d_, orc.UNDIRECTED), srcs[i])
        return np.array_equal(outs[i], want)

    with cf.ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        ok = list(ex.map(check, range(len(graphs))))
    assert all(ok), [i for i, x in enumerate(ok) if not x][:10]


def test_server_mix_with_large_graphs(gb, orc):
    specs = [("grid", 1024, 21), ("grid", 1536, 22), ("rmat", 18, 23), ("rmat", 14, 24), ("grid", 300, 25),
             ("er", 50_000, 26)]
    graphs = []
    for kind, size, seed in specs:
        if kind == "rmat":
            s, d = gb.gen_rmat(size, 16, seed=seed)
            n = 1 << size
            flags = gb.UNDIRECTED | gb.HUB_FIRST
        elif kind == "grid":
            s, d = gb.gen_grid(size, 0.1, 0.001, 8, seed=seed)
            n = size * size
            flags = gb.UNDIRECTED
        else:
            s, d = gb.gen_er(size, 4 * size, seed)
            n = size
            flags = gb.UNDIRECTED
        g = gb.Graph.from_edges(n, s, d, flags)
        row, col = g.csr()
        graphs.append((g, orc.CSR(n, row.astype(np.int64), col), np.flatnonzero(np.diff(row) > 0)))
    rng = np.random.default_rng(9)
    plan = []
    for _ in range(240):
        gi = int(rng.integers(len(graphs)))
        plan.append((gi, int(rng.choice(graphs[gi][2]))))
    with gb.Server(mem_budget_bytes=16 << 30, num_slots=4, max_lanes=64, batch_window_us=500,
                   window_pct=50) as srv:
        gids = [srv.add_graph(g) for g, _, _ in graphs]
        tickets = [None] * len(plan)

        def submitter(lo, hi):
            for i in range(lo, hi):
                gi, s = plan[i]
                tickets[i] = srv.submit(gids[gi], s)

        ths = [threading.Thread(target=submitter, args=(k * 60, (k + 1) * 60)) for k in range(4)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        mixed, lanes = [], []
        for i in range(len(plan)):
            got, info = srv.wait(tickets[i])
            assert info.status == 0
            mixed.append(got)
            lanes.append(info.batch_lanes)
        assert max(lanes) > 1  # queries shared launches
        # the large graphs were in the mix
        assert {gi for gi, _ in plan} == set(range(len(graphs)))
    # each query alone (one single-source launch on the whole GPU) and the oracle
    for i, (gi, s) in enumerate(plan):
        alone = graphs[gi][0].bfs(s)
        assert np.array_equal(mixed[i], alone), (i, gi, s)
    want = {}
    with cf.ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        futs = {i: ex.submit(orc.bfs_queue, graphs[gi][1], s) for i, (gi, s) in enumerate(plan)}
        for i, f in futs.items():
            want[i] = f.result()
    for i in range(len(plan)):
        assert np.array_equal(mixed[i], want[i]), (i, plan[i])
