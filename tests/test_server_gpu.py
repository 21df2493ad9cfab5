"""GPU: the continuous-batching server (results alone == results in the mix)."""
from __future__ import annotations

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _graphs(gb, orc):
    specs = [("rmat", 14, 1), ("rmat", 12, 2), ("grid", 60, 3), ("er", 3000, 4)]
    out = []
    for kind, size, seed in specs:
        if kind == "rmat":
            s, d = gb.gen_rmat(size, 16, seed=seed)
            n = 1 << size
        elif kind == "grid":
            s, d = gb.gen_grid(size, 0.1, 0.001, 8, seed=seed)
            n = size * size
        else:
            s, d = gb.gen_er(size, 3 * size, seed)
            n = size
        g = gb.Graph.from_edges(n, s, d)
        out.append((g, orc.csr_build(n, s, d, orc.UNDIRECTED)))
    return out


@pytest.mark.parametrize("window_pct", [0, 50])
def test_server_mix_equals_alone(gb, orc, window_pct):
    graphs = _graphs(gb, orc)
    with gb.Server(mem_budget_bytes=8 << 30, num_slots=3, max_lanes=64, batch_window_us=300,
                   window_pct=window_pct) as srv:
        gids = [srv.add_graph(g) for g, _ in graphs]
        rng = np.random.default_rng(5)
        plan = [(int(rng.integers(len(graphs))), None) for _ in range(400)]
        plan = [(gi, int(rng.integers(graphs[gi][0].n))) for gi, _ in plan]
        tickets = [None] * len(plan)

        def submitter(lo, hi):
            for i in range(lo, hi):
                gi, s = plan[i]
                tickets[i] = srv.submit(gids[gi], s)

        ths = [threading.Thread(target=submitter, args=(k * 100, (k + 1) * 100)) for k in range(4)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        lanes = []
        for i, (gi, s) in enumerate(plan):
            got, info = srv.wait(tickets[i])
            assert info.status == 0
            lanes.append(info.batch_lanes)
            want = orc.bfs_queue(graphs[gi][1], s)
            assert np.array_equal(got, want), (gi, s)
        st = srv.stats()
        assert st["completed"] == len(plan)
        assert st["mean_batch_lanes"] > 1.0          # queries were batched
        assert max(lanes) > 1
        assert st["p99_ms"] >= st["p50_ms"] > 0
        # the same query alone gives the same levels
        gi, s = plan[0]
        t = srv.submit(gids[gi], s)
        alone, info = srv.wait(t)
        assert info.batch_lanes == 1
        assert np.array_equal(alone, orc.bfs_queue(graphs[gi][1], s))


def test_server_budget_and_errors(gb, orc):
    for bad in ({"window_pct": -1}, {"window_pct": 1001}, {"max_lanes": 65}, {"num_slots": 0}):
        with pytest.raises(gb.GbfsError) as e:
            gb.Server(mem_budget_bytes=1 << 30, **bad)
        assert e.value.code == gb._lib.ERR_INVALID_ARG
    graphs = _graphs(gb, orc)
    g = graphs[0][0]
    with gb.Server(mem_budget_bytes=1 << 20, num_slots=2) as srv:
        with pytest.raises(gb.GbfsError) as e:
            srv.add_graph(g)
        assert e.value.code == gb._lib.ERR_BUDGET
        assert srv.stats()["rejected"] == 1
    with gb.Server(mem_budget_bytes=4 << 30, num_slots=2) as srv:
        gid = srv.add_graph(g)
        with pytest.raises(gb.GbfsError) as e:
            srv.submit(gid + 100, 0)
        assert e.value.code == gb._lib.ERR_NOT_FOUND
        with pytest.raises(gb.GbfsError) as e:
            srv.submit(gid, g.n)
        assert e.value.code == gb._lib.ERR_INVALID_ARG
        t = srv.submit(gid, 0)
        srv.wait(t)
        srv.remove_graph(gid)
        with pytest.raises(gb.GbfsError):
            srv.remove_graph(gid)


def test_bounded_wait_reports_timeout_and_context_survives(gb, orc):
    lib = gb._lib.lib
    assert lib.gbfs_selftest_wait_timeout(50) == gb._lib.ERR_TIMEOUT
    # the context is still usable afterwards
    s, d = gb.gen_er(1000, 3000, 1)
    g = gb.Graph.from_edges(1000, s, d)
    assert np.array_equal(g.bfs(0), orc.bfs_queue(orc.csr_build(1000, s, d, orc.UNDIRECTED), 0))


def test_server_with_concurrent_param_changes(gb, orc):
    """Parameters changed from another thread while the server runs: results stay exact."""
    graphs = _graphs(gb, orc)
    stop = threading.Event()

    def toggler():
        i = 0
        while not stop.is_set():
            for g, _ in graphs:
                g.set_params(alpha=8 if i % 2 else 14, direction=i % 3)
            i += 1

    th = threading.Thread(target=toggler)
    th.start()
    try:
        with gb.Server(mem_budget_bytes=8 << 30, num_slots=3, max_lanes=64, batch_window_us=200) as srv:
            gids = [srv.add_graph(g) for g, _ in graphs]
            rng = np.random.default_rng(9)
            plan = [(int(rng.integers(len(graphs))), 0) for _ in range(150)]
            plan = [(gi, int(rng.integers(graphs[gi][0].n))) for gi, _ in plan]
            tickets = [srv.submit(gids[gi], s) for gi, s in plan]
            for t, (gi, s) in zip(tickets, plan):
                got, info = srv.wait(t)
                assert info.status == 0
                assert np.array_equal(got, orc.bfs_queue(graphs[gi][1], s)), (gi, s)
    finally:
        stop.set()
        th.join()


def test_server_directed_graphs(gb, orc):
    """Directed graphs in the server: single queries and batches step
    bottom-up / pull over the transpose built at admission."""
    graphs = []
    for scale, seed in ((13, 21), (11, 22)):
        s, d = gb.gen_rmat(scale, 16, seed=seed)
        n = 1 << scale
        flags = gb.DEDUP | gb.DROP_SELF_LOOPS
        graphs.append((gb.Graph.from_edges(n, s, d, flags), orc.csr_build(n, s, d, flags)))
    s, d = gb.gen_er(5000, 20000, 23)
    graphs.append((gb.Graph.from_edges(5000, s, d, 0), orc.csr_build(5000, s, d, 0)))
    graphs[2][0].set_params(direction=1)  # stays top-down: no transpose
    with gb.Server(mem_budget_bytes=4 << 30, num_slots=2, max_lanes=64, batch_window_us=300) as srv:
        gids = [srv.add_graph(g) for g, _ in graphs]
        rng = np.random.default_rng(24)
        plan = [int(rng.integers(len(graphs))) for _ in range(300)]
        plan = [(gi, int(rng.integers(graphs[gi][0].n))) for gi in plan]
        tickets = [srv.submit(gids[gi], s0) for gi, s0 in plan]
        for t, (gi, s0) in zip(tickets, plan):
            got, info = srv.wait(t)
            assert info.status == 0
            assert np.array_equal(got, orc.bfs_queue(graphs[gi][1], s0)), (gi, s0)
        for gi, (g, o) in enumerate(graphs):  # one query alone (single-source kernel)
            t = srv.submit(gids[gi], 0)
            got, info = srv.wait(t)
            assert info.batch_lanes == 1 and np.array_equal(got, orc.bfs_queue(o, 0))
