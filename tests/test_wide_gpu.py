"""GPU: graphs with 64-bit row offsets ("wide"), bit for bit.

Small graphs built with GBFS_WIDE_ROWS run every wide kernel (the CSR
build's scatter, sorts and compaction, the grid kernel's top-down and
bottom-up steps, the label-correcting kernel, parents) against the oracle
and against the same graph with 32-bit offsets; the full-size test builds a
graph of more than 2^31 stored edges, which only the wide layout can hold.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair(gb, n, src, dst, flags):
    return gb.Graph.from_edges(n, src, dst, flags), gb.Graph.from_edges(n, src, dst, flags | gb.WIDE_ROWS)


def test_wide_csr_equals_narrow(gb):
    src, dst = gb.gen_rmat(16, 16, seed=5)
    n = 1 << 16
    for flags in (gb.UNDIRECTED, gb.UNDIRECTED | gb.HUB_FIRST, gb.DEDUP | gb.DROP_SELF_LOOPS, 0):
        g32, g64 = _pair(gb, n, src, dst, flags)
        assert not g32.wide and g64.wide
        r32, c32 = g32.csr()
        r64, c64 = g64.csr()
        assert r64.dtype == np.int64
        assert np.array_equal(r32.astype(np.int64), r64)
        assert np.array_equal(c32, c64)
        assert g32.max_degree == g64.max_degree and g32.nonisolated == g64.nonisolated
        # the int32 export refuses 64-bit offsets
        row = np.empty(n + 1, np.int32)
        col = np.empty(max(g64.m, 1), np.int32)
        rc = gb._lib.lib.gbfs_graph_get_csr(g64.handle, row.ctypes.data, col.ctypes.data)
        assert rc == gb._lib.ERR_TOO_LARGE
        assert np.array_equal(g64.row_offsets(), r64) and np.array_equal(g32.row_offsets(), r64)


@pytest.mark.parametrize("direction", [0, 1, 2])
def test_wide_rmat_levels(gb, orc, direction):
    src, dst = gb.gen_rmat(17, 16, seed=6)
    n = 1 << 17
    g32, g64 = _pair(gb, n, src, dst, gb.UNDIRECTED | gb.HUB_FIRST)
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    deg = np.diff(g32.csr()[0])
    for g in (g32, g64):
        g.set_params(direction=direction)
    sources = [int(np.argmax(deg))] + [int(s) for s in np.random.default_rng(1).choice(np.flatnonzero(deg > 0), 4)]
    for s in sources:
        want = orc.bfs_queue(o, s)
        got, st = g64.bfs(s, stats=True)
        assert np.array_equal(got, want), s
        _, st32 = g32.bfs(s, stats=True)
        for k in ("levels", "vertices_reached", "edges_in_component", "edges_traversed", "td_levels", "bu_levels"):
            assert getattr(st, k) == getattr(st32, k), (k, s)
    # several sources back to back, device output, multi-root
    outs, _ = g64.bfs_many(sources)
    for i, s in enumerate(sources):
        assert np.array_equal(outs[i], orc.bfs_queue(o, s))
    assert np.array_equal(g64.bfs_multiroot(sources[:3]), g32.bfs_multiroot(sources[:3]))


def test_wide_high_diameter_and_parents(gb, orc):
    side = 400
    src, dst = gb.gen_grid(side, 0.1, 0.001, 8, seed=3)
    n = side * side
    g32, g64 = _pair(gb, n, src, dst, gb.UNDIRECTED)
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    for s in (0, n // 2 + 7, n - 1):
        got, st = g64.bfs(s, stats=True)
        assert np.array_equal(got, orc.bfs_queue(o, s)), s
        assert st.launches == 2  # grid kernel, then the label-correcting kernel
        assert st.vertices_reached == int((got >= 0).sum())
        assert st.edges_in_component == orc.component_edges(o, got)
        assert any(r["dir"] == "relaxed" for r in g64.last_trace())
        lv, par = g64.bfs_parents(s)
        lv32, par32 = g32.bfs_parents(s)
        assert np.array_equal(lv, lv32) and np.array_equal(par, par32)


def test_wide_directed_stays_topdown(gb, orc):
    src, dst = gb.gen_rmat(15, 8, seed=7)
    n = 1 << 15
    flags = gb.DEDUP | gb.DROP_SELF_LOOPS
    g = gb.Graph.from_edges(n, src, dst, flags | gb.WIDE_ROWS)
    o = orc.csr_build(n, src, dst, orc.DEDUP | orc.DROP_SELF_LOOPS)
    deg = np.diff(g.csr()[0])
    for s in [int(np.argmax(deg)), 3, 100]:
        got, st = g.bfs(s, stats=True)  # no transpose for wide graphs: top-down only
        assert np.array_equal(got, orc.bfs_queue(o, s))
        assert st.bu_levels == 0
        lv, par = g.bfs_parents(s)
        assert np.array_equal(lv, got)
        assert np.array_equal(par, orc.min_parents(o, lv))


def test_wide_save_load_and_refusals(gb, orc, tmp_path):
    src, dst = gb.gen_rmat(14, 16, seed=8)
    n = 1 << 14
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | gb.WIDE_ROWS)
    path = str(tmp_path / "wide.bin")
    g.save(path)
    h = gb.Graph.load(path)
    assert h.wide and h.m == g.m
    r1, c1 = g.csr()
    r2, c2 = h.csr()
    assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
    assert np.array_equal(h.bfs(5), g.bfs(5))
    # hub-first rows are not sorted: loading checks symmetry on a sorted copy
    gh = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | gb.HUB_FIRST | gb.WIDE_ROWS)
    gh.save(path)
    hh = gb.Graph.load(path)
    assert hh.wide and np.array_equal(hh.csr()[1], gh.csr()[1])
    assert np.array_equal(hh.bfs(5), g.bfs(5))
    too_large = gb._lib.ERR_TOO_LARGE
    with pytest.raises(gb.GbfsError) as e:
        g.bfs_multi([0, 1])
    assert e.value.code == too_large
    g.set_params(per_level_launch=1)
    with pytest.raises(gb.GbfsError) as e:
        g.bfs(0)
    assert e.value.code == too_large
    g.set_params(per_level_launch=0)
    with gb.Server(mem_budget_bytes=1 << 30, num_slots=1) as srv:
        with pytest.raises(gb.GbfsError) as e:
            srv.add_graph(g)
        assert e.value.code == too_large
    with pytest.raises(gb.GbfsError) as e:
        gb.GraphSet.from_graphs([g])
    assert e.value.code == too_large
    # a wide graph set from edges runs the fused multi-root search
    gs = gb.GraphSet.from_edges([(n, src, dst), (n, src, dst)], flags=gb.UNDIRECTED | gb.WIDE_ROWS)
    outs = gs.bfs([5, 9])
    assert np.array_equal(outs[0], g.bfs(5)) and np.array_equal(outs[1], g.bfs(9))


def test_wide_beyond_int32_edges(gb, orc):
    """RMAT scale 26, edge factor 24: 1.6 G pairs, about 3.2 G stored
    directed edges, more than 2^31-1: only 64-bit offsets hold it."""
    free, _ = __import__("torch").cuda.mem_get_info()
    if free < 80 << 30:
        pytest.skip("needs about 60 GB of free device memory")
    import bench
    src, dst = gb.gen_rmat(26, 24, 0.57, 0.19, 0.19, seed=1)
    n = 1 << 26
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | gb.HUB_FIRST)
    del src, dst
    assert g.wide and g.m > 2**31
    row, col = g.csr()
    assert row.dtype == np.int64 and int(row[-1]) == g.m
    deg = np.diff(row)
    s = int(bench.pick_sources(deg, 1)[0])
    got, st = g.bfs(s, stats=True)
    o = orc.CSR(n, row, col)
    want = orc.bfs_queue(o, s)
    assert np.array_equal(got, want)
    assert st.vertices_reached == int((want >= 0).sum())
    assert st.bu_levels > 0
