"""GPU parity at the benchmark sizes.

RMAT scale 22 (128M directed edges) and the 7000x7000 perturbed grid
(49M vertices, thousands of levels): the device CSR is compared with the
oracle's CSR build, the levels with the oracle's BFS, bit for bit, and the
levels are also checked against properties that hold for exact BFS
distances whatever the CSR order (source at 0; across every edge a reached
vertex's neighbour is reached and at most one level further; every reached
vertex but the source has a neighbour exactly one level closer).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def check_bfs_properties(row: np.ndarray, col: np.ndarray, level: np.ndarray, source: int) -> None:
    n = len(row) - 1
    deg = np.diff(row).astype(np.int64)
    assert level[source] == 0
    assert level.min() >= -1
    owner = np.repeat(np.arange(n, dtype=np.int32), deg)
    lu = level[owner].astype(np.int64)
    lv = level[col].astype(np.int64)
    reached_u = lu >= 0
    assert (lv[reached_u] >= 0).all(), "a reached vertex has an unreached neighbour"
    assert (lv[reached_u] <= lu[reached_u] + 1).all(), "a level jumps by more than one across an edge"
    # every reached v != source has a neighbour at level(v) - 1
    big = np.int64(1) << 40
    lv_or_big = np.where(lv >= 0, lv, big)
    nz = np.flatnonzero(deg > 0)
    mins = np.minimum.reduceat(lv_or_big, row[nz].astype(np.int64))
    reached = level[nz] >= 0
    notsrc = nz != source
    sel = reached & notsrc
    assert (mins[sel] == level[nz][sel].astype(np.int64) - 1).all(), "a reached vertex has no parent one level up"
    iso = np.flatnonzero(deg == 0)
    assert (level[iso[iso != source]] == -1).all()


def test_rmat22_full_size(gb, orc):
    n = 1 << 22
    src, dst = gb.gen_rmat(22, 16, 0.57, 0.19, 0.19, seed=1)
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | gb.HUB_FIRST)
    row, col = g.csr()
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    del src, dst
    assert np.array_equal(row, o.row_offset) and g.m == o.m
    deg = np.diff(row)
    # hub-first rows hold the same neighbours as the oracle's sorted rows
    for r in np.flatnonzero(deg >= 2)[::997][:3000]:
        assert np.array_equal(np.sort(col[row[r]:row[r + 1]]), o.col_idx[row[r]:row[r + 1]])
    rng = np.random.default_rng(1)
    sources = rng.choice(np.flatnonzero(deg > 0), 2, replace=False)
    for s in sources:
        got = g.bfs(int(s))
        assert np.array_equal(got, orc.bfs_queue(o, int(s)))
        check_bfs_properties(row, col, got, int(s))


def test_grid_7000_full_size(gb, orc):
    side = 7000
    n = side * side
    src, dst = gb.gen_grid(side, 0.1, 0.001, 8, seed=1)
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED)
    del src, dst
    row, col = g.csr()
    deg = np.diff(row)
    s = int(np.random.default_rng(2).choice(np.flatnonzero(deg > 0)))
    got, st = g.bfs(s, stats=True)
    assert st.levels > 1000 and st.launches == 2  # grid and label-correcting launches
    check_bfs_properties(row, col, got, s)
    o = orc.CSR(n, row.astype(np.int64), col)
    assert np.array_equal(got, orc.bfs_queue(o, s))
