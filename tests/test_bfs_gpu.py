"""GPU parity: CSR build and single-source / multi-root BFS against the oracle.

Every level array must equal the oracle's (which is pinned to the
reference's own CPU BFS by tests/test_oracle.py) bit for bit, including -1
for unreachable and isolated vertices.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_names, load_golden, synthetic_edges

pytestmark = pytest.mark.gpu

MODES = {"opt": 0, "td": 1, "bu": 2}


def sorted_rows_equal(row_a, col_a, row_b, col_b) -> bool:
    if not np.array_equal(np.asarray(row_a, np.int64), np.asarray(row_b, np.int64)):
        return False
    for r in range(len(row_a) - 1):
        a = np.sort(col_a[row_a[r]:row_a[r + 1]])
        b = np.sort(col_b[row_b[r]:row_b[r + 1]])
        if not np.array_equal(a, b):
            return False
    return True


@pytest.mark.parametrize("name", golden_names("ref_"))
def test_reference_fixtures(gb, orc, name):
    d = load_golden(name)
    n = int(d["n"])
    g = gb.Graph.from_edges(n, d["src"], d["dst"], 0)   # directed, as stored
    row, col = g.csr()
    o = orc.csr_build(n, d["src"], d["dst"], 0)
    assert sorted_rows_equal(row, col, o.row_offset, o.col_idx)
    for s, want in zip(d["sources"], d["levels"]):
        got = g.bfs(int(s))
        assert np.array_equal(got, want), (name, int(s))
    if "ref_row" in d:  # the reference's own (unsorted) CSR through from_csr
        g2 = gb.Graph.from_csr(d["ref_row"], d["ref_col"])
        for s, want in zip(d["sources"], d["levels"]):
            assert np.array_equal(g2.bfs(int(s)), want)
    for mode in (1, 2):  # a launch per level: host loop, then a CUDA graph
        g.set_params(per_level_launch=mode)
        for s, want in zip(d["sources"], d["levels"]):
            assert np.array_equal(g.bfs(int(s)), want), (name, int(s), mode)


@pytest.mark.parametrize("name", golden_names("syn_"))
@pytest.mark.parametrize("mode", list(MODES))
def test_synthetic_golden(gb, orc, name, mode):
    d = load_golden(name)
    n, src, dst = synthetic_edges(d)
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED)
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    row, col = g.csr()
    assert np.array_equal(row, o.row_offset) and np.array_equal(col, o.col_idx)
    g.set_params(direction=MODES[mode])
    for s, want in zip(d["sources"], d["levels"]):
        got, st = g.bfs(int(s), stats=True)
        assert np.array_equal(got, want)
        assert st.vertices_reached == int((want >= 0).sum())
        assert st.edges_in_component == orc.component_edges(o, want)
        assert st.levels == int(want.max()) + 1


def _check_against_oracle(gb, orc, n, src, dst, sources, flags=None, params=None):
    flags = gb.UNDIRECTED if flags is None else flags
    g = gb.Graph.from_edges(n, src, dst, flags)
    o = orc.csr_build(n, src, dst, flags)
    row, col = g.csr()
    if flags & gb.DEDUP:
        assert np.array_equal(row, o.row_offset) and np.array_equal(col, o.col_idx)
    if params:
        g.set_params(**params)
    for s in sources:
        want = orc.bfs_queue(o, int(s))
        got = g.bfs(int(s))
        assert np.array_equal(got, want), int(s)
    return g, o


@pytest.mark.parametrize("params", [
    {}, {"threads_per_block": 256, "blocks_per_sm": 4}, {"threads_per_block": 1024, "blocks_per_sm": 1},
    {"alpha": 2, "beta": 4}, {"alpha": 96, "beta": 96}, {"big_degree": 32}, {"big_degree": 4096},
    {"direction": 1}, {"direction": 2}, {"per_level_launch": 1}, {"per_level_launch": 2},
    {"per_level_launch": 2, "direction": 2},
])
def test_rmat18_param_grid(gb, orc, params):
    src, dst = gb.gen_rmat(18, 16, seed=2)
    deg = np.bincount(np.concatenate([src, dst]), minlength=1 << 18)
    rng = np.random.default_rng(0)
    sources = rng.choice(np.flatnonzero(deg > 0), 3, replace=False)
    _check_against_oracle(gb, orc, 1 << 18, src, dst, list(sources) + [int(np.argmax(deg))], params=params)


def test_grid_high_diameter(gb, orc):
    side = 400
    src, dst = gb.gen_grid(side, 0.1, 0.001, 8, seed=3)
    g, o = _check_against_oracle(gb, orc, side * side, src, dst, [0, side * side // 2 + 7])
    want, st = g.bfs(0, stats=True)
    assert st.levels > side  # hundreds of levels
    # degree <= 16: the persistent grid launch hands the search to the
    # label-correcting launch queued behind it at level 4
    assert st.launches == 2
    assert any(r["dir"] == "relaxed" for r in g.last_trace())
    g.set_params(per_level_launch=1)  # the reference's shape: a launch per level
    got, st2 = g.bfs(0, stats=True)
    assert np.array_equal(got, want)
    assert st2.launches == st.levels + 1 and st2.levels == st.levels
    g.set_params(per_level_launch=2)  # the same launches replayed by a CUDA graph
    for s0 in (0, side * side // 2 + 7, 0):  # the second query of the same shape reuses the graph
        got3, st3 = g.bfs(s0, stats=True)
        assert np.array_equal(got3, orc.bfs_queue(o, s0))
        assert st3.launches == st3.levels + 1
    # multi-root through the graph (roots from device memory)
    mr = g.bfs_multiroot([0, side * side - 1])
    g.set_params(per_level_launch=0)
    assert np.array_equal(mr, g.bfs_multiroot([0, side * side - 1]))


def test_er_and_directed(gb, orc):
    src, dst = gb.gen_er(200000, 800000, seed=4)
    _check_against_oracle(gb, orc, 200000, src, dst, [0, 5, 199999])
    # directed as stored: bottom-up steps probe the transpose (in-edges)
    src, dst = gb.gen_er(50000, 150000, seed=5)
    g, _ = _check_against_oracle(gb, orc, 50000, src, dst, [0, 1, 2], flags=0)
    g.set_params(direction=2)
    o = orc.csr_build(50000, src, dst, 0)
    assert np.array_equal(g.bfs(3), orc.bfs_queue(o, 3))


@pytest.mark.parametrize("direction", [0, 1, 2])
def test_directed_rmat_direction_optimising(gb, orc, direction):
    """Directed power-law graph: top-down, bottom-up over the transpose, and
    the switching rule between them all give the oracle's levels."""
    n = 1 << 17
    src, dst = gb.gen_rmat(17, 16, seed=71)
    flags = gb.DEDUP | gb.DROP_SELF_LOOPS
    o = orc.csr_build(n, src, dst, flags)
    g = gb.Graph.from_edges(n, src, dst, flags)
    g.set_params(direction=direction)
    outdeg = np.diff(o.row_offset)
    sources = [int(np.argmax(outdeg)), int(np.flatnonzero(outdeg > 0)[7]), 5]
    for s0 in sources:
        got, st = g.bfs(s0, stats=True)
        want = orc.bfs_queue(o, s0)
        assert np.array_equal(got, want), (direction, s0)
        if direction == 1:
            assert st.bu_levels == 0
    lv, par = g.bfs_parents(sources[0])
    assert np.array_equal(par, orc.min_parents(o, lv))
    gs = g.bfs_multiroot(sources)
    assert gs.shape == (n,)


def test_edge_cases(gb, orc):
    # single vertex, no edges
    g = gb.Graph.from_edges(1, np.array([], np.int32), np.array([], np.int32))
    assert g.bfs(0).tolist() == [0]
    # isolated source and isolated vertices
    g = gb.Graph.from_edges(6, [1, 2], [2, 3])
    assert g.bfs(0).tolist() == [0, -1, -1, -1, -1, -1]
    assert g.bfs(1).tolist() == [-1, 0, 1, 2, -1, -1]
    # self-loops and duplicates only
    g = gb.Graph.from_edges(3, [0, 0, 1, 1], [0, 1, 0, 1], 0)
    assert g.bfs(0).tolist() == [0, 1, -1]
    g = gb.Graph.from_edges(3, [0, 0, 1, 1], [0, 1, 0, 1], gb.UNDIRECTED)
    assert g.m == 2 and g.bfs(1).tolist() == [1, 0, -1]
    # n not a multiple of 32, last vertex reached
    n = 33
    g = gb.Graph.from_edges(n, np.arange(n - 1), np.arange(1, n))
    assert g.bfs(0).tolist() == list(range(n))
    assert g.bfs(n - 1).tolist() == list(range(n - 1, -1, -1))
    # errors
    with pytest.raises(gb.GbfsError) as e:
        g.bfs(n)
    assert e.value.code == gb._lib.ERR_INVALID_ARG
    with pytest.raises(gb.GbfsError) as e:
        g.bfs(-1)
    with pytest.raises(gb.GbfsError) as e:
        gb.Graph.from_edges(4, [0, 5], [1, 2])
    assert e.value.code == gb._lib.ERR_INVALID_ARG
    with pytest.raises(gb.GbfsError):
        gb.Graph.from_csr(np.array([0, 2, 1], np.int32), np.array([1, 0], np.int32))
    with pytest.raises(gb.GbfsError):
        gb.Graph.from_csr(np.array([0, 1, 2], np.int32), np.array([1, 7], np.int32))


def test_device_output_and_input(gb, orc):
    torch = pytest.importorskip("torch")
    src, dst = gb.gen_rmat(14, 16, seed=6)
    o = orc.csr_build(1 << 14, src, dst, orc.UNDIRECTED)
    g = gb.Graph.from_edges(1 << 14, torch.from_numpy(src).cuda(), torch.from_numpy(dst).cuda())
    out = torch.empty(1 << 14, dtype=torch.int32, device="cuda")
    s = int(np.argmax(np.diff(o.row_offset)))
    g.bfs(s, out=out)
    assert np.array_equal(out.cpu().numpy(), orc.bfs_queue(o, s))
    row, col = g.csr()
    g2 = gb.Graph.from_csr(torch.from_numpy(row).cuda(), torch.from_numpy(col).cuda())
    assert np.array_equal(g2.bfs(s), orc.bfs_queue(o, s))


def test_multiroot(gb, orc):
    src, dst = gb.gen_rmat(15, 16, seed=8)
    n = 1 << 15
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    g = gb.Graph.from_edges(n, src, dst)
    roots = [3, 77, 77, 1000, 30000]
    want = None
    for r in roots:
        lv = orc.bfs_queue(o, r)
        lv = np.where(lv < 0, np.iinfo(np.int32).max, lv)
        want = lv if want is None else np.minimum(want, lv)
    want = np.where(want == np.iinfo(np.int32).max, -1, want).astype(np.int32)
    got, st = g.bfs_multiroot(roots, stats=True)
    assert np.array_equal(got, want)
    assert st.vertices_reached == int((want >= 0).sum())


def test_save_load_roundtrip(gb, orc, tmp_path):
    src, dst = gb.gen_er(5000, 20000, seed=9)
    g = gb.Graph.from_edges(5000, src, dst)
    p = tmp_path / "g.csr"
    g.save(str(p))
    g2 = gb.Graph.load(str(p))
    r1, c1 = g.csr()
    r2, c2 = g2.csr()
    assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
    assert np.array_equal(g.bfs(0), g2.bfs(0))


def test_reference_interface_mirror(gb, orc, tmp_path):
    d = load_golden("ref_test2")
    p = tmp_path / "test2.txt"
    p.write_text("\n".join([str(int(d["n"])), str(len(d["src"]))] +
                           [f"{a + 1} {b + 1}" for a, b in zip(d["src"], d["dst"])]))
    graph = gb.csr(str(p))
    assert graph.num_nodes == int(d["n"]) and graph.num_edges == len(d["src"])
    for s, want in zip(d["sources"], d["levels"]):
        b = gb.gpuBFS(graph, int(s))
        assert np.array_equal(b.host_distance, want)
        assert b.iteration == int(want.max()) + 1
        assert b.total_edges_traversed == int((want >= 0).sum()) - 1
        assert b.exec_time > 0


@pytest.mark.parametrize("flags_name", ["UNDIRECTED", "UNDIRECTED|HUB_FIRST", "DIRECTED"])
def test_bottom_up_short_rows(gb, orc, flags_name):
    """Bottom-up on rows of 0, 1, 2 and 3 entries (the first probe reads the
    compact first / second entries, then the rest of the row)."""
    flags = {"UNDIRECTED": gb.UNDIRECTED, "UNDIRECTED|HUB_FIRST": gb.UNDIRECTED | gb.HUB_FIRST,
             "DIRECTED": gb.DEDUP | gb.DROP_SELF_LOOPS}[flags_name]
    rng = np.random.default_rng(77)
    cases = []
    n = 41
    cases.append((n, np.arange(n - 1), np.arange(1, n)))                        # a path (rows of 1-2)
    cases.append((n, np.zeros(n - 1, np.int64), np.arange(1, n)))               # a star
    tri = [(i, i + 1) for i in range(0, 30, 3)] + [(i, i + 2) for i in range(0, 30, 3)]
    cases.append((n, np.array([a for a, _ in tri]), np.array([b for _, b in tri])))  # rows of 2-3, isolated tail
    for _ in range(3):
        m = int(rng.integers(40, 120))
        cases.append((200, rng.integers(0, 200, m), rng.integers(0, 200, m)))
    for nn, s, d in cases:
        s = np.asarray(s, np.int32)
        d = np.asarray(d, np.int32)
        o = orc.csr_build(nn, s, d, flags & 7)
        g = gb.Graph.from_edges(nn, s, d, flags)
        for direction in (0, 2):
            g.set_params(direction=direction)
            for s0 in range(0, nn, 7):
                assert np.array_equal(g.bfs(s0), orc.bfs_queue(o, s0)), (flags_name, direction, s0)


@pytest.mark.parametrize("seed", range(6))
def test_random_graphs_all_paths(gb, orc, seed):
    """Randomised parity sweep over graph shapes (power-law with assorted
    skew, uniform, stars and chains glued together), row layouts (sorted,
    hub-first), directed or symmetrised storage, the three directions and
    small/large deferral thresholds: every level array equals the oracle's."""
    rng = np.random.default_rng(1000 + seed)
    for case in range(5):
        kind = rng.integers(4)
        if kind == 0:
            scale = int(rng.integers(8, 15))
            a_ = float(rng.uniform(0.45, 0.7))
            b_ = c_ = (1 - a_) * 0.4
            src, dst = gb.gen_rmat(scale, int(rng.integers(2, 20)), a_, b_, c_, seed=int(rng.integers(1 << 30)))
            n = 1 << scale
        elif kind == 1:
            n = int(rng.integers(100, 50000))
            src, dst = gb.gen_er(n, int(n * rng.uniform(0.5, 12)), int(rng.integers(1 << 30)))
        elif kind == 2:  # a few stars joined by a chain, plus noise
            n = int(rng.integers(2000, 30000))
            hubs = rng.choice(n, 4, replace=False)
            leaves = [rng.choice(n, int(rng.integers(50, n // 2)), replace=False) for _ in hubs]
            src = np.concatenate([np.full(len(l), h) for h, l in zip(hubs, leaves)] + [hubs[:-1]])
            dst = np.concatenate(leaves + [hubs[1:]])
            noise = rng.integers(0, n, (2, n // 10))
            src, dst = np.concatenate([src, noise[0]]), np.concatenate([dst, noise[1]])
        else:  # long chains with shortcuts (many small levels)
            n = int(rng.integers(1000, 20000))
            perm = rng.permutation(n)
            src, dst = perm[:-1], perm[1:]
            extra = rng.integers(0, n, (2, n // 50))
            src, dst = np.concatenate([src, extra[0]]), np.concatenate([dst, extra[1]])
        src = np.asarray(src, np.int32)
        dst = np.asarray(dst, np.int32)
        base = [gb.UNDIRECTED, gb.DEDUP | gb.DROP_SELF_LOOPS, 0][int(rng.integers(3))]
        flags = base | (gb.HUB_FIRST if rng.random() < 0.5 else 0)
        o = orc.csr_build(n, src, dst, base & 7)
        g = gb.Graph.from_edges(n, src, dst, flags)
        deg = np.diff(o.row_offset)
        cand = np.flatnonzero(deg > 0)
        sources = [int(x) for x in rng.choice(cand if len(cand) else np.arange(n), 3)]
        for direction in (0, 1, 2):
            g.set_params(direction=direction, big_degree=int(rng.choice([32, 256, 4096])))
            for s0 in sources:
                assert np.array_equal(g.bfs(s0), orc.bfs_queue(o, s0)), (seed, case, kind, flags, direction, s0)
        got = g.bfs_multi(sources)  # the 64-lane kernel on the same graph (last direction set)
        for i, s0 in enumerate(sources):
            assert np.array_equal(got[i], orc.bfs_queue(o, s0)), (seed, case, "multi", s0)


def test_hub_first_layout(gb, orc):
    n = 1 << 16
    src, dst = gb.gen_rmat(16, 16, seed=21)
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | gb.HUB_FIRST)
    row, col = g.csr()
    assert sorted_rows_equal(row, col, o.row_offset, o.col_idx)
    deg = np.diff(o.row_offset)
    for r in np.flatnonzero(deg >= 2)[:2000]:
        nb = col[row[r]:row[r + 1]]
        assert deg[nb[0]] == deg[nb].max()
    rng = np.random.default_rng(3)
    for s in rng.choice(np.flatnonzero(deg > 0), 4, replace=False):
        for mode in (0, 1, 2):
            g.set_params(direction=mode)
            assert np.array_equal(g.bfs(int(s)), orc.bfs_queue(o, int(s)))
    # an unsorted symmetric CSR is still recognised as symmetric (bottom-up on)
    g2 = gb.Graph.from_csr(row, col)
    _, st = g2.bfs(int(np.argmax(deg)), stats=True)
    assert st.bu_levels > 0
    # and an unsorted asymmetric one is not
    src2, dst2 = gb.gen_er(4000, 12000, seed=22)
    o2 = orc.csr_build(4000, src2, dst2, 0)
    rev = o2.col_idx.copy()
    for r in range(4000):
        rev[o2.row_offset[r]:o2.row_offset[r + 1]] = rev[o2.row_offset[r]:o2.row_offset[r + 1]][::-1]
    g3 = gb.Graph.from_csr(o2.row_offset.astype(np.int32), rev)
    g3.set_params(direction=2)
    assert np.array_equal(g3.bfs(0), orc.bfs_queue(o2, 0))


@pytest.mark.parametrize("out_kind", ["host", "pinned", "device", "none"])
def test_back_to_back_launches(gb, orc, out_kind):
    """gbfs_bfs_many: one launch per source; host results go through two
    alternating device buffers copied on a second stream."""
    torch = pytest.importorskip("torch")
    n = 1 << 15
    src, dst = gb.gen_rmat(15, 16, seed=61)
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    g = gb.Graph.from_edges(n, src, dst)
    deg = np.diff(o.row_offset)
    sources = [int(x) for x in np.random.default_rng(62).choice(np.flatnonzero(deg > 0), 7, replace=False)]
    sources[3] = int(np.flatnonzero(deg == 0)[0]) if (deg == 0).any() else sources[3]
    if out_kind == "host":
        out = np.full((7, n), 99, np.int32)
    elif out_kind == "pinned":
        out = torch.full((7, n), 99, dtype=torch.int32).pin_memory().numpy()
    elif out_kind == "device":
        out = torch.full((7, n), 99, dtype=torch.int32, device="cuda")
    else:
        out = None
    for _ in range(2):  # the second call reuses the buffers and the copy stream
        got, sts = g.bfs_many(sources, out=out, keep=out is not None)
        assert len(sts) == 7 and all(s.ms > 0 for s in sts)
        for i, s in enumerate(sources):
            want = orc.bfs_queue(o, s)
            assert sts[i].vertices_reached == int((want >= 0).sum())
            if out is not None:
                row = got[i].cpu().numpy() if out_kind == "device" else got[i]
                assert np.array_equal(row, want), (out_kind, i)


def _bounded_degree_graph(n_path: int, n_exp: int, seed: int):
    """A path of n_path vertices (0 .. n_path-1) ending in a random graph of
    degree <= 3 on n_exp vertices (three random perfect matchings): from
    vertex 0 the frontier stays at one vertex for n_path levels, then roughly
    doubles each level."""
    rng = np.random.default_rng(seed)
    src = list(range(n_path - 1))
    dst = list(range(1, n_path))
    src.append(n_path - 1)
    dst.append(n_path)
    for _ in range(3):
        perm = rng.permutation(n_exp) + n_path
        src.extend(perm[0::2][: n_exp // 2].tolist())
        dst.extend(perm[1::2][: n_exp // 2].tolist())
    return n_path + n_exp, np.array(src, np.int32), np.array(dst, np.int32)


@pytest.mark.parametrize("direction", [0, 1])
def test_relaxed_phase_thin_start(gb, orc, direction):
    """The label-correcting phase takes over on a long thin start (level 4
    on) and keeps the search when the frontier explodes into the bounded-
    degree random part (pieces too large to hop: one level per round);
    levels and counts stay exact from several sources, including ones in
    the random part, where the grid kernel steps bottom-up first."""
    n, src, dst = _bounded_degree_graph(40, 1 << 20, 7)
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED)
    assert g.max_degree <= 16
    g.set_params(direction=direction)
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    for s0 in (0, 5, 39, 40 + 12345, n - 1):
        got, st = g.bfs(s0, stats=True)
        assert np.array_equal(got, orc.bfs_queue(o, s0)), s0
        assert st.launches == 2
        assert st.vertices_reached == int((got >= 0).sum())
        assert st.edges_in_component == orc.component_edges(o, got)
        assert st.levels == int(got.max()) + 1
    # back-to-back launches and a device output buffer
    sources = [0, 40 + 7, 3]
    outs, sts = g.bfs_many(sources)
    for i, s0 in enumerate(sources):
        assert np.array_equal(outs[i], orc.bfs_queue(o, s0))


def test_relaxed_phase_multiroot_and_directed(gb, orc):
    side = 300
    src, dst = gb.gen_grid(side, 0.1, 0.001, 8, seed=11)
    n = side * side
    g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED)
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    roots = [0, n - 1, n // 2]
    got = g.bfs_multiroot(roots)
    want = np.min(np.stack([np.where(lv < 0, 1 << 30, lv) for lv in (orc.bfs_queue(o, r) for r in roots)]), axis=0)
    want = np.where(want == 1 << 30, -1, want).astype(np.int32)
    assert np.array_equal(got, want)
    # the grid as stored (directed: in-edges from a transpose for bottom-up)
    gd = gb.Graph.from_edges(n, src, dst, gb.DEDUP | gb.DROP_SELF_LOOPS)
    od = orc.csr_build(n, src, dst, orc.DEDUP | orc.DROP_SELF_LOOPS)
    for s0 in (0, n // 3):
        assert np.array_equal(gd.bfs(s0), orc.bfs_queue(od, s0))


def _ring_with_chords(n: int, chords: int, reach: int, seed: int):
    rng = np.random.default_rng(seed)
    a = np.arange(n, dtype=np.int64)
    c = rng.integers(0, n, chords)
    src = np.concatenate([a, c]).astype(np.int32)
    dst = np.concatenate([(a + 1) % n, (c + rng.integers(2, reach + 1, chords)) % n]).astype(np.int32)
    return src, dst


def test_relaxed_phase_shapes(gb, orc):
    """Label-correcting rounds on shapes that stress them: a ring whose two
    arms meet at the far end (pieces of different CTAs race towards the same
    vertices) with short chords (a CTA can reach a vertex before the piece
    holding its shortest path), a long path (one-vertex frontiers, hundreds
    of rounds), a directed comb whose teeth are sinks (reached vertices of
    out-degree 0) and several components; levels, reached counts, component
    edges and level counts against the oracle."""
    cases = []
    n = 200_000
    s_, d_ = _ring_with_chords(n, 400, 8, 3)
    cases.append(("ring", n, s_, d_, gb.UNDIRECTED, orc.UNDIRECTED, [0, 12345, n - 1]))
    n = 60_000
    s_ = np.arange(n - 1, dtype=np.int32)
    cases.append(("path", n, s_, s_ + 1, gb.UNDIRECTED, orc.UNDIRECTED, [0, n // 2 + 3]))
    k = 30_000  # comb: 0 -> 1 -> ... -> k-1, tooth i -> k + i (a sink)
    spine = np.arange(k - 1, dtype=np.int32)
    teeth = np.arange(k, dtype=np.int32)
    cases.append(("comb", 2 * k, np.concatenate([spine, teeth]), np.concatenate([spine + 1, teeth + k]),
                  gb.DEDUP | gb.DROP_SELF_LOOPS, orc.DEDUP | orc.DROP_SELF_LOOPS, [0, 7, k + 3]))
    side = 500  # two grids and an isolated path
    gs, gd = gb.gen_grid(side, 0.1, 0.001, 8, seed=5)
    m = side * side
    extra = np.arange(2 * m, 2 * m + 999, dtype=np.int32)
    cases.append(("components", 2 * m + 1000, np.concatenate([gs, gs + m, extra]),
                  np.concatenate([gd, gd + m, extra + 1]), gb.UNDIRECTED, orc.UNDIRECTED, [0, m + 17, 2 * m + 5]))
    for name, n, s_, d_, flags, oflags, sources in cases:
        g = gb.Graph.from_edges(n, s_, d_, flags)
        assert g.max_degree <= 16, name
        o = orc.csr_build(n, s_, d_, oflags)
        for s0 in sources:
            got, st = g.bfs(s0, stats=True)
            want = orc.bfs_queue(o, s0)
            assert np.array_equal(got, want), (name, s0)
            assert st.vertices_reached == int((want >= 0).sum()), (name, s0)
            assert st.edges_in_component == orc.component_edges(o, want), (name, s0)
            assert st.levels == int(want.max()) + 1, (name, s0)
            assert st.launches == 2


def _random_small_degree_graph(kind: str, n: int, rng):
    """Seeded graphs whose out-degree stays at most 16 (the label-correcting
    phase's domain): shuffled binary trees, paths with short and long chords,
    unions of random perfect matchings, and grids with random holes."""
    perm = rng.permutation(n).astype(np.int32)
    if kind == "tree":
        i = np.arange(1, n)
        src, dst = perm[i], perm[(i - 1) // 2]
    elif kind == "chords":
        i = np.arange(n - 1)
        c = rng.integers(0, n - 40, n // 50)
        far = rng.integers(0, n, n // 2000)
        src = np.concatenate([perm[i], perm[c], perm[far]])
        dst = np.concatenate([perm[i + 1], perm[c + rng.integers(2, 40, c.size)], perm[rng.integers(0, n, far.size)]])
    elif kind == "matchings":
        m = n - n % 2
        parts = [rng.permutation(m) for _ in range(3)]
        src = np.concatenate([p[0::2] for p in parts]).astype(np.int32)
        dst = np.concatenate([p[1::2] for p in parts]).astype(np.int32)
    else:  # holes
        side = int(np.sqrt(n))
        n = side * side
        v = np.arange(n).reshape(side, side)
        keep = rng.random((side, side)) > 0.15
        h = (keep[:, :-1] & keep[:, 1:])
        w = (keep[:-1, :] & keep[1:, :])
        src = np.concatenate([v[:, :-1][h], v[:-1, :][w]])
        dst = np.concatenate([v[:, 1:][h], v[1:, :][w]])
    return n, np.ascontiguousarray(src, np.int32), np.ascontiguousarray(dst, np.int32)


@pytest.mark.parametrize("wide", [False, True])
def test_relaxed_phase_random_sweep(gb, orc, wide):
    """Twenty seeded graphs of four small-degree families, five sources each
    (the hops, overflowing local frontiers and racing pieces of the
    label-correcting phase at random), int32 and int64 row offsets: levels
    and counts against the oracle."""
    rng = np.random.default_rng(2024)
    for t in range(20):
        kind = ("tree", "chords", "matchings", "holes")[t % 4]
        n, src, dst = _random_small_degree_graph(kind, int(rng.integers(20_000, 200_000)), rng)
        g = gb.Graph.from_edges(n, src, dst, gb.UNDIRECTED | (gb.WIDE_ROWS if wide else 0))
        assert g.max_degree <= 16 and g.wide == wide
        o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
        deg = np.diff(g.row_offsets())
        for s0 in rng.choice(np.flatnonzero(deg > 0), 5, replace=False):
            got, st = g.bfs(int(s0), stats=True)
            want = orc.bfs_queue(o, int(s0))
            assert np.array_equal(got, want), (kind, t, int(s0))
            assert st.vertices_reached == int((want >= 0).sum())
            assert st.edges_in_component == orc.component_edges(o, want)
            assert st.levels == int(want.max()) + 1
