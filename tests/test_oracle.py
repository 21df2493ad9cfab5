"""The CPU oracle pinned against the reference's own outputs (CPU only)."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import golden_names, load_golden, synthetic_edges


@pytest.mark.parametrize("name", golden_names("ref_"))
def test_oracle_matches_reference_fixture(orc, name):
    d = load_golden(name)
    n = int(d["n"])
    g = orc.csr_build(n, d["src"], d["dst"], 0)
    if "ref_row" in d:  # the reference loader's own CSR, bit for bit
        assert np.array_equal(g.row_offset, d["ref_row"].astype(np.int64))
        assert np.array_equal(g.col_idx, d["ref_col"])
    for s, want in zip(d["sources"], d["levels"]):
        assert np.array_equal(orc.bfs_levelsync(g, int(s)), want), (name, s)
        assert np.array_equal(orc.bfs_queue(g, int(s)), want), (name, s)


@pytest.mark.parametrize("name", golden_names("syn_"))
def test_oracle_matches_reference_synthetic(orc, name):
    d = load_golden(name)
    n, src, dst = synthetic_edges(d)
    h = hashlib.sha256(np.ascontiguousarray(src).tobytes() + np.ascontiguousarray(dst).tobytes()).hexdigest()
    assert h == str(d["edge_sha256"]), "generator output drifted from the golden graph"
    g = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    assert g.m == int(d["m"])
    for s, want in zip(d["sources"], d["levels"]):
        assert np.array_equal(orc.bfs_levelsync(g, int(s)), want)
        assert np.array_equal(orc.bfs_queue(g, int(s)), want)


def test_known_answers(orc):
    """Known answers from the reference fixtures (source = file vertex 1)."""
    want = {
        "ref_test3": [0, 1, 1, 1, 1],
        "ref_test4": [0, 1, 2, 3, 4, -1, -1, -1],
        "ref_test_isolated_node": [0, -1, -1, -1],
        "ref_tree": [0, 1, 1, 2, 2, 2, 2, -1],
    }
    for name, lv in want.items():
        d = load_golden(name)
        g = orc.csr_build(int(d["n"]), d["src"], d["dst"], 0)
        assert orc.bfs_levelsync(g, 0).tolist() == lv
    # graphs/test.txt: vertex 1 -> 2..1029, vertex 2 -> 1030..2058 (a two-level tree)
    d = load_golden("ref_test")
    g = orc.csr_build(int(d["n"]), d["src"], d["dst"], 0)
    lv = orc.bfs_levelsync(g, 0)
    assert np.bincount(lv).tolist() == [1, 1028, 1029]


def test_csr_flags(orc):
    src = np.array([0, 0, 1, 2, 2, 3], np.int32)
    dst = np.array([1, 1, 2, 2, 0, 0], np.int32)
    g = orc.csr_build(4, src, dst, 0)
    assert g.row_offset.tolist() == [0, 2, 3, 5, 6]
    assert g.col_idx.tolist() == [1, 1, 2, 2, 0, 0]
    g = orc.csr_build(4, src, dst, orc.UNDIRECTED)
    assert g.row_offset.tolist() == [0, 3, 5, 7, 8]
    assert g.col_idx.tolist() == [1, 2, 3, 0, 2, 0, 1, 0]
    g = orc.csr_build(4, src, dst, orc.SYMMETRIZE)
    assert g.m == 12
    g = orc.csr_build(4, src, dst, orc.DEDUP)
    assert g.col_idx.tolist() == [1, 2, 0, 2, 0]
    with pytest.raises(ValueError):
        orc.csr_build(3, src, dst, 0)


def test_scan_and_pred(orc):
    x = np.arange(1, 11, dtype=np.int32)
    assert orc.exclusive_scan(x).tolist() == [0, 1, 3, 6, 10, 15, 21, 28, 36, 45]
    d = load_golden("syn_er1000")
    n, src, dst = synthetic_edges(d)
    g = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    lv, pred, te = orc.bfs_levelsync(g, 0, with_pred=True)
    reached = lv >= 0
    assert te == reached.sum() - 1
    for v in np.flatnonzero(reached):
        if v == 0:
            continue
        p = pred[v]
        assert lv[p] == lv[v] - 1
        assert v in g.col_idx[g.row_offset[p]:g.row_offset[p + 1]]


def test_reference_binaries_agree_when_present(orc):
    if not orc.ref_available():
        pytest.skip("reference binaries are built only where the reference is mounted")
    d = load_golden("syn_rmat10")
    n, src, dst = synthetic_edges(d)
    g = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    for s in d["sources"]:
        l9, _ = orc.ref_bfs("c9", int(s), csr=g)
        assert np.array_equal(l9, orc.bfs_levelsync(g, int(s)))


def check_bfs_tree(g, source: int, level: np.ndarray, parent: np.ndarray) -> None:
    """Graph500-style validation of a BFS tree against its level array."""
    n = g.n
    assert parent[source] == -1 and level[source] == 0
    reached = level >= 0
    assert np.all(parent[~reached] == -1)
    v = np.flatnonzero(reached & (np.arange(n) != source))
    p = parent[v]
    assert np.all((p >= 0) & (p < n))
    assert np.all(level[p] == level[v] - 1)
    # every tree edge p -> v exists in the graph
    row, col = g.row_offset, g.col_idx
    for vi, pi in zip(v, p):
        assert vi in col[row[pi]:row[pi + 1]]


@pytest.mark.parametrize("name", golden_names("ref_"))
def test_oracle_parents_on_reference_fixtures(orc, name):
    d = load_golden(name)
    g = orc.csr_build(int(d["n"]), d["src"], d["dst"], 0)
    for s in d["sources"]:
        level, pred = orc.bfs_levelsync_pred(g, int(s))
        mp = orc.min_parents(g, level)
        check_bfs_tree(g, int(s), level, mp)
        check_bfs_tree(g, int(s), level, pred)  # the reference's own predecessors
        # the canonical parent is the smallest valid one
        assert np.all(mp[pred >= 0] <= pred[pred >= 0]) and np.all(mp[pred < 0] == -1)


def test_oracle_parents_small_graph(orc):
    # 0 -> {2, 1}, 1 -> 3, 2 -> 3: vertex 3 has parents 1 and 2 one level up
    g = orc.csr_build(5, np.array([0, 0, 2, 1], np.int32), np.array([2, 1, 3, 3], np.int32), 0)
    level, pred = orc.bfs_levelsync_pred(g, 0)
    assert level.tolist() == [0, 1, 1, 2, -1]
    assert pred[3] == 2  # row 0 lists 2 first, so 2 discovers 3 first
    assert orc.min_parents(g, level).tolist() == [-1, 0, 0, 1, -1]


@pytest.mark.parametrize("name", golden_names("syn_"))
def test_oracle_generators_reproduce_golden_edges(orc, name):
    """The oracle's copy of the seeded generators gives the bytes the golden
    graphs were made from, and the same bytes as the engine's copy."""
    import ast
    import hashlib
    d = load_golden(name)
    kind = str(d["kind"])
    args = ast.literal_eval(str(d["args"]))
    if kind == "er":
        src, dst = orc.gen_er(args["n"], args["pairs"], args["seed"])
    elif kind == "rmat":
        src, dst = orc.gen_rmat(args["scale"], args["edge_factor"], seed=args["seed"])
    else:
        src, dst = orc.gen_grid(args["side"], args["drop"], args["extra"], args["radius"], args["seed"])
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(src, np.int32).tobytes())
    h.update(np.ascontiguousarray(dst, np.int32).tobytes())
    assert h.hexdigest() == str(d["edge_sha256"])
    _, s2, d2 = synthetic_edges(d)
    assert np.array_equal(src, s2) and np.array_equal(dst, d2)
