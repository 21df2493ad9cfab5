"""GPU parity: canonical BFS-tree parents against the oracle, plus tree validation."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_names, load_golden, synthetic_edges
from test_oracle import check_bfs_tree

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_names("ref_"))
def test_parents_reference_fixtures(gb, orc, name):
    d = load_golden(name)
    n = int(d["n"])
    o = orc.csr_build(n, d["src"], d["dst"], 0)
    g = gb.Graph.from_edges(n, d["src"], d["dst"], 0)
    for s in d["sources"]:
        lv, par = g.bfs_parents(int(s))
        assert np.array_equal(lv, d["levels"][list(d["sources"]).index(s)])
        assert np.array_equal(par, orc.min_parents(o, lv))
        check_bfs_tree(o, int(s), lv, par)


@pytest.mark.parametrize("name", golden_names("syn_"))
def test_parents_synthetic(gb, orc, name):
    d = load_golden(name)
    n, src, dst = synthetic_edges(d)
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    for flags in (gb.UNDIRECTED, gb.UNDIRECTED | gb.HUB_FIRST):
        g = gb.Graph.from_edges(n, src, dst, flags)
        for s in d["sources"][:3]:
            lv, par = g.bfs_parents(int(s))
            want_lv = orc.bfs_queue(o, int(s))
            assert np.array_equal(lv, want_lv)
            assert np.array_equal(par, orc.min_parents(o, want_lv))


@pytest.mark.parametrize("kind", ["rmat", "er_directed", "grid"])
def test_parents_generated(gb, orc, kind):
    if kind == "rmat":
        n = 1 << 16
        src, dst = gb.gen_rmat(16, 16, seed=41)
        flags = gb.UNDIRECTED
    elif kind == "er_directed":
        n = 30000
        src, dst = gb.gen_er(n, 120000, seed=42)
        flags = 0
    else:
        side = 300
        n = side * side
        src, dst = gb.gen_grid(side, 0.1, 0.001, 8, seed=43)
        flags = gb.UNDIRECTED
    o = orc.csr_build(n, src, dst, flags)
    g = gb.Graph.from_edges(n, src, dst, flags)
    deg = np.diff(o.row_offset)
    for s in [int(np.argmax(deg)), int(np.flatnonzero(deg > 0)[0])]:
        lv, par = g.bfs_parents(s)
        want_lv = orc.bfs_queue(o, s)
        assert np.array_equal(lv, want_lv)
        want = orc.min_parents(o, want_lv)
        assert np.array_equal(par, want)
        if kind != "rmat":
            check_bfs_tree(o, s, lv, par)


def test_parents_device_buffers_and_isolated_source(gb, orc):
    torch = pytest.importorskip("torch")
    n = 5000
    src, dst = gb.gen_er(n, 8000, seed=44)
    o = orc.csr_build(n, src, dst, orc.UNDIRECTED)
    g = gb.Graph.from_edges(n, src, dst)
    lv = torch.empty(n, dtype=torch.int32, device="cuda")
    par = torch.empty(n, dtype=torch.int32, device="cuda")
    g.bfs_parents(7, levels=lv, parents=par)
    want_lv = orc.bfs_queue(o, 7)
    assert np.array_equal(lv.cpu().numpy(), want_lv)
    assert np.array_equal(par.cpu().numpy(), orc.min_parents(o, want_lv))
    iso = int(np.flatnonzero(np.diff(o.row_offset) == 0)[0])
    lv2, par2 = g.bfs_parents(iso)
    assert lv2[iso] == 0 and np.all(par2 == -1)
