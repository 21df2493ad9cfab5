"""Generate tests/golden/*.npz from the reference's own CPU BFS.

Run where a checkout of the reference project is available, named by
GBFS_REFERENCE_ROOT (or --reference <dir>); it builds
oracle/_ref/ref_c9 and ref_c10 from the reference's unmodified sources
(oracle/Makefile), then records:

  * text fixtures of the reference (graphs/*.txt and the migration copies):
    the reference loader's own CSR (csc(file,1,1) of 2D Partition) and the
    levels of its level-synchronous CPU BFS (2D Partition/src/cpuBFS.cpp)
    from several sources, cross-checked against the queue BFS of the
    migration path (include/cpu/cpuBFS.cpp);
  * wiki-Vote (migration/GPU_Graphs/graphs/wiki-Vote.txt), whose header
    declares 7115 vertices while its ids reach 8297 (the reference loaders
    would index out of bounds), re-headed with n = largest id;
  * seeded synthetic graphs (ER, RMAT, perturbed grid, built undirected by
    the oracle's CSR builder) injected into the reference BFS objects.

The .npz files hold only inputs and outputs; nothing at test time reads the
reference.  Usage:
  GBFS_REFERENCE_ROOT=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent

TEXT_FIXTURES = {
    "ref_test": "graphs/test.txt",
    "ref_test2": "graphs/test2.txt",
    "ref_test3": "graphs/test3.txt",
    "ref_test4": "graphs/test4.txt",
    "ref_test_isolated_node": "graphs/test_isolated_node.txt",
    "ref_tree": "graphs/tree.txt",
    "ref_mig_tree": "1D Partition/migration/GPU_Graphs/graphs/tree.txt",
    "ref_mig_test_isolated_node": "1D Partition/migration/GPU_Graphs/graphs/test_isolated_node.txt",
}

# name -> (generator, args, flags, sources)
SYNTHETIC = {
    "er1000": ("er", dict(n=1000, pairs=3000, seed=7), [0, 1, 17, 999]),
    "er16": ("er", dict(n=65536, pairs=262144, seed=1), [0]),
    "rmat10": ("rmat", dict(scale=10, edge_factor=16, seed=3), None),
    "grid32": ("grid", dict(side=32, drop=0.1, extra=0.001, radius=8, seed=5), [0, 513, 1023]),
}


def parse_text(path: Path) -> tuple[int, np.ndarray, np.ndarray]:
    """The reference text format, 1-based ids -> 0-based (csc.cpp:14-25)."""
    toks = path.read_text().split()
    n = int(toks[0])
    pairs = np.array(toks[2:], dtype=np.int64).reshape(-1, 2) - 1
    return n, pairs[:, 0].astype(np.int32), pairs[:, 1].astype(np.int32)


def ref_csr(path: Path) -> tuple[np.ndarray, np.ndarray]:
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "g.csr")
        subprocess.run([str(oracle.REF_DIR / "ref_c9"), "csrdump", str(path), out], check=True)
        b = open(out, "rb").read()
    n = int(np.frombuffer(b[:4], np.int32)[0])
    a = np.frombuffer(b[12:], np.int32)
    return a[: n + 1].copy(), a[n + 1:].copy()


def ref_levels_text(path: Path, sources) -> np.ndarray:
    rows = []
    for s in sources:
        l9, _ = oracle.ref_bfs("c9", int(s), text=str(path))
        l10, _ = oracle.ref_bfs("c10", int(s), text=str(path))
        assert (l9 == l10).all(), f"reference BFS variants disagree on {path} source {s}"
        rows.append(l9)
    return np.stack(rows)


def ref_levels_csr(g: oracle.CSR, sources) -> np.ndarray:
    rows = []
    for s in sources:
        l9, _ = oracle.ref_bfs("c9", int(s), csr=g)
        l10, _ = oracle.ref_bfs("c10", int(s), csr=g)
        assert (l9 == l10).all(), f"reference BFS variants disagree (source {s})"
        rows.append(l9)
    return np.stack(rows)


def edge_hash(src: np.ndarray, dst: np.ndarray) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(src, np.int32).tobytes())
    h.update(np.ascontiguousarray(dst, np.int32).tobytes())
    return h.hexdigest()


def main() -> None:
    global REF
    if "--reference" in sys.argv:
        os.environ["GBFS_REFERENCE_ROOT"] = sys.argv[sys.argv.index("--reference") + 1]
    if not os.environ.get("GBFS_REFERENCE_ROOT"):
        sys.exit("name the reference checkout: GBFS_REFERENCE_ROOT=<dir> or --reference <dir>")
    REF = Path(os.environ["GBFS_REFERENCE_ROOT"])
    if not REF.exists():
        sys.exit(f"reference not found at {REF}")
    oracle.REFERENCE_ROOT = REF
    oracle.build(ref=True)
    for name, rel in TEXT_FIXTURES.items():
        path = REF / rel
        n, src, dst = parse_text(path)
        row, col = ref_csr(path)
        sources = list(range(n)) if n <= 16 else [0, 1, n // 2, n - 1]
        levels = ref_levels_text(path, sources)
        np.savez_compressed(OUT / f"{name}.npz", n=n, src=src, dst=dst, flags=0, sources=np.array(sources, np.int32),
                            levels=levels, ref_row=row, ref_col=col, origin=rel)
        print(name, n, len(src), levels.shape)

    # wiki-Vote: header fixed to the largest id so the reference loader stays in bounds
    rel = "1D Partition/migration/GPU_Graphs/graphs/wiki-Vote.txt"
    toks = (REF / rel).read_text().split()
    pairs = np.array(toks[2:], dtype=np.int64).reshape(-1, 2)
    n = int(pairs.max())
    with tempfile.TemporaryDirectory() as td:
        fixed = Path(td) / "wiki.txt"
        fixed.write_text(f"{n}\n{len(pairs)}\n" + "\n".join(f"{a} {b}" for a, b in pairs) + "\n")
        src = (pairs[:, 0] - 1).astype(np.int32)
        dst = (pairs[:, 1] - 1).astype(np.int32)
        deg = np.bincount(src, minlength=n)
        sources = [0, int(np.argmax(deg)), 29, 5000]
        levels = ref_levels_text(fixed, sources)
    np.savez_compressed(OUT / "ref_wiki_vote.npz", n=n, src=src, dst=dst, flags=0,
                        sources=np.array(sources, np.int32), levels=levels, origin=rel)
    print("ref_wiki_vote", n, len(src), levels.shape)

    gb = oracle  # the seeded generators (host code, linked into the oracle library)
    for name, (kind, args, sources) in SYNTHETIC.items():
        if kind == "er":
            src, dst = gb.gen_er(args["n"], args["pairs"], args["seed"])
            n = args["n"]
        elif kind == "rmat":
            src, dst = gb.gen_rmat(args["scale"], args["edge_factor"], seed=args["seed"])
            n = 1 << args["scale"]
        else:
            src, dst = gb.gen_grid(args["side"], args["drop"], args["extra"], args["radius"], args["seed"])
            n = args["side"] ** 2
        g = oracle.csr_build(n, src, dst, oracle.UNDIRECTED)
        if sources is None:
            deg = g.degrees()
            rng = np.random.default_rng(11)
            sources = [int(x) for x in rng.choice(np.flatnonzero(deg > 0), 4, replace=False)]
        levels = ref_levels_csr(g, sources)
        np.savez_compressed(OUT / f"syn_{name}.npz", n=n, kind=kind, args=repr(args), edge_sha256=edge_hash(src, dst),
                            flags=oracle.UNDIRECTED, sources=np.array(sources, np.int32), levels=levels,
                            m=g.m)
        print("syn_" + name, n, g.m, levels.shape)


if __name__ == "__main__":
    main()
