"""Biconnected components against the reference's own tools: bicc_decomposition (main.sh's
settings: no degree pruning, bridges dropped) and Relabeller, built from its sources by
oracle/Makefile, then its host library and de Pina loop (oracle/_ref/ref_dump) on every
relabelled component file.  bcc_split must produce, for every component, the graph the
reference's per-component run reads: the same candidate list (root, edge offset,
weight, in rank order) and the same selected cycles, not only the same weights.
Components are matched by their edge sets in input vertex ids.  Skipped where the
reference's tools are not built."""
import glob
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from minimumcyclebasis_gb300 import Graph, Problem, bcc_split, block_tree_graph, random_graph

REF = os.path.join(ROOT, "oracle", "_ref")
TOOLS = [os.path.join(REF, x) for x in ("bicc_decomposition", "Relabeller", "ref_dump")]

pytestmark = pytest.mark.skipif(not all(os.path.exists(t) for t in TOOLS),
                                reason="the reference's bicc tools (oracle/_ref) are not built here")


def read_mtx_edges(path):
    with open(path) as f:
        lines = [ln for ln in f if not ln.startswith("%")]
    n, _, m = map(int, lines[0].split())
    e = np.array([list(map(int, ln.split())) for ln in lines[1:1 + m]], np.int64).reshape(-1, 3)
    return n, e


def ref_dump(path):
    r = subprocess.run([TOOLS[2], path, "2", "-1", "noE"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    C = np.array([[int(x) for x in ln.split()[1:]] for ln in r.stdout.splitlines() if ln.startswith("C ")],
                 np.int64).reshape(-1, 4)
    S = np.array([[int(x) for x in ln.split()[1:]] for ln in r.stdout.splitlines() if ln.startswith("S ")],
                 np.int64).reshape(-1, 5)
    W = [int(ln.split()[1]) for ln in r.stdout.splitlines() if ln.startswith("W ")]
    return C, S, W[-1] if W else None


def reference_components(tmp_path, mtx, nodes):
    out = tmp_path / "bicc"
    out.mkdir()
    r = subprocess.run(["bash", "-c", "ulimit -s unlimited; %s %s %s/ 0 %d 0 1" % (TOOLS[0], mtx, out, nodes)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    comps = {}
    for f in glob.glob(str(out / "*.mtx")):
        _, e = read_mtx_edges(f)  # input ids, 1-based
        key = frozenset((int(a) - 1, int(b) - 1) for a, b, _ in e)
        rel = str(tmp_path / ("r_" + os.path.basename(f)))
        rr = subprocess.run([TOOLS[1], f, rel, "1"], capture_output=True, text=True, timeout=600)
        assert rr.returncode == 0, rr.stderr[-2000:]
        comps[key] = rel
    return comps


GRAPHS = {
    "block_tree": lambda: block_tree_graph(25, 20, 60, seed=71),
    "block_tree_w3": lambda: block_tree_graph(25, 20, 60, wlo=1, whi=3, seed=72),
    "random_sparse": lambda: random_graph(400, 470, 1, 50, 73),
}


@pytest.mark.parametrize("name", sorted(GRAPHS) + ["golden_blocktree12_s2"])
def test_components_equal_the_reference_tools(tmp_path, name):
    import oracle
    if name.startswith("golden_"):
        mtx = os.path.join(GOLDEN, name[len("golden_"):] + ".mtx")
        n, e = read_mtx_edges(mtx)
        g = Graph(n, (e[:, 0] - 1).astype(np.int32), (e[:, 1] - 1).astype(np.int32), e[:, 2].astype(np.int32))
    else:
        g = GRAPHS[name]()
        mtx = str(tmp_path / "g.mtx")
        g.write_mtx(mtx)
    ref = reference_components(tmp_path, mtx, g.nodes)
    ours = bcc_split(g, with_ids=True)
    assert len(ours) == len(ref)
    checked = 0
    for cg, ids in ours:
        key = frozenset((int(ids[a]), int(ids[b])) for a, b in zip(cg.u.tolist(), cg.v.tolist()))
        assert key in ref, "a component the reference's tool does not produce"
        C, S, W = ref_dump(ref[key])
        p = Problem.from_graph(cg).prepare(threads=2, keep_trees=True)
        if p.info.single_cycle:
            assert W == int(cg.w.astype(np.int64).sum())
            continue
        root, edge, w, _ = p.candidates()
        assert np.array_equal(C[:, 1], root) and np.array_equal(C[:, 2], edge) and np.array_equal(C[:, 3], w)
        sel, tot, _ = oracle.solve(p, threads=2)
        assert np.array_equal(S[:, 1], sel), "the selected cycles differ"
        assert tot == W
        checked += 1
    assert checked > 0
