"""GPU shortest-path trees (mcbgpu_trees_*) against the host's: distances equal
everywhere, the tie flag equal to the rule's, and parent slots equal wherever the
root has no tie; the shared-memory form (n' <= 53248) and the global one; and the
host preparation fed by the GPU trees equals prepare()."""
import numpy as np
import pytest

from minimumcyclebasis_gb300 import GpuTrees, Problem, planar_chain_graph, random_graph
from test_parent_rule import distances_from_parents, rule_parents

pytestmark = pytest.mark.gpu

GRAPHS = {
    "random_w1000": lambda: random_graph(600, 1200, 1, 1000, 101),
    "random_w30": lambda: random_graph(600, 1200, 1, 30, 102),
    "planar": lambda: planar_chain_graph(600, 30, 30, 8, 1, 1000, 103),
}


def check_roots(p, dist, ps, tied, idx):
    rows, cols, w, rev, _ = p.reduced_graph()
    w = w.astype(np.int64)
    _, roots = p.fvs()
    tp = p.tree_parents().reshape(p.F, p.n)
    for i, t in enumerate(idx):
        src = int(roots[t])
        d = distances_from_parents(src, tp[t].astype(np.int64), rows, w, p.n)
        assert np.array_equal(dist[i], d), t
        _, amb = rule_parents(d, rows, cols, w, rev, p.n)
        amb[src] = False
        assert bool(tied[i]) == bool(amb.any()), t
        if not tied[i]:
            assert np.array_equal(ps[i], tp[t]), t


@pytest.mark.parametrize("family", sorted(GRAPHS))
def test_gpu_trees_equal_the_host_trees(family):
    p = Problem.from_graph(GRAPHS[family]()).prepare(threads=4, keep_trees=True)
    gt = GpuTrees.from_problem(p, max_roots=p.F)
    _, roots = p.fvs()
    dist, ps, tied = gt.run(roots)
    check_roots(p, dist, ps, tied, range(p.F))
    gt.close()


def test_gpu_trees_global_form():
    # more than 53248 vertices after contraction: distances in per-CTA global slices
    p = Problem.from_graph(random_graph(66000, 132000, 1, 1000, 104)).prepare(threads=0, keep_trees=True)
    assert p.n > 53248
    gt = GpuTrees.from_problem(p, max_roots=16)
    _, roots = p.fvs()
    idx = list(range(0, p.F, p.F // 16))[:16]
    dist, ps, tied = gt.run(roots[idx])
    check_roots(p, dist, ps, tied, idx)
    gt.close()


@pytest.mark.parametrize("family", sorted(GRAPHS))
def test_preparation_with_gpu_trees_equals_prepare(family):
    g = GRAPHS[family]()
    p = Problem.from_graph(g).prepare(threads=4, keep_trees=True)
    box = {}

    def begin(n, ro, cols, w, rev):
        box["gt"] = GpuTrees(n, ro, cols, w, rev, max_roots=64)

    q = Problem.from_graph(g).prepare_with_trees(lambda r: box["gt"].run(r), chunk=64, threads=4, keep_trees=True,
                                                 begin=begin)
    for x, y in zip(p.candidates(), q.candidates()):
        assert np.array_equal(x, y)
    for x, y in zip(p.cycle_lists(), q.cycle_lists()):
        assert np.array_equal(x, y)
    assert np.array_equal(p.tree_parents(), q.tree_parents())
    assert q.info.trees_supplied > 0
    box["gt"].close()
