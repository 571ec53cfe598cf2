"""The distance phase of the GPU tree kernel (csrc/gpu/mcbgpu_trees.cu), modelled on
the CPU: rounds that take lo = the smallest distance among dirty vertices and relax
every dirty vertex nearer than lo + delta (delta = the mean weight) converge to the
exact distances of the reference's trees within n + 1 rounds.  This model relaxes a
round's vertices with the distances they had when the round began, one of the
orders the kernel's threads may take."""
import numpy as np
import pytest

from minimumcyclebasis_gb300 import Problem, planar_chain_graph, random_graph
from test_parent_rule import distances_from_parents


def bucket_rounds(n, ro, cols, w, src, delta):
    big = np.iinfo(np.int64).max // 4
    dist = np.full(n, big, np.int64)
    dist[src] = 0
    dirty = np.zeros(n, bool)
    dirty[src] = True
    deg = np.diff(ro.astype(np.int64))
    rounds = 0
    while dirty.any():
        rounds += 1
        assert rounds <= n + 1
        dv = np.flatnonzero(dirty)
        lo = dist[dv].min()
        act = dv[dist[dv] < lo + delta]
        dirty[act] = False
        cnt = deg[act]
        first = np.repeat(ro[act].astype(np.int64), cnt)
        idx = first + np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
        before = dist.copy()
        np.minimum.at(dist, cols[idx].astype(np.int64), np.repeat(dist[act], cnt) + w[idx])
        dirty |= dist < before
    return dist, rounds


@pytest.mark.parametrize("family", ["random", "planar", "random_w3"])
def test_bucket_rounds_reach_the_reference_distances(family):
    g = {"random": lambda: random_graph(1500, 3000, 1, 1000, 91),
         "planar": lambda: planar_chain_graph(1500, 30, 30, 8, 1, 1000, 92),
         "random_w3": lambda: random_graph(1500, 3000, 1, 3, 93)}[family]()
    p = Problem.from_graph(g).prepare(threads=2, keep_trees=True)
    rows, cols, w, rev, ro = p.reduced_graph()
    w = w.astype(np.int64)
    _, roots = p.fvs()
    tp = p.tree_parents().reshape(p.F, p.n)
    delta = int(np.ceil(w.mean()))
    for t in range(0, p.F, max(1, p.F // 12)):
        src = int(roots[t])
        d, rounds = bucket_rounds(p.n, ro, cols, w, src, delta)
        assert np.array_equal(d, distances_from_parents(src, tp[t].astype(np.int64), rows, w, p.n))
        assert rounds <= p.n + 1
