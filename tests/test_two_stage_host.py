"""The host half of a device candidate generation: prepare(structure_only) +
search_trees + a candidate test done elsewhere + rank_candidates gives exactly the
candidate list prepare() gives (roots, edge offsets, weights, trees, in rank order).

The candidate test here is a numpy restatement of the one the device runs per root
(include/Dijkstra.h:205-254, is_edge_cycle): a non-tree pair (a, b) is a candidate iff
neither root path holds an FVS vertex with a smaller id than the root and the two
paths meet only at the root; its weight is d(a) + d(b) + w(a, b).  Branch and
blocked flags are computed by pointer jumping up the parent chains, as the device
does.  The same restatement is the oracle of the GPU candidate-test tests."""
import numpy as np
import pytest

from minimumcyclebasis_gb300 import Problem, grid_graph, planar_chain_graph, random_graph, rgg_graph
from minimumcyclebasis_gb300._native import MCBError

GRAPHS = {
    "random_w1000": lambda: random_graph(500, 1000, 1, 1000, 201),
    "random_w3": lambda: random_graph(400, 800, 1, 3, 202),
    "planar": lambda: planar_chain_graph(500, 30, 30, 8, 1, 1000, 203),
    "rgg": lambda: rgg_graph(400, 4, 204),
    "grid": lambda: grid_graph(12, 12, 1, 100, 205),
}


def root_candidates(src, dist, pedge, rows, cols, w, rev, fvs_array, pair_slot):
    """Accepted pairs (ascending pair index) and weights of one root's tree."""
    n = dist.shape[0]
    v = np.arange(n)
    par = np.where(pedge >= 0, rows[np.maximum(pedge, 0)].astype(np.int64), src)
    par[src] = src
    anc = par.copy()
    top = v.copy()
    blk = (fvs_array >= 0) & (v < src)
    blk[src] = False
    while True:
        open_ = anc != src
        if not open_.any():
            break
        a = anc[open_]
        blk_new, top_new, anc_new = blk.copy(), top.copy(), anc.copy()
        blk_new[open_] = blk[open_] | blk[a]
        top_new[open_] = top[a]
        anc_new[open_] = anc[a]
        blk, top, anc = blk_new, top_new, anc_new
    branch = top
    branch[src] = -1
    o = pair_slot.astype(np.int64)
    a, b = rows[o].astype(np.int64), cols[o].astype(np.int64)
    tree_pair = (pedge[b] == o) | (pedge[a] == rev[o].astype(np.int64))
    ok = ~tree_pair & ~blk[a] & ~blk[b] & ((a == src) | (b == src) | (branch[a] != branch[b]))
    k = np.nonzero(ok)[0]
    return k.astype(np.uint32), (dist[a[k]].astype(np.int64) + dist[b[k]] + w[o[k]]).astype(np.int32)


def two_stage(g, threads=2):
    q = Problem.from_graph(g).prepare(threads=threads, structure_only=True)
    rows, cols, w, rev, _ = q.reduced_graph()
    fa, roots = q.fvs()
    pair_slot = q.pairs()
    dist, ps = q.search_trees(np.arange(q.F), threads=threads)
    offs, pis, ws = [0], [], []
    for t in range(q.F):
        k, wk = root_candidates(int(roots[t]), dist[t], ps[t].astype(np.int64), rows, cols, w.astype(np.int64), rev,
                                fa, pair_slot)
        pis.append(k)
        ws.append(wk)
        offs.append(offs[-1] + len(k))
    q.rank_candidates(np.array(offs, np.int64), np.concatenate(pis), np.concatenate(ws), threads=threads)
    return q, dist, ps


@pytest.mark.parametrize("family", sorted(GRAPHS))
def test_two_stage_preparation_equals_prepare(family):
    g = GRAPHS[family]()
    p = Problem.from_graph(g).prepare(threads=2, keep_trees=True)
    q, dist, ps = two_stage(g)
    assert q.K == p.K and q.N == p.N and q.F == p.F
    for x, y in zip(p.candidates(), q.candidates()):
        assert np.array_equal(x, y)
    # the host searches of stage two are the reference's trees
    assert np.array_equal(ps.reshape(-1), p.tree_parents())
    assert q.info.cycle_nnz == 0


def test_rank_candidates_rejects_bad_input_and_misuse():
    g = GRAPHS["grid"]()
    q = Problem.from_graph(g).prepare(threads=2, structure_only=True)
    F = q.F
    offs = np.zeros(F + 1, np.int64)
    offs[1:] = 2
    with pytest.raises(MCBError):  # pairs of a root not ascending
        q.rank_candidates(offs, np.array([5, 3], np.uint32), np.array([1, 1], np.int32))
    p = Problem.from_graph(g).prepare(threads=2)
    with pytest.raises(MCBError):  # only after a structure-only preparation
        p.rank_candidates(np.zeros(p.F + 1, np.int64), np.zeros(0, np.uint32), np.zeros(0, np.int32))
    with pytest.raises(MCBError):  # FVS index out of range
        q.search_trees(np.array([F], np.int32))
