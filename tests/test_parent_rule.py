"""The parent rule that lets any exact shortest-path search reproduce the reference's
trees (the basis of a GPU form of candidate generation): with weights of at least 1,
the parent the reference's heap search keeps for a vertex c is, among c's
shortest-path neighbours x (d[x] + w(x, c) = d[c]), the nearest one, entered through
its first slot to c of that weight; only where two distinct neighbours tie at that
nearest distance does the heap's order decide.  Checked on every root of several
graphs against the tree parents of the reference's own search (include/Dijkstra.h:78-124),
from distances alone."""
import numpy as np
import pytest

from minimumcyclebasis_gb300 import Problem, planar_chain_graph, random_graph


def distances_from_parents(src, pedge, rows, w, n):
    """d[v] = d[parent] + w(parent slot), evaluated along each vertex's parent chain."""
    d = np.full(n, -1, np.int64)
    d[src] = 0
    for v in range(n):
        chain = []
        x = v
        while d[x] < 0:
            chain.append(x)
            x = int(rows[pedge[x]])
        for y in reversed(chain):
            d[y] = d[int(rows[pedge[y]])] + int(w[pedge[y]])
    return d


def rule_parents(d, rows, cols, w, rev, n):
    """(parent slot by the rule, ambiguous flag) for every vertex, from distances."""
    c, x = rows.astype(np.int64), cols.astype(np.int64)
    opt = d[x] + w == d[c]  # slot c->x: x is a shortest-path neighbour of c
    oc, ox, orev = c[opt], x[opt], rev[opt].astype(np.int64)
    # per vertex c: the nearest such neighbour, then its first slot to c
    order = np.lexsort((orev, d[ox], oc))
    oc, ox, orev = oc[order], ox[order], orev[order]
    first = np.ones(len(oc), bool)
    first[1:] = oc[1:] != oc[:-1]
    pedge = np.full(n, -1, np.int64)
    pedge[oc[first]] = orev[first]
    # ambiguous: a different neighbour at the same (nearest) distance
    near = d[ox[first]]
    start = np.flatnonzero(first)
    amb = np.zeros(n, bool)
    nxt = start + 1
    ok = nxt < len(oc)
    same_c = np.zeros(len(start), bool)
    same_c[ok] = oc[nxt[ok]] == oc[start[ok]]
    # neighbours of the same c come sorted by distance, so the second distinct
    # neighbour at the nearest distance (if any) is found by scanning that run
    for k in np.flatnonzero(same_c):
        i = start[k] + 1
        while i < len(oc) and oc[i] == oc[start[k]] and d[ox[i]] == near[k]:
            if ox[i] != ox[start[k]]:
                amb[oc[start[k]]] = True
                break
            i += 1
    return pedge, amb


@pytest.mark.parametrize("family", ["random_w1000", "random_w30", "planar"])
def test_parents_follow_from_distances_except_at_ties(family):
    g = {"random_w1000": lambda: random_graph(700, 1400, 1, 1000, 71),
         "random_w30": lambda: random_graph(700, 1400, 1, 30, 72),
         "planar": lambda: planar_chain_graph(700, 30, 30, 8, 1, 1000, 73)}[family]()
    p = Problem.from_graph(g).prepare(threads=2, keep_trees=True, ref_layout=True)  # the heap search on every root
    rows, cols, w, rev, _ = p.reduced_graph()
    w = w.astype(np.int64)
    n, F = p.n, p.F
    _, roots = p.fvs()
    tp = p.tree_parents().reshape(F, n)
    roots_with_ties = 0
    for t in range(F):
        src = int(roots[t])
        pedge = tp[t].astype(np.int64)
        d = distances_from_parents(src, pedge, rows, w, n)
        rp, amb = rule_parents(d, rows, cols, w, rev, n)
        rp[src] = -1
        amb[src] = False
        assert np.array_equal(rp[~amb], pedge[~amb]), (family, t)
        roots_with_ties += bool(amb.any())
        # at a tie the reference's parent is one of the tied nearest neighbours
        for v in np.flatnonzero(amb):
            par = int(rows[pedge[v]])
            assert d[par] + w[pedge[v]] == d[v] and d[par] == d[int(rows[rp[v]])]
    assert roots_with_ties < F
