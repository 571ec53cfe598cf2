"""mcbh_prepare_with_trees: per-root trees from an outside supplier (the GPU's, in the
driver) are checked before use, and the result is always prepare()'s.  Here the
supplier offers the reference's own trees (from a normal preparation), corrupted
trees, skipped roots, or fails; candidates, cycle lists and tree parents must equal
the host's own, and info.trees_supplied must count exactly the trees that pass."""
import numpy as np
import pytest

from minimumcyclebasis_gb300 import Problem, planar_chain_graph, random_graph
from minimumcyclebasis_gb300._native import MCBError
from test_parent_rule import distances_from_parents, rule_parents

GRAPHS = {
    "random_w1000": lambda: random_graph(600, 1200, 1, 1000, 81),
    "random_w30": lambda: random_graph(600, 1200, 1, 30, 82),
    "planar": lambda: planar_chain_graph(600, 30, 30, 8, 1, 1000, 83),
}


def reference_trees(g):
    """The host's own preparation and, per root, its tree as (distances, parent slots),
    plus the number of roots whose tree has a tie (two equally near parents)."""
    p = Problem.from_graph(g).prepare(threads=2, keep_trees=True)
    rows, cols, w, rev, _ = p.reduced_graph()
    w = w.astype(np.int64)
    _, roots = p.fvs()
    tp = p.tree_parents().reshape(p.F, p.n)
    trees, tied = {}, 0
    for t in range(p.F):
        src = int(roots[t])
        pe = tp[t].astype(np.int64)
        d = distances_from_parents(src, pe, rows, w, p.n)
        _, amb = rule_parents(d, rows, cols, w, rev, p.n)
        amb[src] = False
        tied += bool(amb.any())
        trees[src] = (d.astype(np.int32), tp[t].astype(np.int32))
    return p, trees, tied


def same_result(a, b):
    for x, y in zip(a.candidates(), b.candidates()):
        assert np.array_equal(x, y)
    for x, y in zip(a.cycle_lists(), b.cycle_lists()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.tree_parents(), b.tree_parents())


def supplier(trees, change=None, skip=None):
    def f(roots):
        d = np.stack([trees[int(r)][0] for r in roots]).copy()
        ps = np.stack([trees[int(r)][1] for r in roots]).copy()
        sk = np.zeros(len(roots), np.uint8)
        for i, r in enumerate(roots):
            if change is not None:
                change(int(r), d[i], ps[i])
            if skip is not None and skip(int(r)):
                sk[i] = 1
        return d, ps, sk
    return f


@pytest.mark.parametrize("family", sorted(GRAPHS))
def test_supplied_reference_trees_are_adopted_except_at_ties(family):
    g = GRAPHS[family]()
    p, trees, tied = reference_trees(g)
    seen = {}
    q = Problem.from_graph(g).prepare_with_trees(supplier(trees), chunk=37, threads=2, keep_trees=True,
                                                 begin=lambda n, ro, cols, w, rev: seen.update(n=n, slots=len(cols)))
    same_result(p, q)
    assert seen == {"n": p.n, "slots": p.info.reduced_edges2}
    assert q.info.trees_supplied == p.F - tied
    if family == "random_w30":
        assert tied > 0


def test_corrupted_and_skipped_trees_are_searched_on_the_host():
    g = GRAPHS["random_w1000"]()
    p, trees, tied = reference_trees(g)
    assert tied == 0
    roots = sorted(trees)
    bad = set(roots[::3])
    rng = np.random.default_rng(5)

    def corrupt(r, d, ps):
        if r not in bad:
            return
        v = int(rng.integers(0, len(d)))
        while v == r:
            v = int(rng.integers(0, len(d)))
        kind = roots.index(r) % 3
        if kind == 0:
            d[v] += 1  # a distance off by one
        elif kind == 1:
            ps[v] = (ps[v] + 1) % p.info.reduced_edges2  # a parent slot that does not enter v
        else:
            d[:] = d * 2  # consistent-looking but not shortest
    skipped = set(roots[1::5]) - bad
    q = Problem.from_graph(g).prepare_with_trees(supplier(trees, corrupt, lambda r: r in skipped), chunk=50,
                                                 threads=3, keep_trees=True)
    same_result(p, q)
    assert q.info.trees_supplied == p.F - len(bad) - len(skipped)


def test_supplier_failure_and_unused_supplier():
    g = GRAPHS["planar"]()
    p, trees, _ = reference_trees(g)

    def failing(roots):
        raise RuntimeError("no trees")
    f = Problem.from_graph(g)
    with pytest.raises(MCBError, match="-7"):
        f.prepare_with_trees(failing, threads=2)
    with pytest.raises(MCBError, match="-5"):  # no second preparation on a problem left half-prepared
        f.prepare(threads=2)
    # the level-ordered layout follows the heap's settle order: the supplier is not asked
    asked = []
    q = Problem.from_graph(g).prepare_with_trees(lambda r: asked.append(1), threads=2, keep_trees=True,
                                                 ref_layout=True)
    assert not asked and q.info.trees_supplied == 0
    same_result(p, q)
    # weights of 0: neither the radix search nor supplied trees apply
    z = random_graph(300, 600, 0, 3, 84)
    a = Problem.from_graph(z).prepare(threads=2, keep_trees=True)
    b = Problem.from_graph(z).prepare_with_trees(lambda r: asked.append(1), threads=2, keep_trees=True)
    assert not asked and b.info.trees_supplied == 0
    same_result(a, b)


@pytest.mark.parametrize("chunk", [1, 0, 10 ** 6])
def test_chunk_sizes(chunk):
    # one root per call, all at once (0), and a chunk larger than the root count
    g = GRAPHS["random_w1000"]()
    p, trees, tied = reference_trees(g)
    calls = []

    def f(roots):
        calls.append(len(roots))
        return supplier(trees)(roots)
    q = Problem.from_graph(g).prepare_with_trees(f, chunk=chunk, threads=4, keep_trees=True)
    same_result(p, q)
    assert q.info.trees_supplied == p.F - tied
    assert sum(calls) == p.F and max(calls) == (1 if chunk == 1 else p.F)


def test_trusted_supplier_skips_only_the_shortest_path_checks():
    # trust: the reference's trees are adopted (ties included: the rule is not checked),
    # and trees whose structure is broken are still searched on the host
    g = GRAPHS["random_w30"]()
    p, trees, tied = reference_trees(g)
    assert tied > 0
    q = Problem.from_graph(g).prepare_with_trees(supplier(trees), chunk=40, threads=2, keep_trees=True, trust=True)
    same_result(p, q)
    assert q.info.trees_supplied == p.F
    roots = sorted(trees)
    broken = set(roots[::4])

    def corrupt(r, d, ps):
        if r in broken:
            v = next(x for x in range(len(d)) if x != r)
            ps[v] = -1  # a vertex without a parent
    q2 = Problem.from_graph(g).prepare_with_trees(supplier(trees, corrupt), chunk=40, threads=2, keep_trees=True,
                                                  trust=True)
    same_result(p, q2)
    assert q2.info.trees_supplied == p.F - len(broken)


def hop_tree(src, rows, cols, w, rev, n):
    """A breadth-first tree by hop count from `src` (parent slots entering each
    vertex), with distances summed along its parent chains: a consistent tree that is
    not, in general, a tree of shortest paths."""
    ro = np.zeros(n + 1, np.int64)
    np.add.at(ro, rows.astype(np.int64) + 1, 1)
    ro = np.cumsum(ro)
    d = np.full(n, -1, np.int64)
    pe = np.full(n, -1, np.int64)
    d[src] = 0
    frontier = [src]
    while frontier:
        nxt = []
        for x in frontier:
            for o in range(ro[x], ro[x + 1]):
                c = int(cols[o])
                if d[c] < 0:
                    d[c] = d[x] + int(w[o])
                    pe[c] = o
                    nxt.append(c)
        frontier = nxt
    return d.astype(np.int32), pe.astype(np.int32)


def test_trusted_supplier_still_rejects_trees_that_are_not_shortest():
    # a supplier that stopped short of the true distances hands over a consistent
    # tree (distances add up along every parent chain) that is not a shortest-path
    # tree; even when trusted, such a tree is searched again on the host
    g = GRAPHS["random_w1000"]()
    p, trees, _ = reference_trees(g)
    rows, cols, w, rev, _ = p.reduced_graph()
    roots = sorted(trees)
    bad = {}
    for r in roots[::3]:
        d, pe = hop_tree(r, rows, cols, w.astype(np.int64), rev, p.n)
        if not np.array_equal(d, trees[r][0]):
            bad[r] = (d, pe)
    assert bad

    def swap(r, d, ps):
        if r in bad:
            d[:], ps[:] = bad[r]
    q = Problem.from_graph(g).prepare_with_trees(supplier(trees, swap), chunk=40, threads=2, keep_trees=True,
                                                 trust=True)
    same_result(p, q)
    assert q.info.trees_supplied == p.F - len(bad)
