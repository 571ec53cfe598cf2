"""Host preparation vs the reference's own outputs (golden vectors made by
tests/golden/make_golden.py from the reference binaries)."""
import hashlib

import numpy as np
import pytest

from conftest import golden_names, load_golden
from minimumcyclebasis_gb300 import Problem


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()


@pytest.mark.parametrize("name", golden_names())
def test_prepare_matches_reference(name):
    fx = load_golden(name)
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=2)
    i = p.info
    G = fx["G"]
    assert i.nodes == G["nodes"]
    assert i.edges2 == G["edges2"]
    assert i.nodes_removed == G["nodes_removed"]
    assert i.reduced_nodes == G["reduced_nodes"]
    assert i.reduced_edges2 == G["reduced_edges2"]
    assert i.fvs_size == G["fvs_size"]
    assert i.num_coords == G["num_coords"]
    assert i.num_candidates == G["num_candidates"]
    _, fv = p.fvs()
    assert fv.tolist() == fx["fvs_vertices"]
    ce, ec = p.coords()
    assert ce.tolist() == fx["coord_edges"]
    root, edge, w, tree = p.candidates()
    assert sha(root) == fx["candidates_sha256"]["root"]
    assert sha(edge) == fx["candidates_sha256"]["edge"]
    assert sha(w) == fx["candidates_sha256"]["weight"]
    if "candidates" in fx:
        assert root.tolist() == fx["candidates"]["root"]
        assert edge.tolist() == fx["candidates"]["edge"]
        assert w.tolist() == fx["candidates"]["weight"]
    # the stats CSV of the reference CPU driver agrees on the counts
    csv = fx["mcb_cpu_csv"]
    assert int(csv["Fvs_size"]) == i.fvs_size
    assert int(csv["Initial_Cycles"]) == i.num_candidates
    assert int(csv["Node_removed"]) == i.nodes_removed


@pytest.mark.parametrize("name", golden_names())
def test_cycle_lists_are_sorted_coordinate_sets(name):
    fx = load_golden(name)
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=2, keep_trees=True)
    off, co = p.cycle_lists()
    assert off[0] == 0 and off[-1] == co.shape[0]
    assert np.all(np.diff(off) >= 0)
    assert co.size == 0 or (co.min() >= 0 and co.max() < p.N)
    # strictly ascending inside each list
    d = np.diff(co)
    starts = np.zeros(co.shape[0], bool)
    starts[off[:-1][off[:-1] < co.shape[0]]] = True
    assert np.all((d > 0) | starts[1:])
    # lists equal the reference's get_cycle_vector (include/cycles.h:144-195) on a sample
    import oracle
    rng = np.random.default_rng(0)
    for r in rng.choice(p.K, size=min(p.K, 25), replace=False):
        words = oracle.cycle_vector(p, int(r))
        bits = [c for c in range(p.N) if (int(words[c >> 6]) >> (c & 63)) & 1]
        assert bits == co[off[r]:off[r + 1]].tolist()


def test_threads_do_not_change_the_order():
    fx = load_golden("rand2000_w20_s11")
    a = Problem.from_mtx(fx["mtx"]).prepare(threads=1)
    b = Problem.from_mtx(fx["mtx"]).prepare(threads=8)
    for x, y in zip(a.candidates(), b.candidates()):
        assert np.array_equal(x, y)
    for x, y in zip(a.cycle_lists(), b.cycle_lists()):
        assert np.array_equal(x, y)


def test_reference_layout_is_level_ordered():
    fx = load_golden("grid8x8_s3")
    p = Problem.from_mtx(fx["mtx"]).prepare(ref_layout=True, keep_trees=True)
    lv, pp, eo, ni = p.ref_layout()
    n, F = p.n, p.F
    rows, cols, _, _, _ = p.reduced_graph()
    tp = p.tree_parents()
    for t in range(F):
        L = lv[t * (n + 1):(t + 1) * (n + 1)]
        P = pp[t * n:(t + 1) * n]
        E = eo[t * n:(t + 1) * n]
        NI = ni[t * n:(t + 1) * n]
        assert L[0] == 0 and L[1] == 1 and L[n] == n
        assert E[0] == -1
        for pos in range(1, n):
            assert P[pos] < pos
            child = cols[E[pos]]
            assert NI[child] == pos
            assert tp[t * n + child] == E[pos]


@pytest.mark.parametrize("family", ["random_w1000", "random_w30", "planar", "batch_w255"])
def test_fast_and_exact_tree_searches_agree(family):
    # the level-ordered layout is built from the reference's heap search alone;
    # without it the radix-queue search runs (falling back where two parents tie)
    from minimumcyclebasis_gb300 import batch_graphs, planar_chain_graph, random_graph
    g = {"random_w1000": lambda: random_graph(3000, 6000, 1, 1000, 21),
         "random_w30": lambda: random_graph(3000, 6000, 1, 30, 22),
         "planar": lambda: planar_chain_graph(2500, 30, 30, 8, 1, 1000, 23),
         "batch_w255": lambda: max(batch_graphs(24, nmin=1000, nmax=3000, seed=24), key=lambda x: x.nodes)}[family]()
    exact = Problem.from_graph(g).prepare(threads=4, keep_trees=True, ref_layout=True)
    fast = Problem.from_graph(g).prepare(threads=4, keep_trees=True)
    assert exact.F > 64  # past the first roots, where the fast search is always tried
    for x, y in zip(exact.candidates(), fast.candidates()):
        assert np.array_equal(x, y)
    for x, y in zip(exact.cycle_lists(), fast.cycle_lists()):
        assert np.array_equal(x, y)
    assert np.array_equal(exact.tree_parents(), fast.tree_parents())


def test_prepare_many_equals_prepare_and_flags_failures():
    from minimumcyclebasis_gb300 import batch_graphs, prepare_many
    from minimumcyclebasis_gb300._native import MCBError
    from minimumcyclebasis_gb300.host import Graph
    graphs = batch_graphs(20, nmin=50, nmax=800, seed=31)
    one = [Problem.from_graph(g).prepare(threads=2) for g in graphs]
    many = prepare_many([Problem.from_graph(g) for g in graphs], threads=4)
    for a, b in zip(one, many):
        assert b.prepared and a.info.single_cycle == b.info.single_cycle
        if a.info.single_cycle:
            continue
        for x, y in zip(a.candidates(), b.candidates()):
            assert np.array_equal(x, y)
        for x, y in zip(a.cycle_lists(), b.cycle_lists()):
            assert np.array_equal(x, y)
    # a triangle and a K4 with no edge between them: the spanning tree fails
    bad = Graph(7, np.array([0, 1, 2, 3, 3, 3, 4, 4, 5], np.int32), np.array([1, 2, 0, 4, 5, 6, 5, 6, 6], np.int32),
                np.ones(9, np.int32))
    probs = [Problem.from_graph(graphs[0]), Problem.from_graph(bad), Problem.from_graph(graphs[1])]
    with pytest.raises(MCBError):
        prepare_many(probs, threads=2)
    assert probs[0].prepared and not probs[1].prepared and probs[2].prepared


@pytest.mark.parametrize("name", golden_names())
def test_reference_basis_is_gf2_independent(name):
    # re-verification by elimination: the reference's N selected cycles have rank N;
    # a basis with one cycle listed twice has rank N - 1
    fx = load_golden(name)
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=2)
    if p.info.single_cycle:
        pytest.skip("one cycle: nothing to eliminate")
    sel = np.array(fx["selected_ranks"], np.int64)
    assert len(sel) == p.N and p.gf2_rank(sel, threads=2) == p.N
    if p.N > 1:
        dup = sel.copy()
        dup[-1] = dup[0]
        assert p.gf2_rank(dup, threads=2) == p.N - 1


def test_gf2_rank_of_oracle_bases_and_bad_arguments():
    import oracle
    from minimumcyclebasis_gb300 import random_graph
    from minimumcyclebasis_gb300._native import MCBError
    for seed in (61, 62, 63):
        p = Problem.from_graph(random_graph(400, 900, 1, 30, seed)).prepare(threads=2, keep_trees=True)
        sel, _, _ = oracle.solve(p, threads=2)
        assert p.gf2_rank(sel) == p.N
        # the first N candidates in rank order are not in general a basis
        assert p.gf2_rank(np.arange(p.N)) <= p.N
    with pytest.raises(MCBError):
        p.gf2_rank([p.info.num_candidates])  # past the last candidate
    q = Problem.from_graph(random_graph(50, 80, 1, 9, 64))
    with pytest.raises(MCBError):
        q.gf2_rank([0])  # not prepared
