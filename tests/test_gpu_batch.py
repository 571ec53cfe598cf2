"""GPU parity of the batched solver (one persistent launch, one CTA per problem):
every problem's selected ranks and weight equal the reference's
golden vectors, the oracle's, or the single-problem blocked solver's, bit for bit."""
import numpy as np
import pytest

import oracle
from conftest import golden_names, load_golden
from minimumcyclebasis_gb300 import (BatchSolver, Problem, Solver, batch_graphs, bcc_split, block_tree_graph,
                                     random_graph, solve_batch)

pytestmark = pytest.mark.gpu


def items_of(probs):
    out = []
    for p in probs:
        _, _, w, _ = p.candidates()
        off, co = p.cycle_lists()
        out.append((p.N, w, off, co))
    return out


def test_golden_fixtures_in_one_batch():
    fxs, probs = [], []
    for name in golden_names():
        fx = load_golden(name)
        p = Problem.from_mtx(fx["mtx"]).prepare(threads=4)
        if p.info.single_cycle:
            continue
        fxs.append(fx)
        probs.append(p)
    b = BatchSolver.from_problems(probs)
    b.run()
    sels, tots = b.results()
    for fx, sel, tot in zip(fxs, sels, tots):
        assert sel.tolist() == fx["selected_ranks"], fx["mtx"]
        assert tot == fx["total_weight"]
    assert b.launches >= 1
    b.close()


def test_sizes_around_the_block_width_against_oracle():
    probs, refs = [], []
    for N in [1, 2, 63, 64, 65, 127, 128, 129, 300]:
        g = random_graph(150, 150 + N - 1, 1, 30, 100 + N)
        p = Problem.from_graph(g).prepare(threads=4, keep_trees=True)
        assert p.N == N
        refs.append(oracle.solve(p, threads=4))
        probs.append(p)
    b = BatchSolver.from_problems(probs)
    b.run()
    sels, tots = b.results()
    for (ref, tot, _), sel, t in zip(refs, sels, tots):
        assert sel.tolist() == ref.tolist()
        assert t == tot
    # finished rows hold S_e as it was at iteration e
    p = probs[-1]
    for e in (0, 63, 64, 200, p.N - 1):
        assert np.array_equal(b.support_vector(len(probs) - 1, e), oracle.support_vector_at(p, e)), e
    b.close()


def test_batched_configuration_family_against_single_solver():
    # graphs of the batched configuration's distribution (node counts log-uniform,
    # average degree uniform in [2.5, 5], weights in [1, 255]), fewer and smaller
    graphs = batch_graphs(48, nmin=50, nmax=1500, seed=5)
    probs = [Problem.from_graph(g).prepare(threads=8) for g in graphs]
    probs = [p for p in probs if not p.info.single_cycle and p.N > 0]
    b = BatchSolver.from_problems(probs)
    b.run()
    sels, tots = b.results()
    for p, sel, tot in zip(probs, sels, tots):
        s = Solver.from_problem(p)
        s.run()
        ref, t = s.results()
        s.close()
        assert np.array_equal(sel, ref) and tot == t
    b.close()


def test_size_class_boundaries_against_single_solver():
    probs = []
    for i, N in enumerate([1024, 1025, 4096, 4097, 64, 2000]):
        n = 2 * N
        g = random_graph(n, n + N - 1, 1, 1000, 40 + i)
        probs.append(Problem.from_graph(g).prepare(threads=8))
        assert probs[-1].N == N
    sels, tots = solve_batch(items_of(probs))
    for p, sel, tot in zip(probs, sels, tots):
        s = Solver.from_problem(p)
        s.run()
        ref, t = s.results()
        s.close()
        assert np.array_equal(sel, ref) and tot == t


def test_block_tree_components_add_up_to_the_reference_weight():
    fx = load_golden("blocktree12_s2")
    g = block_tree_graph(*fx["args"])
    total, probs = 0, []
    for c in bcc_split(g):
        p = Problem.from_graph(c).prepare(threads=4)
        if p.info.single_cycle:
            total += int(c.w.astype(np.int64).sum())
        elif p.N > 0:
            probs.append(p)
    _, tots = solve_batch(items_of(probs))
    assert total + int(tots.sum()) == fx["total_weight"]


def test_malformed_and_deficient_problems_are_flagged_per_problem():
    from minimumcyclebasis_gb300._native import MCBError
    good = Problem.from_mtx(load_golden("grid8x8_s3")["mtx"]).prepare(threads=2)
    gi = items_of([good])[0]
    bad_order = (4, np.array([3, 4], np.int32), np.array([0, 2, 3], np.int64), np.array([2, 1, 0], np.int32))
    deficient = (2, np.array([5], np.int32), np.array([0, 1], np.int64), np.array([0], np.int32))
    b = BatchSolver([gi, bad_order, deficient, gi])
    b.run()
    st = b.status()
    assert st[0] == 0 and st[3] == 0 and st[1] != 0 and st[2] != 0
    with pytest.raises(MCBError):
        b.results()
    b.close()


def test_too_large_problem_is_rejected():
    from minimumcyclebasis_gb300._native import MCBError
    n = BatchSolver.max_coords() + 1
    with pytest.raises(MCBError):
        BatchSolver([(n, np.array([1], np.int32), np.array([0, 1], np.int64), np.array([0], np.int32))])


def test_per_problem_profile():
    graphs = batch_graphs(6, nmin=100, nmax=800, seed=9)
    probs = [Problem.from_graph(g).prepare(threads=4) for g in graphs]
    probs = [p for p in probs if not p.info.single_cycle and p.N > 0]
    b = BatchSolver.from_problems(probs)
    b.set_profiling(True)
    b.run()
    pr = b.profile()
    assert pr.shape == (len(probs), 13)
    assert (pr[:, 0] > 0).all() and (pr[:, 2] > 0).all()  # wall time, scan cycles
    assert (pr[:, 6] > 0).all()  # candidates scanned
    # bytes walked: at least the offsets of every candidate of the first scan round of
    # every block, at most every list read in full by every block
    for p, walked in zip(probs, pr[:, 12]):
        off = p.cycle_lists()[0]
        blocks = (p.N + 63) // 64
        assert 16 * min(p.K, 64) <= walked <= blocks * (16 * p.K + 4 * int(off[-1]) + 4 * 8 * p.K)
    assert (pr[:, 9] >= np.array([(p.N + 63) // 64 for p in probs])).all()  # at least one pivot round per block
    b.set_profiling(False)
    sels, tots = b.results()
    for p, sel, tot in zip(probs, sels, tots):
        s = Solver.from_problem(p)
        s.run()
        ref, t = s.results()
        s.close()
        assert np.array_equal(sel, ref) and tot == t
    b.close()
