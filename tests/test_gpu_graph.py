"""The CUDA-graph form of a complete solve (reset + blocked run captured once,
replayed after) gives the stream form's basis and support vectors, replay after
replay, after a new upload into the same handle, and for a prefix of iterations.
Bit-exact."""
import numpy as np
import pytest

import oracle
from conftest import load_golden
from minimumcyclebasis_gb300 import Problem, Solver, random_graph

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["grid32x32_s1", "rand1000_s5", "rand2000_w20_s11"])
def test_graph_replays_give_the_reference_basis(name):
    fx = load_golden(name)
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=4)
    s = Solver.from_problem(p)
    for _ in range(3):  # capture + replay, then two replays
        s.run_graph()
        sel, tot = s.results()
        assert sel.tolist() == fx["selected_ranks"]
        assert tot == fx["total_weight"]
    s.close()


def test_graph_matches_stream_form_with_support_vectors_and_reupload():
    g = random_graph(6000, 12000, 1, 1000, 9)
    p = Problem.from_graph(g).prepare(threads=8)
    s = Solver.from_problem(p)
    s.run()
    want, want_w = s.results()
    rows = sorted({1, p.N // 3, p.N - 1})
    want_S = [s.support_vector(j) for j in rows]
    s.run_graph()
    s.run_graph()
    got, got_w = s.results()
    assert np.array_equal(got, want) and got_w == want_w
    for j, v in zip(rows, want_S):
        assert np.array_equal(s.support_vector(j), v), j
    # a new upload of the same lists into the same buffers: the graph solves it again
    s.upload()
    s.run_graph()
    got, got_w = s.results()
    assert np.array_equal(got, want) and got_w == want_w
    # the stream form after replays starts from its own reset
    s.reset()
    s.run()
    got, got_w = s.results()
    assert np.array_equal(got, want) and got_w == want_w
    s.close()


@pytest.mark.parametrize("iters", [64, 130])
def test_graph_prefix_of_iterations(iters):
    fx = load_golden("rand1000_s5")
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=4, keep_trees=True)
    s = Solver.from_problem(p)
    s.run_graph(max_iterations=iters)
    sel, _ = s.results(iters)
    assert sel.tolist() == fx["selected_ranks"][:iters]
    for e in sorted({0, iters // 2, iters}):
        assert np.array_equal(s.support_vector(e), oracle.support_vector_at(p, e)), e
    s.close()
