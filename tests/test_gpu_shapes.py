"""Search shapes of the blocked run: every candidate shape, forced for a whole solve,
gives the reference's basis, and a tuning run (shapes taking turns group by group)
gives the same basis and support vectors as the default shape, before and after the
per-segment choice is applied.  Bit-exact."""
import numpy as np
import pytest

from conftest import load_golden
from minimumcyclebasis_gb300 import Problem, Solver, planar_chain_graph, random_graph

pytestmark = pytest.mark.gpu


def test_candidate_shapes_are_listed():
    p = Problem.from_mtx(load_golden("grid8x8_s3")["mtx"]).prepare(threads=4)
    s = Solver.from_problem(p)
    info = s.shapes()
    assert len(info["candidates"]) >= 2 and info["segment_shape"] == [0] * Solver.SHAPE_SEGMENTS
    for c in info["candidates"]:
        assert 1 <= c["win_early"] <= 32 and 1 <= c["win_mid"] <= 32 and 1 <= c["win_tail"] <= 32
        assert 1 <= c["lmax"] <= 8 and 0 <= c["rank_early"] <= c["rank_tail"] <= 64
    s.close()


@pytest.mark.parametrize("name", ["grid32x32_s1", "rand1000_s5", "rand2000_w20_s11"])
def test_every_forced_shape_gives_the_reference_basis(name):
    fx = load_golden(name)
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=4)
    s = Solver.from_problem(p)
    for k in range(len(s.shapes()["candidates"])):
        s.set_shape(k)
        s.reset()
        s.run()
        sel, tot = s.results()
        assert sel.tolist() == fx["selected_ranks"], k
        assert tot == fx["total_weight"], k
    s.close()


@pytest.mark.parametrize("family", ["random", "planar"])
def test_tuning_run_and_tuned_shapes_give_the_default_result(family):
    if family == "random":
        g = random_graph(13000, 26000, 1, 1000, 5)
    else:
        g = planar_chain_graph(12500, 30, 30, 8, 1, 1000, 3)
    p = Problem.from_graph(g).prepare(threads=8)
    assert p.N > 64 * 2 * 4 * 4 * 6  # enough two-block groups of every shape in every segment
    s = Solver.from_problem(p)
    s.run()
    want, want_w = s.results()
    rows = sorted({0, p.N // 3, p.N // 2, p.N - 1})
    want_S = [s.support_vector(j) for j in rows]
    info = s.tune()
    got, got_w = s.results()
    assert np.array_equal(got, want) and got_w == want_w
    for j, v in zip(rows, want_S):
        assert np.array_equal(s.support_vector(j), v), j
    ms = np.array(info["ms_per_block"])
    assert ms.shape == (Solver.SHAPE_SEGMENTS, len(info["candidates"])) and (ms > 0).all()
    assert all(0 <= k < len(info["candidates"]) for k in info["segment_shape"])
    assert s.shapes()["segment_shape"] == info["segment_shape"]
    s.reset()
    s.run()
    got, got_w = s.results()
    assert np.array_equal(got, want) and got_w == want_w
    for j, v in zip(rows, want_S):
        assert np.array_equal(s.support_vector(j), v), j
    s.close()
