"""Seeded synthetic inputs: determinism and the shapes the benchmark configs name."""
import numpy as np

from minimumcyclebasis_gb300 import (Problem, batch_graphs, block_tree_graph, grid_graph, planar_chain_graph,
                                     random_graph, rgg_graph)


def components(g):
    """Number of connected components (union-find over the edge list)."""
    parent = np.arange(g.nodes)

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for a, b in zip(g.u.tolist(), g.v.tolist()):
        ra, rb = find(a), find(b)
        if ra != rb:
            parent[ra] = rb
    return len({find(x) for x in range(g.nodes)})


def simple(g):
    keys = np.minimum(g.u, g.v).astype(np.int64) * g.nodes + np.maximum(g.u, g.v)
    return bool(np.all(g.u != g.v)) and np.unique(keys).size == g.m


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
    assert components(g) == 1 and simple(g)
    p = Problem.from_graph(g).prepare(threads=2, cycle_lists=False)
    assert p.N == g.m - g.nodes + 1


def test_planar_chains_shape():
    # config 5 at full scale: ~230k triangulated points, 30% of edges deleted, chains
    g = planar_chain_graph(230000, 30, 30, 8, 1, 1000, 1)
    assert 800_000 < g.nodes < 1_000_000
    assert 240_000 < g.m - g.nodes + 1 < 265_000  # cycle-space dimension ~250k
    assert g.w.min() >= 1 and g.w.max() <= 1000
    h = planar_chain_graph(2000, 30, 30, 8, 1, 1000, 4)
    assert components(h) == 1 and simple(h)
    assert np.array_equal(h.u, planar_chain_graph(2000, 30, 30, 8, 1, 1000, 4).u)
    deg = np.bincount(np.concatenate([h.u, h.v]), minlength=h.nodes)
    assert (deg == 2).sum() > h.nodes // 3  # the subdivided chains
    p = Problem.from_graph(h).prepare(threads=2, cycle_lists=False)
    assert p.N == h.m - h.nodes + 1 and p.info.nodes_removed > 0


def test_block_tree_shape():
    g = block_tree_graph(2000, 50, 150, 2.5, 5.0, 1, 255, 1)
    assert 150_000 < g.nodes < 250_000 and g.w.max() <= 255
    h = block_tree_graph(40, 20, 60, 2.5, 5.0, 1, 255, 3)
    assert components(h) == 1 and simple(h)
    p = Problem.from_graph(h).prepare(threads=2, cycle_lists=False)
    assert p.N == h.m - h.nodes + 1


def test_batch_graphs():
    bs = batch_graphs(64, 50, 5000, 2.5, 5.0, 1, 255, 1)
    n = np.array([g.nodes for g in bs])
    assert n.min() >= 50 and n.max() <= 5000 and len(set(n.tolist())) > 40
    for g in bs[:8]:
        assert components(g) == 1 and simple(g) and g.w.max() <= 255
        assert 2.4 <= 2 * g.m / g.nodes <= 5.1
    again = batch_graphs(64, 50, 5000, 2.5, 5.0, 1, 255, 1)
    assert all(np.array_equal(a.w, b.w) for a, b in zip(bs, again))


def test_mtx_round_trip(tmp_path):
    g = random_graph(200, 400, 1, 50, 9)
    path = str(tmp_path / "g.mtx")
    g.write_mtx(path)
    a = Problem.from_mtx(path).prepare(threads=1)
    b = Problem.from_graph(g).prepare(threads=1)
    for x, y in zip(a.candidates(), b.candidates()):
        assert np.array_equal(x, y)
