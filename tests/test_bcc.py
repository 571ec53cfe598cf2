"""In-process biconnected split (mcbh_bcc_split): the partition of the edges, and the
decomposition the reference's per-component driver loop relies on (bicc/,
main.sh:19-32): the minimum cycle basis of a graph is the union of its biconnected
components' bases, so their weights add up."""
import numpy as np
import pytest
from conftest import load_golden

import oracle
from minimumcyclebasis_gb300 import (Problem, bcc_split, block_tree_graph, planar_chain_graph, random_graph,
                                     rgg_graph)
from minimumcyclebasis_gb300.host import host_lib, ptr


def partition(g):
    comp = np.empty(g.m, np.int32)
    nc = host_lib().mcbh_bcc_split(g.nodes, g.m, ptr(g.u), ptr(g.v), ptr(comp))
    assert nc > 0
    parts = {}
    for i, c in enumerate(comp.tolist()):
        parts.setdefault(c, []).append(i)
    firsts = [min(p) for _, p in sorted(parts.items())]
    assert firsts == sorted(firsts)  # numbered in order of their first edge
    return sorted(sorted(p) for p in parts.values())


GRAPHS = [
    lambda: block_tree_graph(30, 10, 40, 2.5, 5.0, 1, 255, 3),
    lambda: random_graph(300, 330, 1, 9, 4),
    lambda: planar_chain_graph(400, 30, 30, 8, 1, 100, 2),
    lambda: rgg_graph(300, 3, 7),
]


@pytest.mark.parametrize("make", GRAPHS)
def test_partition_matches_networkx(make):
    nx = pytest.importorskip("networkx")
    g = make()
    G = nx.Graph()
    G.add_nodes_from(range(g.nodes))
    G.add_edges_from(zip(g.u.tolist(), g.v.tolist()))
    eid = {(min(a, b), max(a, b)): i for i, (a, b) in enumerate(zip(g.u.tolist(), g.v.tolist()))}
    theirs = sorted(sorted(eid[(min(a, b), max(a, b))] for a, b in c) for c in nx.biconnected_component_edges(G))
    assert partition(g) == theirs


def test_parallel_edges_and_self_loops():
    # a 2-cycle of parallel edges, a self-loop, a bridge and a triangle
    u = np.array([0, 0, 1, 2, 3, 4, 5], np.int32)
    v = np.array([1, 1, 1, 3, 4, 5, 3], np.int32)
    comp = np.empty(7, np.int32)
    nc = host_lib().mcbh_bcc_split(6, 7, ptr(u), ptr(v), ptr(comp))
    parts = sorted(sorted(np.flatnonzero(comp == c).tolist()) for c in range(nc))
    # parallel pair {0,1}, self-loop {2}, bridge 2-3 {3}, triangle 3-4-5 {4,5,6}
    assert [0, 1] in parts and [2] in parts and [4, 5, 6] in parts and [3] in parts


def basis_weight(g):
    """Minimum cycle basis weight by the oracle (a ring is its own basis, as in
    mcb/mcb_cycle_deg_two_remove.cpp:104-111)."""
    p = Problem.from_graph(g).prepare(threads=2, keep_trees=True)
    if p.info.single_cycle:
        return int(g.w.astype(np.int64).sum())
    return int(oracle.solve(p, threads=2)[1])


@pytest.mark.parametrize("make", GRAPHS[:3])
def test_component_weights_add_up(make):
    g = make()
    comps = bcc_split(g)
    assert sum(c.m - c.nodes + 1 for c in comps) == g.m - g.nodes + 1
    assert sum(basis_weight(c) for c in comps) == basis_weight(g)


def test_block_tree_golden_weight():
    # the reference's whole-graph basis weight equals the sum over the components
    fx = load_golden("blocktree12_s2")
    g = block_tree_graph(*fx["args"])
    assert sum(basis_weight(c) for c in bcc_split(g)) == fx["total_weight"]
