"""Candidate generation on the device (mcbgpu_gen_*, minimumcyclebasis_gb300.devprep)
against the host preparation: the same candidates in the same rank order (roots,
edge offsets, weights, trees), the same sorted coordinate lists (built on the
device), and the same basis from a solver fed device to device; across graph
families (ties resolved by the host's heap searches, every root of the RGG family),
chunk boundaries, the shared-memory and the global tree forms, and the golden
fixtures of the reference."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from minimumcyclebasis_gb300 import (GpuGen, Problem, Solver, grid_graph, planar_chain_graph, prepare_on_device,
                                     random_graph, rgg_graph)
from minimumcyclebasis_gb300._native import MCBError

pytestmark = pytest.mark.gpu

GRAPHS = {
    "random_w1000": lambda: random_graph(700, 1400, 1, 1000, 301),
    "random_w30": lambda: random_graph(700, 1400, 1, 30, 302),
    "planar": lambda: planar_chain_graph(700, 30, 30, 8, 1, 1000, 303),
    "rgg": lambda: rgg_graph(600, 4, 304),
    "grid": lambda: grid_graph(16, 16, 1, 100, 305),
}


def same_as_host(g, chunk=0, solve=True):
    import torch
    torch.cuda.set_device(0)
    p = Problem.from_graph(g).prepare(threads=4)
    d, gen = prepare_on_device(g, threads=4, chunk=chunk, keep_gen=True)
    q = d.problem
    assert q.K == p.K and q.N == p.N
    for x, y in zip(p.candidates(), q.candidates()):
        assert np.array_equal(x, y)
    off, co = gen.fetch_lists()
    hoff, hco = p.cycle_lists()
    assert np.array_equal(off, hoff)
    assert np.array_equal(co, hco)
    if solve:
        d.solver.run()
        sel, tot = d.solver.results()
        s = Solver.from_problem(p)
        s.run()
        want, want_tot = s.results()
        assert np.array_equal(sel, want) and tot == want_tot
        s.close()
    d.solver.close()
    gen.close()
    return d


@pytest.mark.parametrize("family", sorted(GRAPHS))
def test_device_generation_equals_host_preparation(family):
    d = same_as_host(GRAPHS[family]())
    if family == "rgg":
        assert d.tied_roots > 0  # small integer weights: ties, searched on the host


@pytest.mark.parametrize("chunk", [1, 7, 64])
def test_device_generation_chunks(chunk):
    same_as_host(GRAPHS["random_w30"](), chunk=chunk, solve=False)


def test_device_generation_global_tree_form():
    # more than 53248 vertices after contraction: the tree kernel's global form
    g = random_graph(64000, 128000, 1, 1000, 306)
    same_as_host(g, solve=False)


@pytest.mark.parametrize("name", [n for n in golden_names() if not n.startswith("tree_plus")])
def test_device_generation_on_golden_graphs(name):
    fx = load_golden(name)
    import torch
    torch.cuda.set_device(0)
    p = Problem.from_mtx(fx["mtx"])
    try:
        d = prepare_on_device(p, threads=4)
    except MCBError:
        pytest.skip("weights below 1: the device generation needs weights >= 1")
    except ValueError:
        pytest.skip("no search needed")
    d.solver.run()
    sel, tot = d.solver.results()
    assert tot == fx["total_weight"]
    assert np.array_equal(sel, np.array(fx["selected_ranks"], np.int64))
    d.solver.close()


def test_put_trees_rejects_roots_outside_the_chunk():
    import torch
    torch.cuda.set_device(0)
    q = Problem.from_graph(GRAPHS["grid"]()).prepare(threads=2, structure_only=True)
    gen = GpuGen(q, chunk=8)
    gen.trees(0, 8)
    d, ps = q.search_trees(np.array([9], np.int32))
    with pytest.raises(MCBError):
        gen.put_trees(np.array([9], np.int32), d, ps)
    gen.close()
