"""Full-size runs (the 50k-node random graph of the plain-GPU benchmark shape, and the
1M-vertex planar-chain graph of the scale configuration) checked
through size-independent properties: the blocked and per-iteration device forms
agree, the selections are distinct, the weights add up, and the de Pina invariants
<C_i, S_j> = 0 (i < j) and <C_j, S_j> = 1 hold on sampled pairs."""
import numpy as np
import pytest

from minimumcyclebasis_gb300 import Problem, Solver, random_graph

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big():
    g = random_graph(50000, 100000, 1, 1000, 1)
    p = Problem.from_graph(g).prepare(threads=0)
    return p


def dot(words, coords):
    return int(sum((int(words[c >> 6]) >> (c & 63)) & 1 for c in np.asarray(coords).tolist()) & 1)


def test_blocked_equals_plain_and_invariants(big):
    p = big
    s = Solver.from_problem(p)
    s.run()
    sel, tot = s.results()
    assert (sel >= 0).all() and np.unique(sel).size == p.N
    _, _, w, _ = p.candidates()
    assert tot == int(w[sel].astype(np.int64).sum())
    off, co = p.cycle_lists()
    rng = np.random.default_rng(3)
    for j in rng.choice(p.N, 12, replace=False).tolist():
        Sj = s.support_vector(j)
        cj = co[off[sel[j]]:off[sel[j] + 1]]
        assert dot(Sj, cj) == 1
        for i in (rng.choice(j, min(j, 20), replace=False).tolist() if j > 0 else []):
            ci = co[off[sel[i]]:off[sel[i] + 1]]
            assert dot(Sj, ci) == 0
    s.reset()
    s.run_plain()
    sel2, tot2 = s.results()
    assert np.array_equal(sel, sel2) and tot == tot2


@pytest.fixture(scope="module")
def scale5():
    """The scale configuration's graph (1M vertices, planar-like with degree-two
    chains, seed 1), prepared with the device candidate generation."""
    import torch

    from minimumcyclebasis_gb300 import planar_chain_graph, prepare_on_device
    torch.cuda.set_device(0)
    d, gen = prepare_on_device(planar_chain_graph(263000, 30, 30, 8, 1, 1000, 1), keep_gen=True)
    yield d, gen
    d.solver.close()
    gen.close()


def test_scale_configuration_blocked_run(scale5):
    # the whole solve: the pinned total weight, distinct selections, the device
    # certificate (rank N of N), and the de Pina invariants on sampled pairs
    d, gen = scale5
    p, s = d.problem, d.solver
    assert (p.n, p.F, p.N, p.K) == (241787, 79113, 288051, 8437310)
    s.run()
    sel, tot = s.results()
    assert tot == 1008336977
    assert (sel >= 0).all() and np.unique(sel).size == p.N
    _, _, w, _ = p.candidates()
    assert tot == int(w[sel].astype(np.int64).sum())
    assert s.verify() == {"rank": p.N, "violations": 0, "first": None}
    off, co = gen.fetch_lists()
    rng = np.random.default_rng(5)
    for j in rng.choice(p.N, 8, replace=False).tolist():
        Sj = s.support_vector(j)
        assert dot(Sj, co[off[sel[j]]:off[sel[j] + 1]]) == 1
        for i in (rng.choice(j, min(j, 16), replace=False).tolist() if j > 0 else []):
            assert dot(Sj, co[off[sel[i]]:off[sel[i] + 1]]) == 0


def test_scale_configuration_blocked_equals_per_iteration_on_a_prefix(scale5):
    # the first 5 blocks (320 iterations) of the blocked run against the reference
    # loop's shape on the device (select + update per iteration), then a window deep
    # in the solve reached by the blocked run
    d, _ = scale5
    p, s = d.problem, d.solver
    s.reset()
    s.run(320)
    blk, _ = s.results(320)
    s.reset()
    for e in range(320):
        s.select(e, fetch=False)
        s.update(e)
    per, _ = s.results(320)
    assert np.array_equal(blk, per)
    e0 = (p.N // 2) // 64 * 64
    s.reset()
    s.run(e0 + 192)
    blk2, _ = s.results(e0 + 192)
    s.reset()
    s.run(e0)
    for e in range(e0, e0 + 192):
        s.select(e, fetch=False)
        s.update(e)
    per2, _ = s.results(e0 + 192)
    assert np.array_equal(blk2[e0:], per2[e0:])
