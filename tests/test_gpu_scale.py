"""Full-size runs (50k-node random graph, the plain-GPU benchmark shape) checked
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
