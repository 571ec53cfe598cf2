"""The CPU oracle vs the reference's selected basis (golden vectors)."""
import numpy as np
import pytest

import oracle
from conftest import golden_names, load_golden
from minimumcyclebasis_gb300 import Problem


@pytest.mark.parametrize("name", golden_names())
def test_oracle_selects_the_reference_basis(name):
    fx = load_golden(name)
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=2, keep_trees=True)
    sel, tot, _ = oracle.solve(p, threads=2)
    assert sel.tolist() == fx["selected_ranks"]
    assert tot == fx["total_weight"]
    assert tot == int(fx["mcb_cpu_csv"]["Total_Weight"])
    _, _, w, _ = p.candidates()
    assert w[sel].tolist() == fx["selected_weights"]


@pytest.mark.parametrize("name", ["grid8x8_s3", "rand300_s0", "rgg500_s3", "grid12x12_w5_s9"])
def test_no_contraction_pipeline_matches_cpu_baseline_weight(name):
    # mcb_cpu_baseline (mcb/mcb_cycle.cpp) skips the chain contraction; the minimum
    # basis weight is the same either way.
    fx = load_golden(name)
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=2, keep_trees=True, contract_chains=False)
    sel, tot, _ = oracle.solve(p, threads=2)
    assert tot == int(fx["mcb_cpu_baseline_csv"]["Total_Weight"])
    assert int(fx["mcb_cpu_baseline_csv"]["Initial_Cycles"]) == p.K
    assert int(fx["mcb_cpu_baseline_csv"]["Fvs_size"]) == p.F


def test_oracle_prefix_is_a_prefix():
    fx = load_golden("rand1000_s5")
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=2, keep_trees=True)
    sel, _, _ = oracle.solve(p, threads=2, max_iter=100)
    assert sel.tolist() == fx["selected_ranks"][:100]


def test_oracle_labels_match_a_direct_walk():
    fx = load_golden("grid8x8_s3")
    p = Problem.from_mtx(fx["mtx"]).prepare(keep_trees=True)
    rng = np.random.default_rng(1)
    S = rng.integers(0, 2**63, size=(p.N + 63) // 64, dtype=np.int64).astype(np.uint64)
    lab = oracle.labels(p, S)
    rows, cols, _, _, _ = p.reduced_graph()
    _, ec = p.coords()
    tp = p.tree_parents()
    n = p.n
    for t in range(p.F):
        for v in range(n):
            par = 0
            x = v
            while tp[t * n + x] >= 0:
                e = int(tp[t * n + x])
                c = int(ec[e])
                if c >= 0:
                    par ^= (int(S[c >> 6]) >> (c & 63)) & 1
                x = int(rows[e])
            assert lab[t, v] == par
