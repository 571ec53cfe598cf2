"""The blocked reformulation used by mcbgpu_solver_run, restated in pure Python,
selects exactly the oracle's sequence (checks the mathematics on the CPU; the GPU
tests check the kernels)."""
import numpy as np
import pytest

import oracle
from minimumcyclebasis_gb300 import Problem, grid_graph, random_graph


def parity(x):
    return bin(x).count("1") & 1


def blocked_select(prob, B):
    N, K = prob.N, prob.K
    off, co = prob.cycle_lists()
    lists = [co[off[r]:off[r + 1]].tolist() for r in range(K)]
    S = [1 << j for j in range(N)]
    dot = lambda s, r: sum((s >> c) & 1 for c in lists[r]) & 1  # noqa: E731
    sel = []
    for e0 in range(0, N, B):
        b = min(B, N - e0)
        # first b candidates (rank order) whose W is independent of all earlier W's
        echelon, piv = {}, []
        for r in range(K):
            W = sum(dot(S[e0 + k], r) << k for k in range(b))
            x = W
            while x:
                p = (x & -x).bit_length() - 1
                if p in echelon:
                    x ^= echelon[p]
                else:
                    echelon[p] = x
                    piv.append((r, W))
                    break
            if len(piv) == b:
                break
        m = [1 << k for k in range(b)]
        g, chosen, used = [], [], set()
        for k in range(b):
            p = next(i for i in range(b) if i not in used and parity(piv[i][1] & m[k]))
            used.add(p)
            chosen.append(p)
            wp = piv[p][1]
            g.append(sum(parity(wp & m[i]) << i for i in range(k)))
            for j in range(k + 1, b):
                if parity(wp & m[j]):
                    m[j] ^= m[k]
        S0 = [S[e0 + l] for l in range(b)]
        for k in range(b):
            v = 0
            for l in range(b):
                if (m[k] >> l) & 1:
                    v ^= S0[l]
            S[e0 + k] = v
        sel += [piv[c][0] for c in chosen]
        for j in range(e0 + b, N):
            D = sum(dot(S[j], piv[chosen[k]][0]) << k for k in range(b))
            beta = 0
            for k in range(b):
                beta |= (((D >> k) & 1) ^ parity(beta & g[k])) << k
            for k in range(b):
                if (beta >> k) & 1:
                    S[j] ^= S[e0 + k]
    return sel


@pytest.mark.parametrize("graph,B", [(grid_graph(6, 6, 1, 10, 3), 64), (grid_graph(6, 6, 1, 10, 3), 5),
                                     (random_graph(200, 400, 1, 20, 2), 64), (random_graph(200, 400, 1, 20, 2), 8),
                                     (grid_graph(10, 10, 1, 3, 9), 7)])
def test_blocked_equals_sequential(graph, B):
    p = Problem.from_graph(graph).prepare(threads=2, keep_trees=True)
    ref, _, _ = oracle.solve(p, threads=2)
    assert blocked_select(p, B) == ref.tolist()
