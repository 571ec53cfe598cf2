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


def batch_select(prob):
    """The formulation of the batched kernel (one CTA per problem): pivots through a
    reduced row echelon basis keyed by lead bit, the first odd pivot without
    excluding used ones, beta through the 64x64 matrix of unit responses, the final
    rows from the transposed block T, D from (coordinate, iteration) pairs."""
    N, K = prob.N, prob.K
    off, co = prob.cycle_lists()
    lists = [co[off[r]:off[r + 1]].tolist() for r in range(K)]
    S = [1 << j for j in range(N)]
    sel = []
    for e0 in range(0, N, 64):
        b = min(64, N - e0)
        bound = e0 + b
        T = [sum(((S[e0 + i] >> c) & 1) << i for i in range(b)) for c in range(bound)]
        assert all(T[c] == 1 << (c - e0) for c in range(e0, bound))
        basis, piv = {}, []  # lead bit -> vector with zeros at every other lead
        for r in range(K):
            W = 0
            for c in lists[r]:
                if c >= bound:
                    break
                W ^= T[c]
            res = W
            for lead in list(basis):
                if (W >> lead) & 1:
                    res ^= basis[lead]
            if res:
                L = (res & -res).bit_length() - 1
                for lead in basis:
                    if (basis[lead] >> L) & 1:
                        basis[lead] ^= res
                basis[L] = res
                piv.append((r, W))
                if len(piv) == b:
                    break
        m = [1 << k for k in range(b)]
        pk = []
        for k in range(b):
            p = next(i for i in range(b) if parity(piv[i][1] & m[k]))
            pk.append(p)
            for j in range(k + 1, b):
                if parity(piv[p][1] & m[j]):
                    m[j] ^= m[k]
        gcol = [sum(parity(piv[pk[k]][1] & m[i]) << i for i in range(k)) for k in range(b)]
        Mrow = []
        for k in range(b):
            bt = 1 << k
            for i in range(k + 1, b):
                bt |= parity(bt & gcol[i]) << i
            Mrow.append(bt)
        F = [sum(parity(T[c] & m[k]) << c for c in range(e0)) | (m[k] << e0) for k in range(b)]
        for k in range(b):
            S[e0 + k] = F[k]
        sel += [piv[p][0] for p in pk]
        pairs = [(c, k) for k in range(b) for c in lists[piv[pk[k]][0]]]
        for j in range(bound, N):
            beta = 0
            for c, k in pairs:
                bit = (S[j] >> c) & 1 if c < e0 else int(c == j)
                if bit:
                    beta ^= Mrow[k]
            for k in range(b):
                if (beta >> k) & 1:
                    S[j] ^= F[k]
    return sel


@pytest.mark.parametrize("graph", [grid_graph(6, 6, 1, 10, 3), random_graph(200, 400, 1, 20, 2),
                                   grid_graph(12, 12, 1, 3, 9)])
def test_batch_formulation_equals_sequential(graph):
    p = Problem.from_graph(graph).prepare(threads=2, keep_trees=True)
    ref, _, _ = oracle.solve(p, threads=2)
    assert batch_select(p) == ref.tolist()


def test_paired_pass_correction_identity():
    """W of a candidate against block B+1's rows after block B's update equals its W
    against those rows before the update, plus parity(W_B & gamma_i) in bit i, with
    gamma_i = XOR of block B's final masks m_k over the update bits beta_i of row i
    (the correction blk_wfix_kernel applies)."""
    p = Problem.from_graph(random_graph(200, 400, 1, 20, 2)).prepare(threads=2, keep_trees=True)
    N, K = p.N, p.K
    off, co = p.cycle_lists()
    lists = [co[off[r]:off[r + 1]].tolist() for r in range(K)]
    S = [1 << j for j in range(N)]
    dot = lambda s, r: sum((s >> c) & 1 for c in lists[r]) & 1  # noqa: E731
    Wof = lambda rows, r: sum(dot(rows[i], r) << i for i in range(len(rows)))  # noqa: E731
    checked = 0
    for e0 in range(0, N, 64):
        b = min(64, N - e0)
        W0 = {}
        if e0 + 64 < N:
            nxt = S[e0 + 64:e0 + 128]
            W0 = {r: Wof(nxt, r) for r in range(0, K, 7)}
        WB = {r: Wof(S[e0:e0 + b], r) for r in W0}
        # the block as in blocked_select
        echelon, piv = {}, []
        for r in range(K):
            W = Wof(S[e0:e0 + b], r)
            x = W
            while x:
                q = (x & -x).bit_length() - 1
                if q in echelon:
                    x ^= echelon[q]
                else:
                    echelon[q] = x
                    piv.append((r, W))
                    break
            if len(piv) == b:
                break
        m = [1 << k for k in range(b)]
        g, chosen, used = [], [], set()
        for k in range(b):
            q = next(i for i in range(b) if i not in used and parity(piv[i][1] & m[k]))
            used.add(q)
            chosen.append(q)
            g.append(sum(parity(piv[q][1] & m[i]) << i for i in range(k)))
            for j in range(k + 1, b):
                if parity(piv[q][1] & m[j]):
                    m[j] ^= m[k]
        S0 = [S[e0 + l] for l in range(b)]
        for k in range(b):
            S[e0 + k] = 0
            for l in range(b):
                if (m[k] >> l) & 1:
                    S[e0 + k] ^= S0[l]
        betas = []
        for j in range(e0 + b, N):
            D = sum(dot(S[j], piv[chosen[k]][0]) << k for k in range(b))
            beta = 0
            for k in range(b):
                beta |= (((D >> k) & 1) ^ parity(beta & g[k])) << k
            betas.append(beta)
            for k in range(b):
                if (beta >> k) & 1:
                    S[j] ^= S[e0 + k]
        if W0:
            nb = min(64, N - e0 - 64)
            gam = []
            for i in range(nb):
                x = 0
                for k in range(b):
                    if (betas[i] >> k) & 1:
                        x ^= m[k]
                gam.append(x)
            for r, w0 in W0.items():
                want = Wof(S[e0 + 64:e0 + 64 + nb], r)
                corr = sum(parity(WB[r] & gam[i]) << i for i in range(nb))
                assert want == w0 ^ corr
                checked += 1
    assert checked > 50


def test_grouped_pass_correction_identity_three_blocks():
    """The grouped pass over three blocks B, B+1, B+2: W of a candidate against block
    B+2's rows at its start equals W0 (against those rows at B's start) plus, for each
    earlier block i in {B, B+1}, bit r: parity(W_i & gamma_ir), gamma_ir = XOR of block
    i's final masks over row r's update bits in block i, W_i = the candidate's W in
    block i (the two corrections blk_wfix_kernel<2> applies)."""
    p = Problem.from_graph(random_graph(260, 520, 1, 20, 5)).prepare(threads=2, keep_trees=True)
    N, K = p.N, p.K
    off, co = p.cycle_lists()
    lists = [co[off[r]:off[r + 1]].tolist() for r in range(K)]
    S = [1 << j for j in range(N)]
    dot = lambda s, r: sum((s >> c) & 1 for c in lists[r]) & 1  # noqa: E731
    Wof = lambda rows, r: sum(dot(rows[i], r) << i for i in range(len(rows)))  # noqa: E731
    sample = list(range(0, K, 11))
    hist = []  # per block: (e0, W of the sample, masks, betas by row)
    W0 = {}
    checked = 0
    for e0 in range(0, N, 64):
        b = min(64, N - e0)
        bi = e0 // 64
        if bi % 3 == 0 and e0 + 128 < N:
            W0 = {r: Wof(S[e0 + 128:e0 + 192], r) for r in sample}
        if bi % 3 == 2 and W0:
            nb = min(64, N - e0)
            for r in sample:
                want = Wof(S[e0:e0 + nb], r)
                got = W0[r]
                for (ei, Wi, mi, betas) in hist[-2:]:
                    bi_ = min(64, N - ei)
                    corr = 0
                    for row in range(nb):
                        beta = betas[e0 + row]
                        gam = 0
                        for k in range(bi_):
                            if (beta >> k) & 1:
                                gam ^= mi[k]
                        corr |= parity(Wi[r] & gam) << row
                    got ^= corr
                assert got == want
                checked += 1
            W0 = {}
        Wb = {r: Wof(S[e0:e0 + b], r) for r in sample}
        echelon, piv = {}, []
        for r in range(K):
            W = Wof(S[e0:e0 + b], r)
            x = W
            while x:
                q = (x & -x).bit_length() - 1
                if q in echelon:
                    x ^= echelon[q]
                else:
                    echelon[q] = x
                    piv.append((r, W))
                    break
            if len(piv) == b:
                break
        m = [1 << k for k in range(b)]
        g, chosen, used = [], [], set()
        for k in range(b):
            q = next(i for i in range(b) if i not in used and parity(piv[i][1] & m[k]))
            used.add(q)
            chosen.append(q)
            g.append(sum(parity(piv[q][1] & m[i]) << i for i in range(k)))
            for j in range(k + 1, b):
                if parity(piv[q][1] & m[j]):
                    m[j] ^= m[k]
        S0 = [S[e0 + l] for l in range(b)]
        for k in range(b):
            S[e0 + k] = 0
            for l in range(b):
                if (m[k] >> l) & 1:
                    S[e0 + k] ^= S0[l]
        betas = {}
        for j in range(e0 + b, N):
            D = sum(dot(S[j], piv[chosen[k]][0]) << k for k in range(b))
            beta = 0
            for k in range(b):
                beta |= (((D >> k) & 1) ^ parity(beta & g[k])) << k
            betas[j] = beta
            for k in range(b):
                if (beta >> k) & 1:
                    S[j] ^= S[e0 + k]
        hist.append((e0, Wb, m, betas))
    assert checked > 20


def blocked_select_wordlists(prob, B, ww, cap):
    """blocked_select with the far update of the blocked run's word-list form: the B
    rows after a block are near rows (D gathered directly); every later ("far") row is
    either still its unit vector (D from membership of its own coordinate in the
    selected cycles: the scatter), or listed by its nonzero ww-bit words (D from the
    pairs in those words only), or dense past `cap` listed words (D gathered
    directly).  Every far row's D is checked against the direct one at every block,
    and the rows are relisted after they change.  Returns the selected ranks."""
    N, K = prob.N, prob.K
    off, co = prob.cycle_lists()
    lists = [co[off[r]:off[r + 1]].tolist() for r in range(K)]
    S = [1 << j for j in range(N)]
    dot = lambda s, r: sum((s >> c) & 1 for c in lists[r]) & 1  # noqa: E731
    unit = [True] * N
    words = [None] * N  # listed words of a non-unit far row, or "dense"
    mask = (1 << ww) - 1

    def relist(j, Wb):
        nz = [w for w in range(Wb) if (S[j] >> (ww * w)) & mask]
        own = j // ww
        assert own >= Wb and (S[j] >> (ww * own)) & mask == 1 << (j % ww)  # the row's own word: bit j alone
        assert S[j] >> (ww * Wb) == (S[j] >> (ww * own)) << (ww * (own - Wb))  # nothing else above Wb
        nz.append(own)
        words[j] = nz if len(nz) <= cap else "dense"

    sel = []
    checked = {"unit": 0, "sparse": 0, "dense": 0}
    for e0 in range(0, N, B):
        b = min(B, N - e0)
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
        # the selected cycles' (coordinate, k) pairs, by word
        pairs = [(c, k) for k in range(b) for c in lists[piv[chosen[k]][0]]]
        by_word = {}
        for c, k in pairs:
            by_word.setdefault(c // ww, []).append((c, k))
        Wb = (e0 + b + ww - 1) // ww
        far_start = e0 + b + B
        for j in range(e0 + b, N):
            D = sum(dot(S[j], piv[chosen[k]][0]) << k for k in range(b))
            if j >= far_start:
                if unit[j]:
                    Dw = sum(1 << k for c, k in pairs if c == j)
                    checked["unit"] += 1
                elif words[j] == "dense":
                    Dw = D
                    checked["dense"] += 1
                else:
                    Dw = 0
                    for w in words[j]:
                        for c, k in by_word.get(w, []):
                            Dw ^= ((S[j] >> c) & 1) << k
                    checked["sparse"] += 1
                assert Dw == D, (e0, j)
            beta = 0
            for k in range(b):
                beta |= (((D >> k) & 1) ^ parity(beta & g[k])) << k
            for k in range(b):
                if (beta >> k) & 1:
                    S[j] ^= S[e0 + k]
            if j >= far_start and beta:
                unit[j] = False
                relist(j, Wb)
    return sel, checked


@pytest.mark.parametrize("graph,B,cap", [(random_graph(200, 400, 1, 20, 2), 8, 3),
                                         (random_graph(200, 400, 1, 20, 2), 8, 64),
                                         (random_graph(300, 700, 1, 5, 5), 8, 2)])
def test_far_update_by_word_lists(graph, B, cap):
    p = Problem.from_graph(graph).prepare(threads=2, keep_trees=True)
    ref, _, _ = oracle.solve(p, threads=2)
    sel, checked = blocked_select_wordlists(p, B, 8, cap)
    assert sel == ref.tolist()
    assert checked["unit"] > 0 and checked["sparse"] > 0  # all three kinds of far row met
    assert (checked["dense"] > 0) == (cap < 8)


def sequential_pivots(W, b):
    """The first b candidates, in rank order, whose W is independent of every earlier
    W (the pivots of a block)."""
    echelon, piv = {}, []
    for r, w in enumerate(W):
        x = w
        while x:
            p = (x & -x).bit_length() - 1
            if p in echelon:
                x ^= echelon[p]
            else:
                echelon[p] = x
                piv.append(r)
                break
        if len(piv) == b:
            break
    return piv


def reduce_by(x, echelon):
    while x:
        p = (x & -x).bit_length() - 1
        if p not in echelon:
            return x, p
        x ^= echelon[p]
    return 0, -1


def windowed_pivots(W, b, G, tile, shape):
    """The pivot search of blk_pivot_kernel restated step by step: G CTAs, CTA c owning
    the tiles t = c (mod G); per step each CTA scans its next window of tiles from the
    scan start s (the shape's window for the number of pivots known), turns every
    candidate independent of the basis and its own local pivots into a local pivot,
    stops after the shape's local-pivot limit, and reports its local pivots and `end`
    (every one of its candidates below end scanned); the merge takes D = min end and
    accepts, in rank order, the reported local pivots below D independent of the
    basis and of those accepted before them; s = D.  Returns the pivots and the steps."""
    win_early, rank_early, win_mid, rank_tail, win_tail, lmax = shape
    K = len(W)
    ntiles = (K + tile - 1) // tile
    basis, piv, s, steps = {}, [], 0, 0
    while len(piv) < b:
        steps += 1
        wsz = win_early if len(piv) < rank_early else win_tail if len(piv) >= rank_tail else win_mid
        t0 = s // tile
        reports, ends = [], []
        for c in range(G):
            tf = t0 + ((c - t0 % G) % G)
            tiles = [t for t in (tf + m * G for m in range(wsz)) if t < ntiles]
            local = dict(basis)
            nloc, end, trunc = 0, K, False
            for t in tiles:
                lo = max(t * tile, s)
                for r in range(lo, min((t + 1) * tile, K)):
                    x, p = reduce_by(W[r], local)
                    if x:
                        local[p] = x
                        reports.append((r, W[r]))
                        nloc += 1
                        if nloc == lmax:
                            end, trunc = r + 1, True
                            break
                if trunc:
                    break
            if not trunc and len(tiles) == wsz:
                end = min((tiles[-1] + 1) * tile, K)
            ends.append(end)
        D = min(ends)
        for r, w in sorted(x for x in reports if x[0] < D):
            x, p = reduce_by(w, basis)
            if x and len(piv) < b:
                basis[p] = x
                piv.append(r)
        if D >= K and len(piv) < b:
            break  # the candidates do not span
        s = D
    return piv, steps


@pytest.mark.parametrize("seed", range(6))
def test_windowed_pivot_search_is_exact_for_every_shape(seed):
    # W's of a block with its pivots spread over the rank order (each pivot brings a
    # new direction; every other candidate is zero or a combination of the directions
    # seen so far, the common case in a de Pina block): the step-wise search gives the
    # sequential pivots for every window, local-pivot limit and grid size
    rng = np.random.default_rng(seed)
    b, K = 16, 2500
    at = sorted(rng.choice(np.arange(1, K), size=b - 1, replace=False).tolist()) + [0]
    at = sorted(at)
    W, dirs = [], []
    for r in range(K):
        if at and r == at[0]:
            at.pop(0)
            v = (1 << len(dirs)) | (int(rng.integers(0, 1 << len(dirs))) if dirs else 0)
            dirs.append(v)
            W.append(v)
        elif dirs and rng.random() < 0.6:
            w = 0
            for i in rng.choice(len(dirs), size=int(rng.integers(1, 4))):
                w ^= dirs[int(i)]
            W.append(w)
        else:
            W.append(0)
    want = sequential_pivots(W, b)
    assert len(want) == b
    for G in (1, 3, 7):
        for tile in (16, 64):
            for shape in ((2, 8, 6, 12, 8, 6), (1, 4, 4, 12, 12, 8), (4, 8, 8, 12, 12, 1), (3, 5, 2, 9, 1, 3)):
                got, steps = windowed_pivots(W, b, G, tile, shape)
                assert got == want, (G, tile, shape)
                assert steps >= 1
