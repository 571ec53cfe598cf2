"""GPU parity: every device path against the oracle and the reference's golden
vectors.  Bit-exact (integer / GF(2) work): selected ranks, total weight, labels,
cycle vectors and support vectors must be identical."""
import numpy as np
import pytest

import oracle
from conftest import golden_names, load_golden
from minimumcyclebasis_gb300 import GpuStruct, Problem, Solver, random_graph, solve

pytestmark = pytest.mark.gpu


def prep(name, **kw):
    fx = load_golden(name)
    return fx, Problem.from_mtx(fx["mtx"]).prepare(threads=4, keep_trees=True, **kw)


@pytest.mark.parametrize("name", ["grid8x8_s3", "rand300_s0", "grid32x32_s1", "rgg500_s3"])
@pytest.mark.parametrize("chunk", [720, 7])
def test_label_forest_matches_oracle(name, chunk):
    fx, p = prep(name, ref_layout=True)
    rows, cols, w, rev, ro = p.reduced_graph()
    _, ec = p.coords()
    lv, pp, eo, ni = p.ref_layout()
    n, F = p.n, p.F
    gs = GpuStruct(rows.shape[0], p.N, n, F, chunk_size=chunk)
    gs.initialize_memory(ec, lv, pp, eo)
    rng = np.random.default_rng(7)
    vectors = [oracle.support_vector_at(p, 0), oracle.support_vector_at(p, p.N // 2),
               rng.integers(0, 2**63, size=(p.N + 63) // 64, dtype=np.int64).astype(np.uint64)]
    vectors[-1][-1] &= np.uint64((1 << (p.N % 64)) - 1) if p.N % 64 else np.uint64(2**64 - 1)
    NI = ni.reshape(F, n)
    for S in vectors:
        gs.copy_support_vector(S)
        lab, ms = gs.process_shortest_path()
        want = oracle.labels(p, S)
        got = np.take_along_axis(lab, NI.astype(np.int64), axis=1)
        assert np.array_equal(got, want.astype(np.uint32))
    gs.close()


def test_label_forest_flags_levels_that_end_early():
    # tree 1's levels stop after level 1: its deeper positions are on no level, the
    # call reports bad input and those positions read 0; the other trees are intact
    from minimumcyclebasis_gb300._native import MCBError
    fx, p = prep("grid8x8_s3", ref_layout=True)
    rows, cols, w, rev, ro = p.reduced_graph()
    _, ec = p.coords()
    lv, pp, eo, ni = p.ref_layout()
    n, F = p.n, p.F
    lv = lv.reshape(F, n + 1).copy()
    cut = int(lv[1, 2])
    assert 1 < cut < n
    lv[1, 2:] = cut
    gs = GpuStruct(rows.shape[0], p.N, n, F, chunk_size=720)
    gs.initialize_memory(ec, lv.reshape(-1), pp, eo)
    gs.copy_support_vector(oracle.support_vector_at(p, 0))
    out = np.full(F * n, 7, np.uint32)
    import ctypes as C
    ptrs = (C.c_void_p * 1)(out.ctypes.data)
    rc = gs.lib.mcbgpu_struct_process_shortest_path(gs._h, ptrs, 0, None)
    assert rc != 0 and b"status 0x8" in gs.lib.mcbgpu_last_error()
    out = out.reshape(F, n)
    assert (out[1, cut:] == 0).all()
    want = oracle.labels(p, oracle.support_vector_at(p, 0))
    NI = ni.reshape(F, n).astype(np.int64)
    got = np.take_along_axis(out, NI, axis=1)
    keep = np.ones(F, bool)
    keep[1] = False
    assert np.array_equal(got[keep], want[keep].astype(np.uint32))
    gs.close()


@pytest.mark.parametrize("name", golden_names())
def test_blocked_run_matches_reference(name):
    fx, p = prep(name)
    s = Solver.from_problem(p)
    s.run()
    sel, tot = s.results()
    assert sel.tolist() == fx["selected_ranks"]
    assert tot == fx["total_weight"]
    s.close()


@pytest.mark.parametrize("name", ["grid4x4_s7", "grid32x32_s1", "rand300_w3_s2", "rand1000_s5", "tree_plus_one_s4"])
def test_plain_run_matches_reference(name):
    fx, p = prep(name)
    s = Solver.from_problem(p)
    s.run_plain()
    sel, tot = s.results()
    assert sel.tolist() == fx["selected_ranks"]
    assert tot == fx["total_weight"]


@pytest.mark.parametrize("name", ["grid8x8_s3", "rand300_s1"])
def test_per_iteration_calls_match_oracle(name):
    fx, p = prep(name)
    s = Solver.from_problem(p)
    for e in range(p.N):
        r = s.select(e)
        assert r == fx["selected_ranks"][e]
        if e % 7 == 0:
            assert np.array_equal(s.cycle_vector(e), oracle.cycle_vector(p, r))
        s.update(e)
        if e in (0, 3, p.N // 2):
            # rows > e now hold the support vectors as the reference has them after e+1 iterations
            assert np.array_equal(s.support_vector(e + 1), oracle.support_vector_at(p, e + 1))
    sel, tot = s.results()
    assert tot == fx["total_weight"]


@pytest.mark.parametrize("iters", [1, 63, 64, 65, 130])
def test_blocked_prefix_and_support_vectors(iters):
    fx, p = prep("rand1000_s5")
    s = Solver.from_problem(p)
    s.run(max_iterations=iters)
    sel, _ = s.results(iters)
    assert sel.tolist() == fx["selected_ranks"][:iters]
    # finished rows hold S_e as it was at iteration e; the next row holds S_iters
    for e in sorted({0, iters // 2, iters - 1, iters}):
        assert np.array_equal(s.support_vector(e), oracle.support_vector_at(p, e)), e


@pytest.mark.parametrize("N", [1, 2, 63, 64, 65, 127, 128, 129, 300])
def test_blocked_sizes_around_the_block_width(N):
    n = 150
    g = random_graph(n, n + N - 1, 1, 30, 100 + N)
    p = Problem.from_graph(g).prepare(threads=4, keep_trees=True)
    assert p.N == N
    ref, tot, _ = oracle.solve(p, threads=4)
    s = Solver.from_problem(p)
    s.run()
    sel, t = s.results()
    assert sel.tolist() == ref.tolist()
    assert t == tot
    s.reset()
    s.run_plain()
    sel2, t2 = s.results()
    assert sel2.tolist() == ref.tolist() and t2 == tot


def test_one_shot_c_abi_solve():
    fx, p = prep("grid32x32_s2")
    _, _, w, _ = p.candidates()
    off, co = p.cycle_lists()
    sel, tot = solve(p.N, w, off, co)
    assert sel.tolist() == fx["selected_ranks"]
    assert tot == fx["total_weight"]


def test_medium_random_graph_against_oracle():
    g = random_graph(3000, 6000, 1, 1000, 21)
    p = Problem.from_graph(g).prepare(threads=8, keep_trees=True)
    ref, tot, _ = oracle.solve(p, threads=8)
    s = Solver.from_problem(p)
    s.run()
    sel, t = s.results()
    assert np.array_equal(sel, ref) and t == tot


def test_upload_rejects_bad_lists():
    from minimumcyclebasis_gb300._native import MCBError
    w = np.array([3, 4], np.int32)
    off = np.array([0, 2, 3], np.int64)
    with pytest.raises(MCBError):
        Solver(4, w, off, np.array([2, 1, 0], np.int32))  # not ascending
    with pytest.raises(MCBError):
        Solver(4, w, off, np.array([0, 9, 1], np.int32))  # outside [0, N)


@pytest.mark.parametrize("name", ["grid8x8_s3", "rand300_s0", "grid32x32_s1", "planar2000_s2"])
def test_device_independence_certificate(name):
    # the selected cycles against the final support vectors: unit lower triangular,
    # so rank N of N; the host's elimination agrees
    fx, p = prep(name)
    s = Solver.from_problem(p)
    from minimumcyclebasis_gb300._native import MCBError
    with pytest.raises(MCBError):  # not before the run is complete
        s.verify()
    s.run()
    sel, _ = s.results()
    v = s.verify()
    assert v == {"rank": p.N, "violations": 0, "first": None}
    assert p.gf2_rank(sel) == p.N
    s.close()


def test_device_certificate_flags_a_wrong_basis():
    # the per-iteration form run with one selection forced to a repeated candidate is
    # not a de Pina run: its support vectors cannot certify the basis
    fx, p = prep("grid8x8_s3")
    s = Solver.from_problem(p)
    s.run()
    good = s.verify()
    assert good["violations"] == 0
    # a second solver whose lists make candidate 0 appear twice in the basis: the
    # lists of every candidate replaced by candidate 0's
    _, _, w, _ = p.candidates()
    off, co = p.cycle_lists()
    n0 = int(off[1])
    K = len(w)
    off2 = np.arange(K + 1, dtype=np.int64) * n0
    co2 = np.tile(co[:n0], K)
    s2 = Solver(p.N, w, off2, co2)
    s2.run()
    from minimumcyclebasis_gb300._native import MCBError
    with pytest.raises(MCBError):  # no odd candidate after the first iteration
        s2.results()
    s.close()
    s2.close()
