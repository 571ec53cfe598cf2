"""ORACLE — test infrastructure, not part of the product.

ctypes wrapper of oracle/libmcboracle.so, the CPU restatement of the reference's
de Pina main loop (mcb/mcb_non_cpu_rd.cpp:246-342; see mcb_oracle.cpp for the
line-by-line mapping).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline call it, and only as the checker / the timed CPU arm.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "libmcboracle.so")
        if not os.path.exists(path):
            from minimumcyclebasis_gb300.build import build_oracle
            build_oracle()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.mcbo_labels.restype = C.c_int
        L.mcbo_labels.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, C.c_int]
        L.mcbo_solve.restype = C.c_int64
        L.mcbo_solve.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, vp, vp, vp, vp, vp, vp, vp, C.c_int,
                                 C.c_int64, vp, C.POINTER(C.c_int64), C.POINTER(C.c_double)]
        L.mcbo_support_vector_at.restype = C.c_int64
        L.mcbo_support_vector_at.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, vp, vp, vp, vp, vp, vp, C.c_int,
                                             C.c_int64, vp]
        L.mcbo_label_pass_seconds.restype = C.c_double
        L.mcbo_label_pass_seconds.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, C.c_int, C.c_int,
                                              C.c_uint64]
        L.mcbo_update_row_seconds.restype = C.c_double
        L.mcbo_update_row_seconds.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64]
        _lib = L
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


def _inputs(prob):
    rows, cols, _, _, _ = prob.reduced_graph()
    _, ec = prob.coords()
    tp = prob.tree_parents()
    _, edge, w, tree = prob.candidates()
    return rows, cols, ec, tp, edge, w, tree


def solve(prob, threads: int = 0, max_iter: int = -1):
    """Run the de Pina loop on a prepared Problem (prepared with keep_trees=True).

    Returns (selected ranks int64[iters], total weight, seconds)."""
    rows, cols, ec, tp, edge, w, tree = _inputs(prob)
    i = prob.info
    sel = np.full(max(i.num_coords, 1), -1, np.int64)
    tot = C.c_int64()
    sec = C.c_double()
    it = lib().mcbo_solve(i.reduced_nodes, i.fvs_size, i.num_coords, i.num_candidates, _p(rows), _p(cols), _p(ec),
                          _p(tp), _p(edge), _p(w), _p(tree), threads, max_iter, _p(sel), C.byref(tot), C.byref(sec))
    if it < 0:
        raise RuntimeError("oracle: no odd candidate at iteration %d" % (-it - 1))
    return sel[:it], tot.value, sec.value


def labels(prob, S_words: np.ndarray, threads: int = 0) -> np.ndarray:
    """Labels P_t[v] (F x n, uint8) for support vector S (vertex-indexed)."""
    rows, cols, ec, tp, _, _, _ = _inputs(prob)
    i = prob.info
    out = np.zeros(i.fvs_size * i.reduced_nodes, np.uint8)
    S = np.ascontiguousarray(S_words, np.uint64)
    rc = lib().mcbo_labels(i.reduced_nodes, i.fvs_size, _p(rows), _p(cols), _p(ec), _p(tp), _p(S), _p(out),
                           threads)
    if rc:
        raise RuntimeError("oracle labels failed")
    return out.reshape(i.fvs_size, i.reduced_nodes)


def support_vector_at(prob, e: int, threads: int = 0) -> np.ndarray:
    """S_e as it stands at iteration e of the loop."""
    rows, cols, ec, tp, edge, _, tree = _inputs(prob)
    i = prob.info
    out = np.zeros((i.num_coords + 63) // 64, np.uint64)
    rc = lib().mcbo_support_vector_at(i.reduced_nodes, i.fvs_size, i.num_coords, i.num_candidates, _p(rows),
                                      _p(cols), _p(ec), _p(tp), _p(edge), _p(tree), threads, e, _p(out))
    if rc < 0:
        raise RuntimeError("oracle support_vector_at failed")
    return out


def cycle_vector(prob, rank: int) -> np.ndarray:
    """C of candidate `rank` as ceil(N/64) words, walking the tree parents
    (include/cycles.h:144-195)."""
    rows, cols, ec, tp, edge, _, tree = _inputs(prob)
    i = prob.info
    n = i.reduced_nodes
    words = np.zeros((i.num_coords + 63) // 64, np.uint64)
    e = int(edge[rank])
    pe = tp[int(tree[rank]) * n:(int(tree[rank]) + 1) * n]

    def setbit(c):
        words[c >> 6] |= np.uint64(1) << np.uint64(c & 63)

    if ec[e] >= 0:
        setbit(int(ec[e]))
    for x in (int(rows[e]), int(cols[e])):
        while pe[x] >= 0:
            pe_x = int(pe[x])
            if ec[pe_x] >= 0:
                setbit(int(ec[pe_x]))
            x = int(rows[pe_x]) if int(rows[pe_x]) != x else int(cols[pe_x])
    return words


def label_pass_seconds(prob, parent_edge, passes: int = 2, threads: int = 0, seed: int = 1) -> float:
    """Seconds per label pass of the loop over the trees whose parent edges are given
    (count x n, e.g. a sample of the FVS roots from Problem.search_trees), with
    random support vectors."""
    rows, cols, _, _, _ = prob.reduced_graph()
    _, ec = prob.coords()
    pe = np.ascontiguousarray(parent_edge, np.int32)
    F = pe.size // prob.n
    sec = lib().mcbo_label_pass_seconds(prob.n, F, prob.N, _p(rows), _p(cols), _p(ec), _p(pe), passes, threads,
                                        seed)
    if sec < 0:
        raise RuntimeError("oracle label_pass_seconds failed")
    return sec


def update_row_seconds(N: int, rows: int = 2048, passes: int = 3, threads: int = 0, seed: int = 1) -> float:
    """Seconds per row of the loop's full-width independence update at N coordinates."""
    sec = lib().mcbo_update_row_seconds(N, rows, passes, threads, seed)
    if sec < 0:
        raise RuntimeError("oracle update_row_seconds failed")
    return sec
