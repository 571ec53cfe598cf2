"""Preparation with the candidate generation on the device.

The host prepares the graph up to its spanning tree (chain contraction, FVS,
coordinates: Problem.prepare(structure_only=True)); the per-root shortest-path trees,
the candidate test and the cycle coordinate lists run on the GPU (GpuGen over
mcbgpu_gen_*, include/mcbgpu.h); the host keeps the heap-ordered searches of the
roots whose tree has a tie and the ranking (per-root group maps and the sort on
weight, Problem.rank_candidates).  The candidate list, its rank order and the
coordinate lists are those of Problem.prepare(); the lists never leave the device:
they go straight into a Solver.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from ._native import check_gpu, gpu_lib, ptr
from .gpu import Solver, _stream
from .host import Graph, Problem


class GpuGen:
    """Handle over mcbgpu_gen_*: device candidate generation for a structure-only
    prepared Problem."""

    def __init__(self, p: Problem, chunk: int = 0):
        self.lib = gpu_lib()
        rows, cols, w, rev, ro = p.reduced_graph()
        _, ec = p.coords()
        fa, fv = p.fvs()
        pairs = p.pairs()
        self.n, self.F, self.N = p.n, p.F, p.N
        if chunk <= 0:  # about 12 GB of per-chunk buffers (20 bytes per vertex and root)
            chunk = int(min(8192, max(256, (12 << 30) // max(20 * self.n + len(pairs) // 8, 1))))
        self.chunk = min(chunk, self.F)
        # chunks while the tree kernel's shapes are timed: two waves of the largest grid
        self.tune_count = min(self.chunk, 2 * 16 * 152)
        h = C.c_void_p()
        check_gpu(self.lib.mcbgpu_gen_create(C.byref(h), self.n, len(cols), ptr(ro), ptr(rows), ptr(cols),
                                             ptr(np.ascontiguousarray(w, np.int32)), ptr(rev), ptr(ec), self.N,
                                             ptr(fa), ptr(fv), self.F, ptr(pairs), self.chunk), "mcbgpu_gen_create")
        self._h = h

    def trees(self, t0: int, count: int, stream=0) -> np.ndarray:
        tied = np.zeros(max(count, 1), np.uint8)
        check_gpu(self.lib.mcbgpu_gen_trees(self._h, t0, count, ptr(tied), _stream(stream)), "mcbgpu_gen_trees")
        return tied[:count]

    def submit(self, t0: int, count: int, stream=0) -> None:
        check_gpu(self.lib.mcbgpu_gen_trees_submit(self._h, t0, count, _stream(stream)), "mcbgpu_gen_trees_submit")

    def collect(self, t0: int, count: int, stream=0) -> np.ndarray:
        tied = np.zeros(max(count, 1), np.uint8)
        check_gpu(self.lib.mcbgpu_gen_trees_collect(self._h, t0, ptr(tied), _stream(stream)),
                  "mcbgpu_gen_trees_collect")
        return tied[:count]

    def tuning(self) -> bool:
        return bool(self.lib.mcbgpu_gen_tuning(self._h))

    def put_trees(self, trees, dist, parent_slot, stream=0) -> None:
        t = np.ascontiguousarray(trees, np.int32)
        d = np.ascontiguousarray(dist, np.int32)
        ps = np.ascontiguousarray(parent_slot, np.int32)
        check_gpu(self.lib.mcbgpu_gen_put_trees(self._h, ptr(t), len(t), ptr(d), ptr(ps), _stream(stream)),
                  "mcbgpu_gen_put_trees")

    def candidates(self, count: int, stream=0):
        """(pair indices, weights, per-root counts) of the current chunk."""
        counts = np.zeros(max(count, 1), np.int64)
        total = C.c_int64()
        check_gpu(self.lib.mcbgpu_gen_candidates(self._h, ptr(counts), C.byref(total), _stream(stream)),
                  "mcbgpu_gen_candidates")
        k = total.value
        pi = np.empty(max(k, 1), np.uint32)
        wi = np.empty(max(k, 1), np.int32)
        check_gpu(self.lib.mcbgpu_gen_fetch(self._h, k, ptr(pi), ptr(wi), _stream(stream)), "mcbgpu_gen_fetch")
        return pi[:k], wi[:k], counts[:count]

    def lists(self, tree, edge_offset, weight, stream=0) -> int:
        """Builds the sorted coordinate lists of the ranked candidates on the device;
        returns their total length."""
        t = np.ascontiguousarray(tree, np.int32)
        e = np.ascontiguousarray(edge_offset, np.int32)
        w = np.ascontiguousarray(weight, np.int32)
        nnz = C.c_int64()
        check_gpu(self.lib.mcbgpu_gen_lists(self._h, len(t), ptr(t), ptr(e), ptr(w), C.byref(nnz), _stream(stream)),
                  "mcbgpu_gen_lists")
        self.K = len(t)
        self.nnz = nnz.value
        return self.nnz

    def device_lists(self):
        """Device addresses (weight, offsets, coords) of the lists."""
        w, o, c = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check_gpu(self.lib.mcbgpu_gen_get_lists(self._h, C.byref(w), C.byref(o), C.byref(c)), "mcbgpu_gen_get_lists")
        return w.value, o.value, c.value

    def fetch_lists(self, stream=0):
        """The lists copied to the host: (offsets int64[K+1], coords int32[nnz])."""
        off = np.empty(self.K + 1, np.int64)
        co = np.empty(max(self.nnz, 1), np.int32)
        check_gpu(self.lib.mcbgpu_gen_copy_lists(self._h, ptr(off), ptr(co), _stream(stream)),
                  "mcbgpu_gen_copy_lists")
        return off, co[:self.nnz]

    def tree_shapes(self) -> dict:
        """The tree kernel's tuned launch shapes: every shape tried (threads per CTA,
        CTAs per SM, bucket width in quarters of the mean weight) with its
        microseconds per root, and the one kept."""
        cap = 16
        sh = np.zeros(3 * cap, np.int32)
        us = np.zeros(cap, np.float64)
        cnt, ch = C.c_int32(), C.c_int32()
        check_gpu(self.lib.mcbgpu_gen_tree_shapes(self._h, ptr(sh), ptr(us), cap, C.byref(cnt), C.byref(ch)),
                  "mcbgpu_gen_tree_shapes")
        tried = [{"threads": int(sh[3 * i]), "ctas_per_sm": int(sh[3 * i + 1]),
                  "delta_x_mean_weight": sh[3 * i + 2] / 4.0, "us_per_root": round(float(us[i]), 2)}
                 for i in range(min(cnt.value, cap)) if us[i] >= 0]
        return {"tried": tried, "chosen": int(ch.value)}

    def release_trees(self) -> None:
        check_gpu(self.lib.mcbgpu_gen_release_trees(self._h), "mcbgpu_gen_release_trees")

    @property
    def device_bytes(self) -> int:
        return int(self.lib.mcbgpu_gen_device_bytes(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.mcbgpu_gen_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


@dataclass
class DevicePrepared:
    """A problem prepared with the device candidate generation: the host Problem
    (candidates in rank order, no host lists), the Solver holding the lists, and the
    time of each phase (seconds)."""
    problem: Problem
    solver: Solver | None
    K: int
    nnz: int
    tied_roots: int
    times: dict = field(default_factory=dict)
    tree_shapes: dict = field(default_factory=dict)


def generate_candidates(p: Problem, gen: GpuGen, threads: int = 0, stream=0):
    """Every root's tree and candidates on the device, chunk after chunk; the roots the
    device leaves to the host (ties) are searched on the host while the next chunk's
    trees run.  Returns (per-root offsets, pair indices, weights: the arguments of
    Problem.rank_candidates, as lists of arrays), the number of tied roots, and the
    seconds spent in the host searches."""
    F = p.F
    state = {"next": 0}

    def submit():
        t0 = state["next"]
        if t0 >= F:
            return None
        cnt = min(gen.tune_count if gen.tuning() else gen.chunk, F - t0)
        gen.submit(t0, cnt, stream)
        state["next"] = t0 + cnt
        return t0, cnt

    offs, pis, wis = [np.zeros(1, np.int64)], [], []
    base, tied_total, t_host = 0, 0, 0.0
    pending = [submit()]
    while pending:
        t0, cnt = pending.pop(0)
        tied = gen.collect(t0, cnt, stream)
        nxt = submit()  # its trees run on the device while the host searches this chunk's ties
        if nxt is not None:
            pending.append(nxt)
        idx = np.nonzero(tied)[0]
        if len(idx):
            th = time.perf_counter()
            d, ps = p.search_trees(t0 + idx, threads=threads)
            gen.put_trees(t0 + idx, d, ps, stream)
            t_host += time.perf_counter() - th
            tied_total += len(idx)
        pi, wi, counts = gen.candidates(cnt, stream)
        pis.append(pi)
        wis.append(wi)
        offs.append(base + np.cumsum(counts))
        base += int(counts.sum())
    return (np.concatenate(offs), np.concatenate(pis) if pis else np.zeros(0, np.uint32),
            np.concatenate(wis) if wis else np.zeros(0, np.int32), tied_total, t_host)


def prepare_on_device(src, threads: int = 0, chunk: int = 0, stream=0, make_solver: bool = True,
                      keep_gen: bool = False):
    """Graph (or an unprepared Problem) -> DevicePrepared: host structure, device
    trees / candidate test / lists, host ranking, and (make_solver) a Solver with the
    lists uploaded device to device.  With keep_gen the GpuGen handle is returned
    too (its lists stay on the device; its trees are released once the lists are
    built)."""
    times = {}
    t0 = time.perf_counter()
    p = Problem.from_graph(src) if isinstance(src, Graph) else src
    p.prepare(threads=threads, structure_only=True)
    times["structure"] = time.perf_counter() - t0
    if p.info.single_cycle or p.N == 0:
        raise ValueError("the graph needs no search (a single cycle or a forest)")
    t1 = time.perf_counter()
    gen = GpuGen(p, chunk)
    times["device_setup"] = time.perf_counter() - t1
    t2 = time.perf_counter()
    offs, pis, wis, tied_total, t_host_search = generate_candidates(p, gen, threads, stream)
    times["trees_and_candidates"] = time.perf_counter() - t2
    shapes = gen.tree_shapes()
    times["host_searches_of_tied_roots"] = t_host_search
    t3 = time.perf_counter()
    p.rank_candidates(offs, pis, wis, threads=threads)
    _, edge, w, tree = p.candidates()
    times["ranking"] = time.perf_counter() - t3
    t4 = time.perf_counter()
    nnz = gen.lists(tree, edge, w, stream)
    gen.release_trees()  # the lists are built: the F x n' parent slots are not needed any more
    times["lists"] = time.perf_counter() - t4
    solver = None
    if make_solver:
        t5 = time.perf_counter()
        dw, do, dc = gen.device_lists()
        solver = Solver.from_device_lists(p.N, len(w), nnz, dw, do, dc, stream)
        times["solver_upload"] = time.perf_counter() - t5
    times["total"] = time.perf_counter() - t0
    out = DevicePrepared(p, solver, len(w), nnz, tied_total, times, shapes)
    if keep_gen:
        return out, gen
    gen.close()
    return out
