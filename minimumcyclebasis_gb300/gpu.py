"""Python handles over libmcbgpu.so (include/mcbgpu.h).

GpuStruct mirrors the reference's gpu_struct (gpu/gpu_struct.cuh:44-84): trees are
uploaded once, a support vector is copied in, and process_shortest_path returns
every tree's labels.  Solver holds the device-resident main loop: candidates in
rank order, S in HBM, and either the per-iteration calls (select / cycle_vector /
update, as the reference's loop makes them) or the blocked run.

Streams are CUDA stream handles as integers (e.g. torch.cuda.current_stream().cuda_stream);
0 is the legacy default stream.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._native import check_gpu, gpu_lib, ptr


def _stream(s) -> C.c_void_p:
    return C.c_void_p(int(s)) if s else None


def device_info() -> dict:
    lib = gpu_lib()
    d, sm, mem = C.c_int(), C.c_int(), C.c_size_t()
    check_gpu(lib.mcbgpu_init_cuda(C.byref(d), C.byref(sm), C.byref(mem)), "mcbgpu_init_cuda")
    return {"device": d.value, "sm_count": sm.value, "total_global_mem": mem.value}


class GpuStruct:
    """gpu_struct drop-in: labels of every FVS tree for one support vector."""

    def __init__(self, num_edges: int, num_coords: int, nodes: int, fvs_size: int, chunk_size: int = 720,
                 nstreams: int = 1):
        self.lib = gpu_lib()
        self.n, self.F, self.chunk = nodes, fvs_size, chunk_size
        self.size_vector = (num_coords + 63) // 64
        self.rows = (fvs_size + chunk_size - 1) // chunk_size
        h = C.c_void_p()
        check_gpu(self.lib.mcbgpu_struct_create(C.byref(h), num_edges, num_coords, self.size_vector, nodes,
                                                fvs_size, chunk_size, nstreams), "mcbgpu_struct_create")
        self._h = h

    def _rows_of(self, a: np.ndarray, per_tree: int):
        """Split a tree-major array into the per-chunk host rows compressed_trees holds."""
        ptrs = (C.c_void_p * max(self.rows, 1))()
        keep = []
        for r in range(self.rows):
            t0 = r * self.chunk
            part = np.ascontiguousarray(a[t0 * per_tree:min(self.F, t0 + self.chunk) * per_tree])
            keep.append(part)
            ptrs[r] = part.ctypes.data
        return ptrs, keep

    def initialize_memory(self, edge_coord: np.ndarray, level_offsets: np.ndarray, parent_pos: np.ndarray,
                          edge_offset: np.ndarray) -> None:
        n = self.n
        eo, k1 = self._rows_of(np.asarray(edge_offset, np.int32), n)
        lv, k2 = self._rows_of(np.asarray(level_offsets, np.uint32), n + 1)
        pp, k3 = self._rows_of(np.asarray(parent_pos, np.uint32), n)
        m = np.ascontiguousarray(edge_coord, np.int32)
        check_gpu(self.lib.mcbgpu_struct_initialize_memory(self._h, ptr(m), eo, lv, pp),
                  "mcbgpu_struct_initialize_memory")

    def copy_support_vector(self, words: np.ndarray) -> float:
        w = np.ascontiguousarray(words, np.uint64)
        ms = C.c_float()
        check_gpu(self.lib.mcbgpu_struct_copy_support_vector(self._h, ptr(w), C.byref(ms)),
                  "mcbgpu_struct_copy_support_vector")
        return ms.value

    def process_shortest_path(self, fetch: bool = True):
        """Returns (labels F x n uint32 in position order, milliseconds)."""
        ms = C.c_float()
        if not fetch:
            check_gpu(self.lib.mcbgpu_struct_process_shortest_path(self._h, None, 0, C.byref(ms)),
                      "mcbgpu_struct_process_shortest_path")
            return None, ms.value
        out = np.zeros(self.F * self.n, np.uint32)
        ptrs = (C.c_void_p * max(self.rows, 1))()
        for r in range(self.rows):
            ptrs[r] = out.ctypes.data + r * self.chunk * self.n * 4
        check_gpu(self.lib.mcbgpu_struct_process_shortest_path(self._h, ptrs, 0, C.byref(ms)),
                  "mcbgpu_struct_process_shortest_path")
        return out.reshape(self.F, self.n), ms.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            check_gpu(self.lib.mcbgpu_struct_clear_memory(self._h), "mcbgpu_struct_clear_memory")
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """Device-resident de Pina loop over rank-ordered candidates."""

    def __init__(self, num_coords: int, weight: np.ndarray, offsets: np.ndarray, coords: np.ndarray,
                 stream=0, upload: bool = True):
        self.lib = gpu_lib()
        self.N = int(num_coords)
        self.K = int(weight.shape[0])
        self.weight = np.ascontiguousarray(weight, np.int32)
        self.offsets = np.ascontiguousarray(offsets, np.int64)
        self.coords = np.ascontiguousarray(coords, np.int32)
        h = C.c_void_p()
        check_gpu(self.lib.mcbgpu_solver_create(C.byref(h), self.N, self.K, int(self.offsets[-1])),
                  "mcbgpu_solver_create")
        self._h = h
        if upload:
            self.upload(stream)

    @classmethod
    def from_device_lists(cls, num_coords: int, K: int, nnz: int, d_weight: int, d_offsets: int, d_coords: int,
                          stream=0) -> "Solver":
        """A solver whose candidates are already in device memory (a device candidate
        generation's lists): copied device to device (mcbgpu_solver_upload_device).
        No host copies are kept, so upload() needs explicit arrays."""
        self = cls.__new__(cls)
        self.lib = gpu_lib()
        self.N, self.K = int(num_coords), int(K)
        self.weight = self.offsets = self.coords = None
        h = C.c_void_p()
        check_gpu(self.lib.mcbgpu_solver_create(C.byref(h), self.N, self.K, int(nnz)), "mcbgpu_solver_create")
        self._h = h
        check_gpu(self.lib.mcbgpu_solver_upload_device(h, C.c_void_p(d_weight), C.c_void_p(d_offsets),
                                                       C.c_void_p(d_coords), _stream(stream)),
                  "mcbgpu_solver_upload_device")
        return self

    @classmethod
    def from_problem(cls, prob, stream=0) -> "Solver":
        _, _, w, _ = prob.candidates()
        off, co = prob.cycle_lists()
        return cls(prob.N, w, off, co, stream)

    def upload(self, stream=0, weight=None, offsets=None, coords=None) -> None:
        w = self.weight if weight is None else weight
        o = self.offsets if offsets is None else offsets
        c = self.coords if coords is None else coords
        check_gpu(self.lib.mcbgpu_solver_upload(self._h, ptr(w), ptr(o), ptr(c), _stream(stream)),
                  "mcbgpu_solver_upload")

    def reset(self, stream=0) -> None:
        check_gpu(self.lib.mcbgpu_solver_reset(self._h, _stream(stream)), "mcbgpu_solver_reset")

    # per-iteration form
    def select(self, e: int, stream=0, fetch: bool = True):
        r = C.c_int64()
        check_gpu(self.lib.mcbgpu_select(self._h, e, C.byref(r) if fetch else None, _stream(stream)),
                  "mcbgpu_select")
        return r.value if fetch else None

    def cycle_vector(self, e: int, stream=0) -> np.ndarray:
        out = np.zeros((self.N + 63) // 64, np.uint64)
        check_gpu(self.lib.mcbgpu_cycle_vector(self._h, e, ptr(out), _stream(stream)), "mcbgpu_cycle_vector")
        return out

    def update(self, e: int, stream=0) -> None:
        check_gpu(self.lib.mcbgpu_update(self._h, e, _stream(stream)), "mcbgpu_update")

    # whole-loop forms
    def run(self, max_iterations: int = -1, stream=0) -> None:
        check_gpu(self.lib.mcbgpu_solver_run(self._h, max_iterations, _stream(stream)), "mcbgpu_solver_run")

    def run_graph(self, max_iterations: int = -1, stream=0) -> None:
        """Reset + blocked run as one CUDA graph (captured on the first call, replayed after)."""
        check_gpu(self.lib.mcbgpu_solver_run_graph(self._h, max_iterations, _stream(stream)),
                  "mcbgpu_solver_run_graph")

    def run_plain(self, max_iterations: int = -1, stream=0) -> None:
        check_gpu(self.lib.mcbgpu_solver_run_plain(self._h, max_iterations, _stream(stream)),
                  "mcbgpu_solver_run_plain")

    def results(self, count: int | None = None, stream=0):
        """(selected ranks int64[count], total weight) after synchronising `stream`."""
        count = self.N if count is None else count
        sel = np.full(max(count, 1), -1, np.int64)
        tot = C.c_int64()
        check_gpu(self.lib.mcbgpu_solver_results(self._h, ptr(sel), count, C.byref(tot), _stream(stream)),
                  "mcbgpu_solver_results")
        return sel[:count], tot.value

    def verify(self, stream=0) -> dict:
        """The independence certificate of a complete run (mcbgpu_solver_verify):
        {"rank": N if every <C_i, S_j> (i <= j) is as a de Pina run leaves it, else
        None, "violations": count, "first": (i, j) or None}."""
        v, i, j = C.c_int64(), C.c_int64(), C.c_int64()
        check_gpu(self.lib.mcbgpu_solver_verify(self._h, C.byref(v), C.byref(i), C.byref(j), _stream(stream)),
                  "mcbgpu_solver_verify")
        return {"rank": self.N if v.value == 0 else None, "violations": int(v.value),
                "first": None if v.value == 0 else (int(i.value), int(j.value))}

    def support_vector(self, j: int, stream=0) -> np.ndarray:
        out = np.zeros((self.N + 63) // 64, np.uint64)
        check_gpu(self.lib.mcbgpu_solver_get_support(self._h, j, ptr(out), _stream(stream)),
                  "mcbgpu_solver_get_support")
        return out

    def set_profiling(self, enable: bool = True) -> None:
        check_gpu(self.lib.mcbgpu_solver_set_profiling(self._h, int(enable)), "mcbgpu_solver_set_profiling")

    def kernel_stats(self) -> dict:
        """{kernel: {launches, ms, bytes}} since set_profiling(True) (or the last call)."""
        from ._native import KernelStat
        arr = (KernelStat * 32)()
        cnt = C.c_int()
        check_gpu(self.lib.mcbgpu_solver_kernel_stats(self._h, arr, 32, C.byref(cnt)), "mcbgpu_solver_kernel_stats")
        return {arr[i].name.decode(): {"launches": arr[i].launches, "ms": arr[i].ms, "bytes": arr[i].bytes}
                for i in range(min(cnt.value, 32))}

    def diagnostics(self, reset: bool = True) -> dict:
        """Counters of the blocked search since the last reset."""
        out = np.zeros(48, np.int64)
        check_gpu(self.lib.mcbgpu_solver_diagnostics(self._h, ptr(out), 48, int(reset)), "mcbgpu_solver_diagnostics")
        keys = ["pivot_steps", "local_pivots", "merge_candidates", "tiles_loaded", "tiles_computed", "blocks",
                "cycles_scan", "cycles_barrier", "cycles_merge", "timeout_cta_plus1", "timeout_step", "timeout_rank",
                "timeout_gen", "timeout_count", "max_barriers_per_cta", "min_barriers_per_cta", "diverged",
                "div_step", "div_cta", "div_epoch", "cycles_tail_resolve", "cycles_tail_barrier",
                "cycles_tail_tables", "far_rows_gathered", "profile_0", "profile_1", "profile_2", "profile_3",
                "profile_4", "far_beta_bits", "far_rows_changed", "far_pair_words", "far_rows_touched",
                "merge_profile_0", "merge_profile_1", "merge_profile_2", "merge_profile_3", "merge_profile_4",
                "far_sparse_rows", "far_sparse_words", "far_sparse_tests"]
        return dict(zip(keys, out.tolist()))

    SHAPE_SEGMENTS = 4
    SHAPE_INTS = 7
    SHAPE_FIELDS = ("win_early", "rank_early", "win_mid", "rank_tail", "win_tail", "lmax", "stream_pct")

    def shapes(self) -> dict:
        """The candidate search shapes and the shape each segment of a solve uses."""
        n = C.c_int32()
        params = np.zeros(16 * self.SHAPE_INTS, np.int32)
        seg = np.zeros(self.SHAPE_SEGMENTS, np.int32)
        check_gpu(self.lib.mcbgpu_solver_shapes(self._h, ptr(params), 16, C.byref(n), ptr(seg)), "mcbgpu_solver_shapes")
        cands = [dict(zip(self.SHAPE_FIELDS, params[k * self.SHAPE_INTS:(k + 1) * self.SHAPE_INTS].tolist()))
                 for k in range(min(n.value, 16))]
        return {"candidates": cands, "segment_shape": seg.tolist()}

    def tune(self, stream=0) -> dict:
        """One complete blocked run with the candidate shapes taking turns group by group;
        each segment of the solve keeps the fastest.  The run's results stay readable."""
        info = self.shapes()
        n = len(info["candidates"])
        ms = np.zeros(self.SHAPE_SEGMENTS * n, np.float64)
        chosen = np.zeros(self.SHAPE_SEGMENTS, np.int32)
        check_gpu(self.lib.mcbgpu_solver_tune(self._h, ptr(ms), ptr(chosen), _stream(stream)), "mcbgpu_solver_tune")
        info["ms_per_block"] = ms.reshape(self.SHAPE_SEGMENTS, n).round(4).tolist()
        info["segment_shape"] = chosen.tolist()
        return info

    def set_shape(self, shape: int) -> None:
        """Force one candidate shape for every block (-1: the per-segment choice)."""
        check_gpu(self.lib.mcbgpu_solver_set_shape(self._h, int(shape)), "mcbgpu_solver_set_shape")

    @property
    def launches(self) -> int:
        return int(self.lib.mcbgpu_solver_launches(self._h))

    @property
    def device_bytes(self) -> int:
        return int(self.lib.mcbgpu_solver_device_bytes(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            check_gpu(self.lib.mcbgpu_solver_destroy(self._h), "mcbgpu_solver_destroy")
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve(num_coords: int, weight: np.ndarray, offsets: np.ndarray, coords: np.ndarray):
    """One-shot C-ABI call with host buffers: (selected[N], total weight)."""
    lib = gpu_lib()
    w = np.ascontiguousarray(weight, np.int32)
    o = np.ascontiguousarray(offsets, np.int64)
    c = np.ascontiguousarray(coords, np.int32)
    sel = np.full(max(num_coords, 1), -1, np.int64)
    tot = C.c_int64()
    check_gpu(lib.mcbgpu_solve(num_coords, w.shape[0], ptr(w), ptr(o), ptr(c), ptr(sel), C.byref(tot)),
              "mcbgpu_solve")
    return sel[:num_coords], tot.value


class BatchSolver:
    """Many independent de Pina problems in one persistent launch (one CTA per problem).

    `problems` is a list of (num_coords, weight, offsets, coords) tuples, each as
    Solver takes it (offsets local to the problem, starting at 0).  Every problem's
    result equals Solver.run's on the same arrays; problems with N above
    max_coords() are rejected (solve those with Solver)."""

    def __init__(self, problems, stream=0, upload: bool = True):
        self.lib = gpu_lib()
        self.count = len(problems)
        self.N = np.array([int(p[0]) for p in problems], np.int32)
        self.K = np.array([len(p[1]) for p in problems], np.int64)
        ws, offs, cos = [], [], []
        base = 0
        for n, w, o, c in problems:
            o = np.asarray(o, np.int64)
            ws.append(np.asarray(w, np.int32))
            offs.append(o[:-1] + base)
            cos.append(np.asarray(c, np.int32)[: int(o[-1])])
            base += int(o[-1])
        self.weight = np.ascontiguousarray(np.concatenate(ws) if ws else np.zeros(0, np.int32))
        self.offsets = np.ascontiguousarray(np.concatenate(offs + [np.array([base], np.int64)]))
        self.coords = np.ascontiguousarray(np.concatenate(cos) if cos else np.zeros(0, np.int32))
        self.nnz = base
        h = C.c_void_p()
        check_gpu(self.lib.mcbgpu_batch_create(C.byref(h), self.count, ptr(self.N), ptr(self.K), self.nnz),
                  "mcbgpu_batch_create")
        self._h = h
        if upload:
            self.upload(stream)

    @staticmethod
    def max_coords() -> int:
        return int(gpu_lib().mcbgpu_batch_max_coords())

    @classmethod
    def from_problems(cls, probs, stream=0) -> "BatchSolver":
        """From prepared host Problems (none of them a single cycle)."""
        items = []
        for p in probs:
            _, _, w, _ = p.candidates()
            off, co = p.cycle_lists()
            items.append((p.N, w, off, co))
        return cls(items, stream)

    def upload(self, stream=0) -> None:
        check_gpu(self.lib.mcbgpu_batch_upload(self._h, ptr(self.weight), ptr(self.offsets), ptr(self.coords),
                                               _stream(stream)), "mcbgpu_batch_upload")

    def run(self, stream=0) -> None:
        check_gpu(self.lib.mcbgpu_batch_run(self._h, _stream(stream)), "mcbgpu_batch_run")

    def results(self, stream=0):
        """([selected ranks per problem], total weights int64[count]) after synchronising `stream`."""
        sel = np.full(max(int(self.N.sum()), 1), -1, np.int64)
        tot = np.zeros(max(self.count, 1), np.int64)
        check_gpu(self.lib.mcbgpu_batch_results(self._h, ptr(sel), ptr(tot), None, _stream(stream)),
                  "mcbgpu_batch_results")
        bounds = np.concatenate([[0], np.cumsum(self.N.astype(np.int64))])
        return [sel[bounds[i]:bounds[i + 1]] for i in range(self.count)], tot[: self.count]

    def status(self, stream=0) -> np.ndarray:
        """Per-problem status words (0 = solved), without raising."""
        st = np.zeros(max(self.count, 1), np.uint32)
        self.lib.mcbgpu_batch_results(self._h, None, None, ptr(st), _stream(stream))
        return st[: self.count]

    def support_vector(self, problem: int, j: int, stream=0) -> np.ndarray:
        out = np.zeros((int(self.N[problem]) + 63) // 64, np.uint64)
        check_gpu(self.lib.mcbgpu_batch_get_support(self._h, problem, j, ptr(out), _stream(stream)),
                  "mcbgpu_batch_get_support")
        return out

    def set_profiling(self, enable: bool = True) -> None:
        check_gpu(self.lib.mcbgpu_batch_set_profiling(self._h, int(enable)), "mcbgpu_batch_set_profiling")

    def profile(self) -> np.ndarray:
        """Per problem: [ns, cycles in T, scan, resolve, final rows, update, candidates scanned, SM,
        cycles of the scan's list walks, pivot rounds, warp 0's update cycles in D + beta, in row writes,
        bytes the list walks read]."""
        out = np.zeros((max(self.count, 1), 13), np.int64)
        check_gpu(self.lib.mcbgpu_batch_profile(self._h, ptr(out)), "mcbgpu_batch_profile")
        return out[: self.count]

    @property
    def launches(self) -> int:
        return int(self.lib.mcbgpu_batch_launches(self._h))

    @property
    def device_bytes(self) -> int:
        return int(self.lib.mcbgpu_batch_device_bytes(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            check_gpu(self.lib.mcbgpu_batch_destroy(self._h), "mcbgpu_batch_destroy")
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_batch(problems):
    """One-shot C-ABI call: ([selected per problem], total weights)."""
    b = BatchSolver(problems)
    b.run()
    out = b.results()
    b.close()
    return out


class GpuTrees:
    """Shortest-path trees of many roots on the GPU (mcbgpu_trees_*): distances,
    parent slots by the reference's rule, and a per-root tie flag (1: the host must
    search that root itself).  The graph is a prepared Problem's reduced graph."""

    def __init__(self, nodes: int, row_offsets, cols, weights, rev, max_roots: int):
        self.lib = gpu_lib()
        self.n = int(nodes)
        self.max_roots = int(max_roots)
        ro = np.ascontiguousarray(row_offsets, np.uint32)
        c = np.ascontiguousarray(cols, np.uint32)
        w = np.ascontiguousarray(weights, np.int32)
        r = np.ascontiguousarray(rev, np.uint32)
        h = C.c_void_p()
        check_gpu(self.lib.mcbgpu_trees_create(C.byref(h), self.n, len(c), ptr(ro), ptr(c), ptr(w), ptr(r),
                                               self.max_roots), "mcbgpu_trees_create")
        self._h = h

    @classmethod
    def from_problem(cls, p, max_roots: int) -> "GpuTrees":
        rows, cols, w, rev, ro = p.reduced_graph()
        return cls(p.n, ro, cols, w, rev, max_roots)

    def run(self, roots, stream=0):
        """(dist int32[count, n], parent_slot int32[count, n], tied uint8[count])."""
        r = np.ascontiguousarray(roots, np.uint32)
        k = len(r)
        dist = np.empty((max(k, 1), self.n), np.int32)
        ps = np.empty((max(k, 1), self.n), np.int32)
        tied = np.empty(max(k, 1), np.uint8)
        check_gpu(self.lib.mcbgpu_trees_run(self._h, ptr(r), k, ptr(dist), ptr(ps), ptr(tied), _stream(stream)),
                  "mcbgpu_trees_run")
        return dist[:k], ps[:k], tied[:k]

    @property
    def device_bytes(self) -> int:
        return int(self.lib.mcbgpu_trees_device_bytes(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.mcbgpu_trees_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
