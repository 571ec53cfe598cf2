"""ctypes bindings of libmcbhost.so (include/mcbhost.h) and libmcbgpu.so (include/mcbgpu.h).

The libraries are built in-tree by minimumcyclebasis_gb300.build.  Loading the GPU
library needs only the CUDA runtime; calling a compute entry point needs a GPU.
There is no fallback: if a library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

LIBDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib")

_host = None
_gpu = None

vp = C.c_void_p
i32, i64, u64 = C.c_int32, C.c_int64, C.c_uint64
f32p = C.POINTER(C.c_float)


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char_p), ("launches", i64), ("ms", C.c_double), ("bytes", C.c_double)]


class MCBHOptions(C.Structure):
    _fields_ = [("threads", C.c_int), ("contract_chains", C.c_int), ("keep_trees", C.c_int),
                ("ref_layout", C.c_int), ("cycle_lists", C.c_int), ("structure_only", C.c_int)]


TREE_BEGIN = C.CFUNCTYPE(C.c_int, vp, i32, i64, vp, vp, vp, vp)
TREE_TREES = C.CFUNCTYPE(C.c_int, vp, vp, i32, vp, vp, vp)


class MCBHTreeSource(C.Structure):
    _fields_ = [("ctx", vp), ("begin", TREE_BEGIN), ("trees", TREE_TREES), ("chunk", i32), ("trust", i32)]


class MCBHInfo(C.Structure):
    _fields_ = [("nodes", i32), ("edges2", i64), ("single_cycle", i32), ("nodes_removed", i32),
                ("reduced_nodes", i32), ("reduced_edges2", i64), ("source_vertex", i32), ("fvs_size", i32),
                ("num_coords", i32), ("num_candidates", i64), ("cycle_nnz", i64), ("total_weight_input", i64),
                ("t_read", C.c_double), ("t_reduce", C.c_double), ("t_fvs", C.c_double),
                ("t_spanning", C.c_double), ("t_trees", C.c_double), ("t_collect", C.c_double),
                ("trees_supplied", i32)]


HOST_SYMBOLS = {
    "mcbh_problem_from_mtx": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
    "mcbh_problem_from_edges": (C.c_int, [i32, i64, vp, vp, vp, C.POINTER(vp)]),
    "mcbh_prepare": (C.c_int, [vp, C.POINTER(MCBHOptions)]),
    "mcbh_prepare_many": (C.c_int, [vp, i64, C.POINTER(MCBHOptions), vp]),
    "mcbh_gf2_rank": (C.c_int, [vp, vp, i64, C.c_int, C.POINTER(i64)]),
    "mcbh_prepare_with_trees": (C.c_int, [vp, C.POINTER(MCBHOptions), vp]),
    "mcbh_search_trees": (C.c_int, [vp, vp, i32, C.c_int, vp, vp]),
    "mcbh_get_pairs": (C.c_int, [vp, vp]),
    "mcbh_rank_candidates": (C.c_int, [vp, vp, vp, vp, C.c_int]),
    "mcbh_problem_free": (None, [vp]),
    "mcbh_get_info": (C.c_int, [vp, C.POINTER(MCBHInfo)]),
    "mcbh_get_reduced_graph": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "mcbh_get_fvs": (C.c_int, [vp, vp, vp]),
    "mcbh_get_vertex_map": (i32, [vp, vp]),
    "mcbh_get_coords": (C.c_int, [vp, vp, vp]),
    "mcbh_get_candidates": (C.c_int, [vp, vp, vp, vp, vp]),
    "mcbh_get_cycle_lists": (C.c_int, [vp, vp, vp]),
    "mcbh_get_tree_parents": (C.c_int, [vp, vp]),
    "mcbh_get_ref_layout": (C.c_int, [vp, vp, vp, vp, vp]),
    "mcbh_gen_grid": (i64, [i32, i32, i32, i32, u64, vp, vp, vp]),
    "mcbh_gen_random": (i64, [i32, i64, i32, i32, u64, vp, vp, vp]),
    "mcbh_gen_rgg": (i64, [i32, i32, u64, vp, vp, vp]),
    "mcbh_gen_planar_chains": (i64, [i32, i32, i32, i32, i32, i32, u64, vp, vp, vp, vp]),
    "mcbh_gen_block_tree": (i64, [i32, i32, i32, i32, i32, i32, i32, u64, vp, vp, vp, vp]),
    "mcbh_bcc_split": (i64, [i32, i64, vp, vp, vp]),
    "mcbh_edge_slot_order": (i64, [i32, i64, vp, vp, vp]),
    "mcbh_read_mtx": (i64, [C.c_char_p, vp, i64, vp, vp, vp]),
    "mcbh_write_mtx": (C.c_int, [C.c_char_p, i32, i64, vp, vp, vp]),
}

GPU_SYMBOLS = {
    "mcbgpu_last_error": (C.c_char_p, []),
    "mcbgpu_version": (C.c_int, []),
    "init_cuda": (None, []),
    "configure_grid": (C.c_size_t, [C.c_int, C.c_int]),
    "allocate_pinned_memory": (C.POINTER(C.c_uint32), [C.c_int, C.c_int]),
    "free_pinned_memory": (None, [vp]),
    "calculate_chunk_size": (C.c_size_t, [C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t]),
    "mcbgpu_init_cuda": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_size_t)]),
    "mcbgpu_allocate_pinned": (C.c_int, [C.c_size_t, C.POINTER(vp)]),
    "mcbgpu_free_pinned": (C.c_int, [vp]),
    "mcbgpu_struct_create": (C.c_int, [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_int]),
    "mcbgpu_struct_initialize_memory": (C.c_int, [vp, vp, vp, vp, vp]),
    "mcbgpu_struct_copy_support_vector": (C.c_int, [vp, vp, f32p]),
    "mcbgpu_struct_process_shortest_path": (C.c_int, [vp, vp, C.c_int, f32p]),
    "mcbgpu_struct_clear_memory": (C.c_int, [vp]),
    "mcbgpu_label_forest_noalloc": (C.c_int, [vp, vp, vp, vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp, vp]),
    "mcbgpu_solver_create": (C.c_int, [C.POINTER(vp), i32, i64, i64]),
    "mcbgpu_solver_upload": (C.c_int, [vp, vp, vp, vp, vp]),
    "mcbgpu_solver_upload_device": (C.c_int, [vp, vp, vp, vp, vp]),
    "mcbgpu_solver_verify": (C.c_int, [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), vp]),
    "mcbgpu_solver_reset": (C.c_int, [vp, vp]),
    "mcbgpu_select": (C.c_int, [vp, i32, C.POINTER(i64), vp]),
    "mcbgpu_cycle_vector": (C.c_int, [vp, i32, vp, vp]),
    "mcbgpu_update": (C.c_int, [vp, i32, vp]),
    "mcbgpu_solver_run": (C.c_int, [vp, i64, vp]),
    "mcbgpu_solver_run_graph": (C.c_int, [vp, i64, vp]),
    "mcbgpu_solver_run_plain": (C.c_int, [vp, i64, vp]),
    "mcbgpu_solver_results": (C.c_int, [vp, vp, i64, C.POINTER(i64), vp]),
    "mcbgpu_solver_get_support": (C.c_int, [vp, i32, vp, vp]),
    "mcbgpu_solver_set_profiling": (C.c_int, [vp, C.c_int]),
    "mcbgpu_solver_kernel_stats": (C.c_int, [vp, vp, C.c_int, C.POINTER(C.c_int)]),
    "mcbgpu_solver_diagnostics": (C.c_int, [vp, vp, C.c_int, C.c_int]),
    "mcbgpu_solver_tune": (C.c_int, [vp, vp, vp, vp]),
    "mcbgpu_solver_set_shape": (C.c_int, [vp, i32]),
    "mcbgpu_solver_shapes": (C.c_int, [vp, vp, i32, C.POINTER(i32), vp]),
    "mcbgpu_solver_launches": (i64, [vp]),
    "mcbgpu_solver_device_bytes": (i64, [vp]),
    "mcbgpu_solver_destroy": (C.c_int, [vp]),
    "mcbgpu_solve": (C.c_int, [i32, i64, vp, vp, vp, vp, C.POINTER(i64)]),
    "mcbgpu_batch_max_coords": (C.c_int, []),
    "mcbgpu_batch_create": (C.c_int, [C.POINTER(vp), i32, vp, vp, i64]),
    "mcbgpu_batch_upload": (C.c_int, [vp, vp, vp, vp, vp]),
    "mcbgpu_batch_run": (C.c_int, [vp, vp]),
    "mcbgpu_batch_results": (C.c_int, [vp, vp, vp, vp, vp]),
    "mcbgpu_batch_get_support": (C.c_int, [vp, i32, i32, vp, vp]),
    "mcbgpu_batch_set_profiling": (C.c_int, [vp, C.c_int]),
    "mcbgpu_batch_profile": (C.c_int, [vp, vp]),
    "mcbgpu_batch_launches": (i64, [vp]),
    "mcbgpu_batch_device_bytes": (i64, [vp]),
    "mcbgpu_batch_destroy": (C.c_int, [vp]),
    "mcbgpu_trees_create": (C.c_int, [C.POINTER(vp), i32, i64, vp, vp, vp, vp, i32]),
    "mcbgpu_trees_run": (C.c_int, [vp, vp, i32, vp, vp, vp, vp]),
    "mcbgpu_trees_device_bytes": (i64, [vp]),
    "mcbgpu_trees_destroy": (C.c_int, [vp]),
    "mcbgpu_batch_solve": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, vp]),
    "mcbgpu_gen_create": (C.c_int, [C.POINTER(vp), i32, i64, vp, vp, vp, vp, vp, vp, i32, vp, vp, i32, vp, i32]),
    "mcbgpu_gen_trees": (C.c_int, [vp, i32, i32, vp, vp]),
    "mcbgpu_gen_trees_submit": (C.c_int, [vp, i32, i32, vp]),
    "mcbgpu_gen_trees_collect": (C.c_int, [vp, i32, vp, vp]),
    "mcbgpu_gen_tuning": (C.c_int, [vp]),
    "mcbgpu_gen_put_trees": (C.c_int, [vp, vp, i32, vp, vp, vp]),
    "mcbgpu_gen_candidates": (C.c_int, [vp, vp, C.POINTER(i64), vp]),
    "mcbgpu_gen_fetch": (C.c_int, [vp, i64, vp, vp, vp]),
    "mcbgpu_gen_rank": (C.c_int, [vp, i64, vp, vp, vp, vp, vp]),
    "mcbgpu_gen_build_lists": (C.c_int, [vp, i64, C.POINTER(i64), vp]),
    "mcbgpu_gen_lists": (C.c_int, [vp, i64, vp, vp, vp, C.POINTER(i64), vp]),
    "mcbgpu_gen_get_lists": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)]),
    "mcbgpu_gen_copy_lists": (C.c_int, [vp, vp, vp, vp]),
    "mcbgpu_gen_tree_shapes": (C.c_int, [vp, vp, vp, i32, C.POINTER(i32), C.POINTER(i32)]),
    "mcbgpu_gen_release_trees": (C.c_int, [vp]),
    "mcbgpu_gen_device_bytes": (i64, [vp]),
    "mcbgpu_gen_destroy": (C.c_int, [vp]),
    "mcbgpu_mlp_param_count": (C.c_int, []),
    "mcbgpu_mlp_create": (C.c_int, [C.POINTER(vp), vp]),
    "mcbgpu_mlp_get_params": (C.c_int, [vp, vp]),
    "mcbgpu_mlp_forward": (C.c_int, [vp, vp, i64, vp, vp]),
    "mcbgpu_mlp_gradients": (C.c_int, [vp, vp, vp, i64, C.c_float, vp, C.POINTER(C.c_float), vp]),
    "mcbgpu_mlp_train_step": (C.c_int, [vp, vp, vp, i64, C.c_float, C.c_float, C.POINTER(C.c_float), vp]),
    "mcbgpu_mlp_destroy": (C.c_int, [vp]),
}


def _bind(lib, table):
    for name, (res, args) in table.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def host_lib():
    global _host
    if _host is None:
        path = os.path.join(LIBDIR, "libmcbhost.so")
        if not os.path.exists(path):
            raise RuntimeError("libmcbhost.so is not built (run minimumcyclebasis_gb300.build.build_all())")
        _host = _bind(C.CDLL(path), HOST_SYMBOLS)
    return _host


def gpu_lib():
    global _gpu
    if _gpu is None:
        path = os.path.join(LIBDIR, "libmcbgpu.so")
        if not os.path.exists(path):
            raise RuntimeError("libmcbgpu.so is not built (run minimumcyclebasis_gb300.build.build_all())")
        _gpu = _bind(C.CDLL(path), GPU_SYMBOLS)
    return _gpu


class MCBError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str = ""):
        super().__init__("%s failed with %d%s" % (where, code, (": " + msg) if msg else ""))
        self.code = code


def check_host(rc: int, where: str) -> None:
    if rc != 0:
        raise MCBError(rc, where)


def check_gpu(rc: int, where: str) -> None:
    if rc != 0:
        msg = gpu_lib().mcbgpu_last_error()
        raise MCBError(rc, where, msg.decode() if msg else "")


def ptr(a) -> C.c_void_p:
    """Address of a numpy array (or None)."""
    if a is None:
        return None
    return C.c_void_p(a.ctypes.data)
