"""minimumcyclebasis_gb300 — the de Pina minimum-cycle-basis hot path on GB300 (sm_103a).

Host preparation (libmcbhost.so) reproduces the reference driver's reduced graph,
FVS, coordinate order and candidate rank order; the main loop runs on the GPU
(libmcbgpu.so) behind the C ABI in include/mcbgpu.h.
"""
from .host import (Graph, Problem, batch_graphs, bcc_split, block_tree_graph, grid_graph,  # noqa: F401
                   planar_chain_graph, prepare_many, random_graph, rgg_graph)
from .gpu import BatchSolver, GpuStruct, GpuTrees, Solver, device_info, solve, solve_batch  # noqa: F401
from .devprep import DevicePrepared, GpuGen, prepare_on_device  # noqa: F401

__all__ = ["Graph", "Problem", "grid_graph", "random_graph", "rgg_graph", "planar_chain_graph",
           "block_tree_graph", "batch_graphs", "bcc_split", "prepare_many", "GpuStruct", "GpuTrees", "Solver",
           "BatchSolver", "solve_batch", "device_info", "solve", "GpuGen", "DevicePrepared", "prepare_on_device"]
