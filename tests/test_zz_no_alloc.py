"""The allocation-free label entry point (mcbgpu_label_forest_noalloc).

Callers that cannot allocate device memory (a framework that owns every byte of
device memory through its own pool, a latency-critical loop that must not take the
synchronisation of cudaMalloc/cudaFree) pass their own buffers; the entry point
keeps its working memory in a static device array inside the library.  Its labels
must equal those of the allocating entry point, mcbgpu_struct_process_shortest_path,
bit for bit, on two calls in a row (the second reusing the array the first left
behind).  This file is collected last so that a stop-at-first-failure run has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_noalloc_labels_equal_allocating_entry_point_twice():
    import torch

    from minimumcyclebasis_gb300 import GpuStruct, Problem
    from minimumcyclebasis_gb300._native import gpu_lib

    torch.cuda.set_device(0)
    fx = load_golden("grid32x32_s1")
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=4, keep_trees=True, ref_layout=True)
    rows, _, _, _, _ = p.reduced_graph()
    _, ec = p.coords()
    lv, pp, eo, _ = p.ref_layout()
    n, F, N = p.n, p.F, p.N
    words = (N + 63) // 64
    rng = np.random.default_rng(11)

    gs = GpuStruct(rows.shape[0], N, n, F, chunk_size=720)
    gs.initialize_memory(ec, lv, pp, eo)

    dev = torch.device("cuda", 0)
    d_lv = torch.from_numpy(lv.view(np.int32)).to(dev)
    d_pp = torch.from_numpy(pp.view(np.int32)).to(dev)
    d_eo = torch.from_numpy(eo).to(dev)
    d_map = torch.from_numpy(ec).to(dev)
    d_out = torch.empty(F * n, dtype=torch.int32, device=dev)
    lib = gpu_lib()
    stream = torch.cuda.current_stream().cuda_stream

    for call in range(2):
        S = rng.integers(0, 2**63, size=words, dtype=np.int64)
        if N % 64:
            S[-1] &= (1 << (N % 64)) - 1
        d_S = torch.from_numpy(S).to(dev)
        d_out.fill_(7)
        rc = lib.mcbgpu_label_forest_noalloc(
            C.c_void_p(d_lv.data_ptr()), C.c_void_p(d_pp.data_ptr()), C.c_void_p(d_eo.data_ptr()),
            C.c_void_p(d_map.data_ptr()), rows.shape[0], C.c_void_p(d_S.data_ptr()), N, F, n,
            C.c_void_p(d_out.data_ptr()), C.c_void_p(stream))
        assert rc == 0, lib.mcbgpu_last_error()
        got = d_out.cpu().numpy().view(np.uint32).reshape(F, n)
        gs.copy_support_vector(S.view(np.uint64))
        want, _ = gs.process_shortest_path()
        assert np.array_equal(got, want), "call %d differs" % call
    gs.close()


def test_noalloc_flags_levels_that_end_early():
    # the array keeps the previous call's labels: a tree whose levels end before its
    # last position must not hand them out; the call reports bad input and those
    # positions read 0
    import torch

    from minimumcyclebasis_gb300 import Problem
    from minimumcyclebasis_gb300._native import gpu_lib

    torch.cuda.set_device(0)
    fx = load_golden("grid8x8_s3")
    p = Problem.from_mtx(fx["mtx"]).prepare(threads=4, keep_trees=True, ref_layout=True)
    rows, _, _, _, _ = p.reduced_graph()
    _, ec = p.coords()
    lv, pp, eo, _ = p.ref_layout()
    n, F, N = p.n, p.F, p.N
    lv = lv.reshape(F, n + 1).copy()
    cut = int(lv[0, 2])
    assert 1 < cut < n
    lv[0, 2:] = cut
    dev = torch.device("cuda", 0)
    d_lv = torch.from_numpy(lv.reshape(-1).view(np.int32)).to(dev)
    d_pp = torch.from_numpy(pp.view(np.int32)).to(dev)
    d_eo = torch.from_numpy(eo).to(dev)
    d_map = torch.from_numpy(ec).to(dev)
    d_S = torch.from_numpy(np.full((N + 63) // 64, -1, np.int64)).to(dev)
    d_out = torch.full((F * n,), 7, dtype=torch.int32, device=dev)
    lib = gpu_lib()
    rc = lib.mcbgpu_label_forest_noalloc(
        C.c_void_p(d_lv.data_ptr()), C.c_void_p(d_pp.data_ptr()), C.c_void_p(d_eo.data_ptr()),
        C.c_void_p(d_map.data_ptr()), rows.shape[0], C.c_void_p(d_S.data_ptr()), N, F, n,
        C.c_void_p(d_out.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc != 0 and b"status 0x8" in lib.mcbgpu_last_error()
    got = d_out.cpu().numpy().reshape(F, n)
    assert (got[0, cut:] == 0).all()


def test_noalloc_rejects_trees_beyond_the_scratch():
    from minimumcyclebasis_gb300._native import gpu_lib
    lib = gpu_lib()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.mcbgpu_label_forest_noalloc(dummy, dummy, dummy, dummy, 4, dummy, 1, 1, (16 << 20) + 1, dummy, None)
    assert rc != 0
    assert b"static scratch" in lib.mcbgpu_last_error()
