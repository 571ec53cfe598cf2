"""The C-ABI libraries load and export every function their headers declare.
No compute call is made (no GPU needed)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADERS = {
    "mcbgpu.h": os.path.join(ROOT, "minimumcyclebasis_gb300", "lib", "libmcbgpu.so"),
    "mcbhost.h": os.path.join(ROOT, "minimumcyclebasis_gb300", "lib", "libmcbhost.so"),
}


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = []
    for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_\s\*]*?)\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{]*?)\)\s*;", text):
        ret, name = m.group(1).strip(), m.group(2)
        if not ret or ret.startswith("typedef") or name in ("if", "while", "for", "return"):
            continue
        names.append(name)
    return names


@pytest.mark.parametrize("header", sorted(HEADERS))
def test_library_exports_every_declared_function(header):
    names = declared_functions(header)
    assert len(names) >= 10
    lib = ctypes.CDLL(HEADERS[header])
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_gpu_layer_names_are_exported():
    # gpu/common.cuh:18-27 of the reference
    lib = ctypes.CDLL(HEADERS["mcbgpu.h"])
    for n in ["init_cuda", "configure_grid", "allocate_pinned_memory", "free_pinned_memory",
              "calculate_chunk_size"]:
        assert hasattr(lib, n)


def test_python_bindings_cover_the_headers():
    from minimumcyclebasis_gb300 import _native
    for header, table in (("mcbgpu.h", _native.GPU_SYMBOLS), ("mcbhost.h", _native.HOST_SYMBOLS)):
        assert set(declared_functions(header)) == set(table), header


def test_error_string_without_gpu():
    from minimumcyclebasis_gb300._native import gpu_lib
    lib = gpu_lib()
    assert lib.mcbgpu_version() == 1
    assert lib.mcbgpu_last_error() is not None


def test_size_checks_before_any_device_call():
    # argument checks run before the library touches the device, so they answer on
    # a machine without a GPU
    import ctypes as C

    import numpy as np

    from minimumcyclebasis_gb300._native import gpu_lib, ptr
    lib = gpu_lib()
    h = C.c_void_p()
    big = np.array([lib.mcbgpu_batch_max_coords() + 1], np.int32)
    k = np.array([1], np.int64)
    assert lib.mcbgpu_batch_create(C.byref(h), 1, ptr(big), ptr(k), 1) == -1
    assert b"mcbgpu_solver" in lib.mcbgpu_last_error()  # points to the single-problem solver
    neg = np.array([-1], np.int32)
    assert lib.mcbgpu_batch_create(C.byref(h), 1, ptr(neg), ptr(k), 1) == -1
    assert lib.mcbgpu_batch_create(None, 0, None, None, 0) == -1
    assert lib.mcbgpu_solver_create(C.byref(h), 1 << 26, 1, 1) == -1
    assert lib.mcbgpu_batch_max_coords() == 12288
