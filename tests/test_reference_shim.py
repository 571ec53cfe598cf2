"""The reference-side binding of the gpu_struct layer (include/reference_shim/gpu/):
the reference's own GPU driver, mcb/mcb_cycle_deg_two_remove.cpp, compiles unchanged
against the shim headers in place of gpu/common.cuh and gpu/gpu_struct.cuh and links
against libmcbgpu.so.  Compile and link only (no GPU is needed); runs where the
reference's sources were found by the oracle recipe (oracle/_ref/ref_path)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_PATH = os.path.join(ROOT, "oracle", "_ref", "ref_path")


def reference_checkout():
    if not os.path.exists(REF_PATH):
        return None
    ref = open(REF_PATH).read().strip()
    return ref if os.path.isdir(os.path.join(ref, "mcb")) else None


@pytest.mark.skipif(reference_checkout() is None, reason="reference sources not found (oracle recipe not run)")
def test_reference_driver_links_against_the_shim(tmp_path):
    ref = reference_checkout()
    lib = os.path.join(ROOT, "minimumcyclebasis_gb300", "lib")
    ct = os.path.join(ROOT, "oracle", "_ref", "ct.o")
    assert os.path.exists(os.path.join(lib, "libmcbgpu.so")) and os.path.exists(ct)
    srcs = [os.path.join(ref, "mcb", "mcb_cycle_deg_two_remove.cpp")] + [
        os.path.join(ref, "include", f) for f in ("mmio.cpp", "Host_Timer.cpp", "CsrGraphSpanningTree.cpp",
                                                  "CsrGraphDegreeTwoRemoval.cpp", "CsrGraphMultiSpanningTree.cpp",
                                                  "FVS.cpp")]
    out = str(tmp_path / "mcb_cuda_shim")
    cmd = ["g++", "-std=c++11", "-fopenmp", "-fpermissive", "-w", "-include", "cmath", "-include", "cassert",
           "-DNDEBUG", "-I" + os.path.join(ROOT, "include", "reference_shim"), "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ref, "include"), "-I" + ref, "-O0", "-o", out] + srcs + [
        ct, "-L" + lib, "-lmcbgpu", "-Wl,-rpath," + lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # the driver's GPU symbols resolve to libmcbgpu.so, not to anything of the reference's gpu/ tree
    nm = subprocess.run(["nm", "-D", "--undefined-only", out], capture_output=True, text=True).stdout
    for sym in ("mcbgpu_struct_create", "mcbgpu_struct_process_shortest_path", "init_cuda", "calculate_chunk_size",
                "allocate_pinned_memory"):
        assert sym in nm, sym
