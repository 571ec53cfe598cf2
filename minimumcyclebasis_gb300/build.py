"""Build recipe for the native libraries of minimumcyclebasis_gb300.

Everything is compiled in-tree (outputs under minimumcyclebasis_gb300/lib/ and
oracle/), with plain nvcc / g++ invocations run in parallel:

  lib/libmcbhost.so   host preprocessing (C++17, OpenMP)        csrc/host/mcb_host.cpp
  lib/libmcbgpu.so    sm_103a kernels + C ABI (nvcc)             csrc/gpu/*.cu
  lib/mcb_gb300       drop-in driver executable (C++ over both)  csrc/host/mcb_driver.cpp
  oracle/libmcboracle.so   CPU oracle (test infrastructure only)  oracle/mcb_oracle.cpp

`python -m minimumcyclebasis_gb300.build` builds all of them.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB = os.path.join(PKG, "lib")
INC = os.path.join(ROOT, "include")
CSRC = os.path.join(PKG, "csrc")
ORACLE = os.path.join(ROOT, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
GPU_SOURCES = ["mcbgpu_runtime.cu", "mcbgpu_labels.cu", "mcbgpu_solver.cu", "mcbgpu_batch.cu", "mcbgpu_trees.cu",
               "mcbgpu_gen.cu", "mcbgpu_mlp.cu"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmcbgpu.so")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    gdir = os.path.join(CSRC, "gpu")
    hs += [os.path.join(gdir, f) for f in os.listdir(gdir) if f.endswith(".cuh")]
    hdir = os.path.join(CSRC, "host")
    hs += [os.path.join(hdir, f) for f in os.listdir(hdir) if f.endswith(".h")]
    return hs


def build_host(force: bool = False) -> str:
    out = os.path.join(LIB, "libmcbhost.so")
    src = os.path.join(CSRC, "host", "mcb_host.cpp")
    if force or _stale(out, [src] + _headers()):
        _run(["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared", "-I" + INC, "-o", out, src])
    return out


def _defines() -> list[str]:
    """Tuning macros for the GPU library (MCB_DEFINES="-DMCB_NZ_CAP=64 ..."); only -D
    options are taken.  The default build uses none."""
    return [d for d in os.environ.get("MCB_DEFINES", "").split() if d.startswith("-D")]


def build_gpu(force: bool = False) -> str:
    out = os.path.join(LIB, "libmcbgpu.so")
    srcs = [os.path.join(CSRC, "gpu", f) for f in GPU_SOURCES]
    objdir = os.path.join(LIB, "obj")
    os.makedirs(objdir, exist_ok=True)
    stamp = os.path.join(objdir, "defines.txt")
    defines = _defines()
    same = os.path.exists(stamp) and open(stamp).read() == " ".join(defines)
    if not (force or not same or _stale(out, srcs + _headers())):
        return out
    nvcc = _nvcc()
    objs = []

    def compile_one(src: str) -> str:
        obj = os.path.join(objdir, os.path.basename(src).replace(".cu", ".o"))
        _run([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INC,
              "-I" + os.path.join(CSRC, "gpu"), *defines, "-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    _run([nvcc, *ARCH, "-shared", "-o", out, *objs, "-lcudart"])
    with open(stamp, "w") as f:
        f.write(" ".join(defines))
    return out


def build_driver(force: bool = False) -> str:
    out = os.path.join(LIB, "mcb_gb300")
    src = os.path.join(CSRC, "host", "mcb_driver.cpp")
    if not os.path.exists(src):
        return ""
    deps = [src, os.path.join(LIB, "libmcbhost.so"), os.path.join(LIB, "libmcbgpu.so")] + _headers()
    if force or _stale(out, deps):
        cuda = _cuda_home()
        _run(["g++", "-std=c++17", "-O2", "-fopenmp", "-I" + INC, "-I" + os.path.join(cuda, "include"),
              "-o", out, src, "-L" + LIB, "-lmcbhost", "-lmcbgpu", "-Wl,-rpath,$ORIGIN",
              "-L" + os.path.join(cuda, "lib64"), "-lcudart"])
    return out


def build_oracle(force: bool = False) -> str:
    """The CPU oracle (test infrastructure; never linked into the product)."""
    out = os.path.join(ORACLE, "libmcboracle.so")
    src = os.path.join(ORACLE, "mcb_oracle.cpp")
    if force or _stale(out, [src]):
        _run(["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", out, src])
    return out


def build_reference(ref: str | None = None) -> bool:
    """oracle/_ref: the reference's own CPU drivers, built from the reference checkout
    at `ref` (default: the MCB_REFERENCE environment variable), only where its sources
    exist."""
    ref = ref or os.environ.get("MCB_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "mcb")):
        return False
    _run(["make", "-s", "-C", ORACLE, "REF=" + ref, "-j4"])
    return True


def build_all(force: bool = False) -> dict:
    os.makedirs(LIB, exist_ok=True)
    with ThreadPoolExecutor(max_workers=3) as ex:
        fh = ex.submit(build_host, force)
        fg = ex.submit(build_gpu, force)
        fo = ex.submit(build_oracle, force)
        res = {"host": fh.result(), "gpu": fg.result(), "oracle": fo.result()}
    res["driver"] = build_driver(force)
    return res


if __name__ == "__main__":
    r = build_all(force="--force" in sys.argv)
    r["reference"] = build_reference(sys.argv[sys.argv.index("--ref") + 1] if "--ref" in sys.argv else None)
    print(r)
