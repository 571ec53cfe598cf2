"""The candidate sort (csrc/host/weight_sort.h): the parallel sort gives std::sort's
permutation of equal weights on random, tie-dense, presorted and adversarial
(depth-exhausting) inputs, with 1 to 16 threads; compiled with g++ and run."""
import os
import shutil
import subprocess
import tempfile

import pytest

from conftest import ROOT


def test_weight_sort_equals_std_sort():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    src = os.path.join(ROOT, "tests", "weight_sort_check.cpp")
    inc = os.path.join(ROOT, "minimumcyclebasis_gb300", "csrc", "host")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "weight_sort_check")
        subprocess.run([gxx, "-std=c++17", "-O2", "-fopenmp", "-I" + inc, "-o", exe, src], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
