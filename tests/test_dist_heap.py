"""The tree searches' queues (csrc/host/dist_heap.h): DistHeap pops in the same order
as std::priority_queue with the reference's distance-only comparator
(include/Dijkstra.h:37-44), and RadixQueue gives out the same distances in the same
order on monotone sequences; compiled with g++ and run on random sequences dense in ties."""
import os
import shutil
import subprocess
import tempfile

import pytest

from conftest import ROOT


def test_tree_search_queues_against_the_standard_queue():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    src = os.path.join(ROOT, "tests", "dist_heap_check.cpp")
    inc = os.path.join(ROOT, "minimumcyclebasis_gb300", "csrc", "host")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "dist_heap_check")
        subprocess.run([gxx, "-std=c++17", "-O2", "-I" + inc, "-o", exe, src], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
