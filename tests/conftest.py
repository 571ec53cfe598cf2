import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from minimumcyclebasis_gb300.build import build_driver, build_gpu, build_host, build_oracle
    build_host()
    build_oracle()
    build_gpu()
    build_driver()
    yield


def golden_names():
    with open(os.path.join(GOLDEN, "index.json")) as f:
        return json.load(f)


def load_golden(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        fx = json.load(f)
    fx["mtx"] = os.path.join(GOLDEN, name + ".mtx")
    return fx
