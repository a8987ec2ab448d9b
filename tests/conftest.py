import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running test")


@pytest.fixture(scope="session")
def known_answers():
    with open(os.path.join(GOLDEN, "regression_known_answers.json")) as fp:
        return json.load(fp)


@pytest.fixture(scope="session")
def shipped_deck():
    with open(os.path.join(GOLDEN, "shipped_deck.json")) as fp:
        return json.load(fp)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def imex():
    import imexlbm_gb300 as m
    from imexlbm_gb300 import build
    build.build()
    m.load()
    return m


def gpu_available() -> bool:
    try:
        import ctypes
        cudart = None
        for name in ("libcuda.so.1", "libcuda.so"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return False
        n = ctypes.c_int(0)
        if cudart.cuInit(0) != 0:
            return False
        return cudart.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False
