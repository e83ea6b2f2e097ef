"""Test configuration: the `gpu` marker and shared helpers.

Tests marked `gpu` need a CUDA device and call the engine through its C ABI;
every other test runs on the CPU (oracle, host logic, library loading).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def lib():
    from accrqa_gb300 import build
    build.build()
    import accrqa_gb300
    return accrqa_gb300.library()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu(lib):
    from accrqa_gb300 import engine
    if engine.device_count() < 1:
        pytest.fail("GPU test run without a CUDA device")
    return engine


def logistic(n, seed, r=3.9, transient=1000):
    rng = np.random.default_rng(seed)
    v = rng.uniform(0.1, 0.9)
    for _ in range(transient):
        v = r * v * (1.0 - v)
    out = np.empty(n)
    for i in range(n):
        v = r * v * (1.0 - v)
        out[i] = v
    return out
