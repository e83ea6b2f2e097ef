"""GPU: CUDA failures surface as Accrqa_Error codes, without faulting the GPU.

The reference discards the CUDA errors of its GPU paths
(src/AccRQA_functions.cpp:161,175,229,879); this engine returns them.  The
failures are made on the host: a testing hook makes the engine's next device
allocations fail with an out-of-memory error before they reach the driver
(accrqa_gb300_test_fail_allocations), and a server whose memory share is too
small for any request must complete the request with the same code.  After
each failure the library must keep working and give the oracle's results.
"""
import ctypes

import numpy as np
import pytest

import accrqa_gb300 as A
from accrqa_gb300 import _lib, engine, workloads

pytestmark = pytest.mark.gpu
ERR_CUDA_NOT_ENOUGH_MEMORY = 9


@pytest.fixture
def faults():
    lib = _lib.handle()
    lib.accrqa_gb300_test_fail_allocations.argtypes = [ctypes.c_int32]
    yield lib.accrqa_gb300_test_fail_allocations
    lib.accrqa_gb300_test_fail_allocations(0)


def test_allocation_failure_surfaces_in_the_api(gpu, oracle_mod, faults):
    # a series larger than any the tests before used, so the call must allocate
    big = workloads.white(8_000_000, 3).astype(np.float32)
    thr = np.array([0.1], np.float32)
    faults(8)
    with pytest.raises(engine.EngineError) as ei:
        gpu.rr_counts(big, 1, 2, thr, 1)
    assert ei.value.code == ERR_CUDA_NOT_ENOUGH_MEMORY
    assert "cudaMalloc" in str(ei.value)
    # the reference-facing front-end raises with the engine's message
    faults(8)
    with pytest.raises(RuntimeError):
        A.RR(big, np.array([1], np.intc), np.array([2], np.intc), thr,
             A.accrqaDistance("euclidean"), tidy_data=False)
    faults(0)
    x = workloads.logistic(700, 5).astype(np.float32)
    thr = np.array([0.05, 0.2], np.float32)
    np.testing.assert_array_equal(gpu.rr_counts(x, 1, 3, thr, 1),
                                  oracle_mod.rr_counts(x, 1, 3, thr, 1))


def _job(n=3000, seed=1, measures=("det",)):
    x = workloads.ar1(n, seed).astype(np.float32)
    x = (x / np.std(x)).astype(np.float32)
    return dict(x=x, tau=1, emb=3, norm=1, thresholds=np.array([0.2, 0.5], np.float32),
                measures=measures)


def test_server_request_larger_than_its_share(gpu):
    with engine.Server(workers=1, hbm_fraction=1e-9) as srv:
        t = srv.submit(_job())
        with pytest.raises(engine.EngineError) as ei:
            srv.wait(t)
        assert ei.value.code == ERR_CUDA_NOT_ENOUGH_MEMORY


def test_server_allocation_failure_then_recovery(gpu, faults):
    with engine.Server(workers=1) as srv:
        faults(1)   # the admission's device block of the next request
        t = srv.submit(_job(seed=2))
        with pytest.raises(engine.EngineError) as ei:
            srv.wait(t)
        assert ei.value.code == ERR_CUDA_NOT_ENOUGH_MEMORY
        faults(0)
        j = _job(seed=2)
        out, _ = srv.wait(srv.submit(j))
        D = A.accrqaDistance("euclidean")
        want = A.DET(j["x"], np.array([1], np.intc), np.array([3], np.intc),
                     np.array([2], np.intc), j["thresholds"], D, tidy_data=False).reshape(-1, 5)
        np.testing.assert_array_equal(out["det"], want)
