"""The allocation-free RR entry point against the regular device entry point.

accrqa_gb300_rr_dev_noalloc is for callers that may not allocate device
memory (hosts with a fixed memory arena, latency-bound serving loops): its
per-threshold counts live in a
scratch array compiled into the library instead of memory it allocates.
Here it is called through the C ABI twice in a row per case, and every result
must equal what the existing entry point accrqa_gb300_rr_counts_dev gives,
turned into RR the same way (count / nc^2 in double, cast to the series
dtype) -- bit for bit, the tolerance of the other RR parity tests.

The file name sorts last so that a run stopping at its first failure has run
every other test before this one.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry(lib):
    f = lib.accrqa_gb300_rr_dev_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64,
                  ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                  ctypes.c_int32, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


@pytest.mark.parametrize("dt,code", [(np.float32, 0), (np.float64, 1)])
def test_noalloc_rr_matches_regular_entry_point(gpu, dt, code):
    import torch

    from accrqa_gb300 import _lib, workloads

    f = _entry(_lib.handle())
    tdt = torch.float32 if dt == np.float32 else torch.float64
    n = 3000
    x = workloads.lorenz_x(n, 9).astype(dt)
    dx = torch.zeros(n + 128, dtype=tdt, device="cuda")
    dx[:n].copy_(torch.from_numpy(x))
    stream = torch.cuda.current_stream().cuda_stream
    for tau, emb, norm, nthr in [(1, 3, 1, 16), (2, 5, 2, 40), (3, 9, 1, 5)]:
        thr = np.linspace(0.05, 1.5, nthr).astype(dt)
        cnt = torch.zeros(nthr, dtype=torch.int64, device="cuda")
        gpu.rr_counts_dev(cnt.data_ptr(), dx.data_ptr(), code, n, tau, emb, thr, norm, stream)
        torch.cuda.synchronize()
        nc = n - (emb - 1) * tau
        want = (cnt.cpu().numpy().astype(np.float64) / float(nc * nc)).astype(dt)
        for _ in range(2):
            out = torch.full((nthr,), -1.0, dtype=tdt, device="cuda")
            rc = f(out.data_ptr(), dx.data_ptr(), code, n, tau, emb, thr.ctypes.data, nthr,
                   norm, stream)
            assert rc == 0, rc
            torch.cuda.synchronize()
            np.testing.assert_array_equal(out.cpu().numpy(), want)


def test_noalloc_rejects_too_many_thresholds(gpu):
    import torch

    from accrqa_gb300 import _lib

    f = _entry(_lib.handle())
    dx = torch.zeros(300 + 128, dtype=torch.float32, device="cuda")
    out = torch.zeros(1025, dtype=torch.float32, device="cuda")
    thr = np.linspace(0.0, 1.0, 1025).astype(np.float32)
    rc = f(out.data_ptr(), dx.data_ptr(), 0, 300, 1, 2, thr.ctypes.data, 1025, 1, 0)
    assert rc == 2   # ERR_INVALID_ARGUMENT
