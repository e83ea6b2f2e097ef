"""GPU tests of the reference-facing API (py_accrqa_* / R_double_accrqa_* / RP).

Outputs of RR, DET and LAM in the reference's GPU output layout against the
oracle: derived ratios within 1e-6 relative (float32) and 1e-12 (float64);
line lengths (Lmax/TTmax) exactly.  Both output conventions of DET/LAM (all
five measures, and the calc_ENTR = 0 convention with NaN Lmax/ENTR and RR over
(nc-1)^2).  Full-size properties at the benchmark's N where the oracle would
take hours: two independent kernels must agree on the recurrent-cell count.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import accrqa_gb300 as A
from accrqa_gb300 import workloads

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RTOL = {np.float32: 1e-6, np.float64: 1e-12}


def _close(got, want, dt):
    """Ratios within the dtype's tolerance; NaNs must match."""
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    m = ~np.isnan(want)
    np.testing.assert_allclose(got[m], want[m], rtol=RTOL[dt], atol=0)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("norm", ["euclidean", "maximal"])
def test_rr_api(gpu, oracle_mod, dt, norm):
    x = workloads.lorenz_x(900, 17, transient=300).astype(dt)
    taus = np.array([1, 3], np.intc)
    embs = np.array([2, 4, 9], np.intc)
    thr = np.array([0.05, 0.2, 0.6, 1.2], dt)
    out = A.RR(x, taus, embs, thr, A.accrqaDistance(norm), tidy_data=False)
    d = 1 if norm == "euclidean" else 2
    for a, t in enumerate(taus):
        for b, e in enumerate(embs):
            nc = len(x) - (e - 1) * t
            want = oracle_mod.rr_output(oracle_mod.rr_counts(x, t, e, thr, d), nc, dt)
            np.testing.assert_array_equal(out[a, b], want)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("kind", ["DET", "LAM"])
@pytest.mark.parametrize("entr", [True, False])
def test_line_api(gpu, oracle_mod, dt, kind, entr):
    x = workloads.ar1(700, 5).astype(dt)
    x = (x / np.std(x)).astype(dt)
    taus = np.array([1, 2], np.intc)
    embs = np.array([3, 5], np.intc)
    lm = np.array([1, 2, 5], np.intc)
    thr = np.array([0.1, 0.35, 0.8], dt)
    for norm, d in (("euclidean", 1), ("maximal", 2)):
        f = A.DET if kind == "DET" else A.LAM
        out = f(x, taus, embs, lm, thr, A.accrqaDistance(norm), calculate_ENTR=entr,
                tidy_data=False)
        want = oracle_mod.line_output(x, taus, embs, lm, thr, d, 1 if entr else 0,
                                      kind == "DET")
        _close(out, want, dt)


def test_long_lmin_selects_full_convention(gpu, oracle_mod):
    """calc_ENTR = 0 with lmin >= 16 still reports Lmax/ENTR (reference dispatch)."""
    x = workloads.lorenz_x(600, 2, transient=200).astype(np.float64)
    lm = np.array([2, 16], np.intc)
    thr = np.array([0.3], np.float64)
    out = A.DET(x, np.array([1], np.intc), np.array([3], np.intc), lm, thr,
                A.accrqaDistance("euclidean"), calculate_ENTR=False, tidy_data=False)
    want = oracle_mod.line_output(x, [1], [3], lm, thr, 1, 0, True)
    _close(out, want, np.float64)
    assert not np.isnan(out[..., 2]).any()


def test_crqa_known_answers_on_gpu(gpu):
    x = np.load(os.path.join(GOLD, "crqa_input.npy"))
    kat = json.load(open(os.path.join(GOLD, "crqa_kat.json")))["cases"]
    for dist, name in (("1", "euclidean"), ("2", "maximal")):
        D = A.accrqaDistance(name)
        for row in kat["DET"][dist]:
            o = A.DET(x, np.array([int(row["tau"])], np.intc), np.array([int(row["emb"])], np.intc),
                      np.array([int(row["lmin"])], np.intc), np.array([row["thr"]]), D,
                      tidy_data=False).ravel()
            for i, key in ((0, "CRQA_DET"), (1, "CRQA_L"), (3, "CRQA_ENTR"), (4, "CRQA_RR")):
                assert abs(o[i] - row[key]) <= 1e-4
        for row in kat["LAM"][dist]:
            o = A.LAM(x, np.array([int(row["tau"])], np.intc), np.array([int(row["emb"])], np.intc),
                      np.array([int(row["vmin"])], np.intc), np.array([row["thr"]]), D,
                      tidy_data=False).ravel()
            for i, key in ((0, "CRQA_LAM"), (1, "CRQA_TT"), (4, "CRQA_RR")):
                assert abs(o[i] - row[key]) <= 1e-4
        for row in kat["RR"][dist]:
            o = A.RR(x, np.array([int(row["tau"])], np.intc), np.array([int(row["emb"])], np.intc),
                     np.array([row["thr"]]), D, tidy_data=False).ravel()
            assert abs(o[0] - row["CRQA_RR"]) <= 1e-4


def test_rp_api(gpu, oracle_mod):
    x = workloads.logistic(500, 4).astype(np.float64)
    got = A.RP(x, 2, 3, 0.3, A.accrqaDistance("maximal"))
    # the Python shim holds a double threshold in a float, as the reference does
    want = oracle_mod.rp(x, 2, 3, float(np.float32(0.3)), 2)
    np.testing.assert_array_equal(got, want)
    x32 = x.astype(np.float32)
    np.testing.assert_array_equal(A.RP(x32, 1, 4, 0.25, A.accrqaDistance("euclidean")),
                                  oracle_mod.rp(x32, 1, 4, 0.25, 1))


def test_r_shims(gpu, oracle_mod):
    L = A.library()
    x = workloads.logistic(400, 8)
    n = ctypes.c_int(len(x))
    taus = np.array([1, 2], np.intc)
    embs = np.array([2, 3], np.intc)
    lm = np.array([2], np.intc)
    thr = np.array([0.1, 0.3])
    ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    one = lambda v: ctypes.byref(ctypes.c_int(v))
    out = np.zeros(2 * 2 * 1 * 2 * 5)
    L.R_double_accrqa_DET(dp(out), dp(x), ctypes.byref(n), ip(taus), one(2), ip(embs), one(2),
                          ip(lm), one(1), dp(thr), one(2), one(2), one(1), one(1024))
    _close(out.reshape(2, 2, 1, 2, 5), oracle_mod.line_output(x, taus, embs, lm, thr, 2, 1, True),
           np.float64)
    out = np.zeros(2 * 2 * 1 * 2 * 5)
    L.R_double_accrqa_LAM(dp(out), dp(x), ctypes.byref(n), ip(taus), one(2), ip(embs), one(2),
                          ip(lm), one(1), dp(thr), one(2), one(1), one(1), one(1024))
    _close(out.reshape(2, 2, 1, 2, 5), oracle_mod.line_output(x, taus, embs, lm, thr, 1, 1, False),
           np.float64)
    rr = np.zeros(8)
    L.R_double_accrqa_RR(dp(rr), dp(x), ctypes.byref(n), ip(taus), one(2), ip(embs), one(2),
                         dp(thr), one(2), one(1), one(1024))
    for a, t in enumerate(taus):
        for b, e in enumerate(embs):
            nc = len(x) - (e - 1) * t
            np.testing.assert_array_equal(
                rr.reshape(2, 2, 2)[a, b],
                oracle_mod.rr_output(oracle_mod.rr_counts(x, t, e, thr, 1), nc, np.float64))
    rp = np.zeros((len(x) - 2) ** 2, np.intc)
    thv = ctypes.c_double(0.2)
    L.R_double_accrqa_RP(ip(rp), dp(x), ctypes.byref(n), one(2), one(2), ctypes.byref(thv), one(1))
    np.testing.assert_array_equal(rp.reshape(len(x) - 2, -1), oracle_mod.rp_i32(x, 2, 2, 0.2, 1))


@pytest.mark.parametrize("n,tau,emb", [(200_000, 1, 3), (200_000, 8, 8), (1_000_000, 1, 5)])
def test_full_size_count_consistency(gpu, n, tau, emb):
    """RR counts (rr_rows), the LAM histograms' recurrent cells (lam_rows) and the
    DET histograms' (det_diags, upper triangle doubled + line of identity) are
    three different kernels; on finite data they must agree exactly."""
    x = workloads.lorenz_x(n, 77).astype(np.float32) if n <= 200_000 else \
        workloads.white(n, 77).astype(np.float32)
    thr = np.array([0.05, 0.2, 0.5], np.float32)
    rr = gpu.rr_counts(x, tau, emb, thr, 1)
    lam = gpu.lam_histograms(x, tau, emb, thr, 1)
    det = gpu.det_histograms(x, tau, emb, thr, 1)
    lengths = np.arange(lam.shape[1], dtype=np.uint64)
    np.testing.assert_array_equal((lam * lengths).sum(axis=1), rr)
    np.testing.assert_array_equal((det * lengths).sum(axis=1), rr)
    nc = n - (emb - 1) * tau
    assert (det[:, nc] == 1).all()


def _rr_target_one_step_per_call(x, tau, emb, target, D, epsilon, max_iter, tmin, tmax):
    """The reference's RR_target loop (src/accrqa/accrqa.py:555-594), one RR
    call per bisection step."""
    t_ = np.array([tau], np.intc)
    e_ = np.array([emb], np.intc)

    def rr(ts):
        return A.RR(x, t_, e_, np.array(ts, np.float32).astype(x.dtype), D,
                    tidy_data=False).flatten()

    mid = (tmax - tmin) / 2.0 + tmin
    v = rr([tmin, mid, tmax])
    low, hgh, cur = v[0], v[2], v[1]
    for _ in range(1, max_iter + 1):
        mid = (tmax - tmin) / 2.0 + tmin
        cur = rr([mid])[0]
        if abs(cur - target) < epsilon or (hgh - low) < epsilon:
            return mid, cur
        if cur < target:
            tmin = mid
        else:
            tmax = mid
    return (tmax - tmin) / 2.0 + tmin, cur


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_rr_target_equals_one_step_per_call(gpu, dt):
    x = workloads.lorenz_x(3000, 5).astype(dt)
    x = (x / np.std(x.astype(np.float64))).astype(dt)
    D = A.accrqaDistance("euclidean")
    for target, eps, max_iter, tmin, tmax in [(0.05, 0.01, 20, 0.0, 10.0),
                                             (0.05, 1e-6, 20, 0.0, 10.0),
                                             (0.2, 1e-4, 7, 0.0, 5.0),
                                             (0.01, 1e-9, 30, 0.0, 10.0),
                                             (0.5, 1e-3, 3, 0.1, 4.0)]:
        got = A.RR_target(x, 2, 3, target, D, epsilon=eps, max_iter=max_iter,
                          threshold_min=tmin, threshold_max=tmax)
        want = _rr_target_one_step_per_call(x, 2, 3, target, D, eps, max_iter, tmin, tmax)
        assert got[0] == want[0] and got[1] == want[1], (target, eps, got, want)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_rp_bits_equal_byte_plot(gpu, dt):
    """The bit-packed plot (host and device-resident) holds the byte plot's
    cells, including a row length that is not a multiple of 32."""
    import torch
    from accrqa_gb300 import engine
    x = workloads.lorenz_x(1500, 4, transient=500).astype(dt)
    for norm in (1, 2):
        for tau, emb, t in [(1, 3, 0.4), (2, 5, 1.1), (3, 1, 0.0)]:
            nc = len(x) - (emb - 1) * tau
            full = engine.rp(x, tau, emb, t, norm)
            bits = engine.rp_bits(x, tau, emb, t, norm)
            assert bits.shape == (nc, (nc + 31) // 32)
            np.testing.assert_array_equal(engine.unpack_rp_bits(bits, nc), full)
            # padding bits past nc are zero
            if nc % 32:
                assert not np.any(bits[:, -1] >> np.uint32(nc % 32))
            dx = torch.zeros(len(x) + 128, dtype=torch.float32 if dt == np.float32 else torch.float64,
                             device="cuda")
            dx[:len(x)].copy_(torch.from_numpy(x))
            dout = torch.zeros(nc * ((nc + 31) // 32), dtype=torch.int32, device="cuda")
            s = torch.cuda.current_stream()
            engine.rp_bits_dev(dout.data_ptr(), dx.data_ptr(), 0 if dt == np.float32 else 1,
                               len(x), tau, emb, t, norm, s.cuda_stream)
            torch.cuda.synchronize()
            np.testing.assert_array_equal(dout.cpu().numpy().view(np.uint32).reshape(bits.shape),
                                          bits)


def test_logistic_10k_workload(gpu, oracle_mod):
    """The reference's CPU-runnable workload: logistic map N = 10,000 float32,
    tau 1, emb 3, maximal norm, thresholds linspace(0.05, 0.40, 8), RR, DET
    (lmin 2) and LAM (vmin 2) -- raw integers bit for bit, measures within
    the float32 tolerance."""
    from accrqa_gb300 import engine
    x = workloads.logistic(10_000, 2024).astype(np.float32)
    thr = np.linspace(0.05, 0.40, 8).astype(np.float32)
    np.testing.assert_array_equal(engine.rr_counts(x, 1, 3, thr, 2),
                                  oracle_mod.rr_counts(x, 1, 3, thr, 2))
    det = engine.det_histograms(x, 1, 3, thr, 2)
    lam = engine.lam_histograms(x, 1, 3, thr, 2)
    for k, t in enumerate(thr):
        np.testing.assert_array_equal(det[k], oracle_mod.det_hist(x, 1, 3, t, 2))
        np.testing.assert_array_equal(lam[k], oracle_mod.lam_hist(x, 1, 3, t, 2))
    one = np.array([1], np.intc)
    three = np.array([3], np.intc)
    lm = np.array([2], np.intc)
    D = A.accrqaDistance("maximal")
    _close(A.DET(x, one, three, lm, thr, D, tidy_data=False),
           oracle_mod.line_output(x, [1], [3], lm, thr, 2, 1, True), np.float32)
    _close(A.LAM(x, one, three, lm, thr, D, tidy_data=False),
           oracle_mod.line_output(x, [1], [3], lm, thr, 2, 1, False), np.float32)
