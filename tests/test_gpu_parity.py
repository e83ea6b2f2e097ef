"""GPU parity: the engine's raw integers against the oracle, bit for bit.

RR counts and DET/LAM line-length histograms from libaccrqa.so (through its
C ABI) must equal the oracle restatement's exactly, for both dtypes, both
norms, a spread of (tau, emb), thresholds that hit exact ties, and the edge
cases the reference tests: constant input, tiny series, NaN/inf samples,
negative and zero thresholds, more than 16 thresholds (several passes).
"""
import numpy as np
import pytest

from accrqa_gb300 import workloads

pytestmark = pytest.mark.gpu

NORMS = [1, 2]


def _cases():
    rng = np.random.default_rng(11)
    cases = []
    for dt in (np.float32, np.float64):
        for norm in NORMS:
            # tau 8 at emb 3 and 6..8: the carried-term DET with term windows
            # of 16 to 56 positions (the widest at 3 CTAs per SM)
            for (n, tau, emb) in [(97, 1, 1), (300, 1, 3), (451, 2, 5), (530, 3, 4),
                                  (700, 1, 8), (256, 4, 2), (333, 7, 9), (129, 1, 2),
                                  (600, 8, 3), (900, 8, 6), (1100, 8, 7), (1200, 8, 8)]:
                cases.append((dt, norm, n, tau, emb, int(rng.integers(0, 1 << 30))))
    return cases


@pytest.mark.parametrize("dt,norm,n,tau,emb,seed", _cases())
def test_counts_and_histograms_match_oracle(gpu, oracle_mod, dt, norm, n, tau, emb, seed):
    x = workloads.logistic(n, seed).astype(dt)
    if seed % 3 == 0:
        x = (np.round(x * 16) / 16).astype(dt)      # many exact ties at the thresholds
    thr = np.array([0.0, 0.0625, 0.1, 0.125, 0.2, 0.25, 0.3, 0.5, 0.75, 1.0],
                   dtype=dt)
    rr = gpu.rr_counts(x, tau, emb, thr, norm)
    np.testing.assert_array_equal(rr, oracle_mod.rr_counts(x, tau, emb, thr, norm))
    det = gpu.det_histograms(x, tau, emb, thr, norm)
    lam = gpu.lam_histograms(x, tau, emb, thr, norm)
    for k, t in enumerate(thr):
        np.testing.assert_array_equal(det[k], oracle_mod.det_hist(x, tau, emb, t, norm))
        np.testing.assert_array_equal(lam[k], oracle_mod.lam_hist(x, tau, emb, t, norm))


def _diag_cases():
    # float series with a fixed embedding whose RR takes the diagonal walk
    # (emb >= 4 and (emb - 1) tau >= 7, or at most 4 thresholds): residue
    # blocks for tau dividing 32 or not, tau above 32, lengths around the
    # band and chunk edges
    rng = np.random.default_rng(23)
    out = []
    for norm in NORMS:
        for (n, tau, emb) in [(50, 1, 4), (66, 1, 4), (200, 2, 4), (1000, 3, 4), (777, 5, 6),
                              (900, 7, 4), (2100, 33, 4), (3000, 40, 5), (400, 16, 8),
                              (1300, 32, 4), (129, 2, 8), (4000, 1, 8), (2500, 8, 5)]:
            out.append((norm, n, tau, emb, int(rng.integers(0, 1 << 30))))
    return out


@pytest.mark.parametrize("norm,n,tau,emb,seed", _diag_cases())
def test_rr_diagonal_walk_matches_oracle(gpu, oracle_mod, norm, n, tau, emb, seed):
    x = workloads.logistic(n, seed).astype(np.float32)
    if seed % 2 == 0:
        x = (np.round(x * 16) / 16).astype(np.float32)   # exact ties at the thresholds
    if seed % 5 == 0:
        x[n // 3] = np.nan                                # NaN and inf cells, main diagonal too
        x[n // 2] = np.inf
    few = np.array([0.05, 0.125, 0.25, 0.5], np.float32)
    many = np.linspace(0.0, 1.0, 12).astype(np.float32)
    for thr in (few, many):
        np.testing.assert_array_equal(gpu.rr_counts(x, tau, emb, thr, norm),
                                      oracle_mod.rr_counts(x, tau, emb, thr, norm))


@pytest.mark.parametrize("nthr", [1, 3, 4, 5, 8, 9, 16, 17, 40])
def test_threshold_pass_splitting(gpu, oracle_mod, nthr):
    x = workloads.white(400, 5 + nthr).astype(np.float32)
    thr = np.linspace(0.05, 3.0, nthr).astype(np.float32)
    np.testing.assert_array_equal(gpu.rr_counts(x, 2, 3, thr, 1),
                                  oracle_mod.rr_counts(x, 2, 3, thr, 1))
    det = gpu.det_histograms(x, 2, 3, thr, 1)
    for k, t in enumerate(thr):
        np.testing.assert_array_equal(det[k], oracle_mod.det_hist(x, 2, 3, t, 1))


def _nan_variety(dt):
    if dt == np.float32:
        bits = np.array([0xFFC00000, 0x7FC00001, 0xFF800001, 0x7F800001], np.uint32)
    else:
        bits = np.array([0xFFF8000000000000, 0x7FF8000000000001, 0xFFF0000000000001,
                         0x7FF0000000000001], np.uint64)
    big = np.finfo(dt).max
    nans = bits.view(dt)
    base = np.array([0.1, 0.2, 0.15, big, -big, 0.12, 0.11, 0.3, 1e30, -1e30, 0.1, 0.2], dt)
    # concatenation keeps every NaN's bits as they are
    return np.concatenate([np.concatenate([base, nans[k % 4:k % 4 + 1]]) for k in range(8)])


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_edge_series(gpu, oracle_mod, dt):
    specials = {
        "constant": np.ones(50),
        "single": np.array([0.3]),
        "two": np.array([0.1, 0.2]),
        "nan_inf": np.array([0.1, np.nan, 0.3, np.inf, 0.2, -np.inf, 0.25, 0.26, 0.27,
                             0.1, 0.3, 0.5] * 4),
        "long_lines": np.tile(np.arange(10) / 10.0, 70),   # periodic: lines of length ~nc
        # NaNs of both signs and with payloads, and values whose squared
        # differences overflow to inf
        "nan_signs": _nan_variety(dt),
    }
    thr = np.array([-1.0, -0.0, 0.0, 0.05, 0.1, 0.5, np.inf, np.nan], dtype=dt)
    for name, s in specials.items():
        x = s.astype(dt)
        for norm in NORMS:
            emb = 1 if len(x) < 4 else 2
            rr = gpu.rr_counts(x, 1, emb, thr, norm)
            np.testing.assert_array_equal(rr, oracle_mod.rr_counts(x, 1, emb, thr, norm),
                                          err_msg=name)
            det = gpu.det_histograms(x, 1, emb, thr, norm)
            lam = gpu.lam_histograms(x, 1, emb, thr, norm)
            for k, t in enumerate(thr):
                np.testing.assert_array_equal(
                    det[k], oracle_mod.det_hist(x, 1, emb, t, norm), err_msg=f"{name} DET {t}")
                np.testing.assert_array_equal(
                    lam[k], oracle_mod.lam_hist(x, 1, emb, t, norm), err_msg=f"{name} LAM {t}")


def test_edge_series_by_levels(gpu, oracle_mod):
    """The same special series through the float passes of more than 8
    thresholds, which take their levels from the bucket table: NaN and inf
    distances must come out at level 0 in the RR counts, the tile planes
    (level 16 included) and the DET/LAM walks."""
    specials = {
        "nan_inf": np.array([0.1, np.nan, 0.3, np.inf, 0.2, -np.inf, 0.25, 0.26, 0.27,
                             0.1, 0.3, 0.5] * 4),
        "nan_signs": _nan_variety(np.float32),
        "long_lines": np.tile(np.arange(10) / 10.0, 70),
    }
    thr = np.array([0.01, 0.02, 0.05, 0.08, 0.1, 0.15, 0.2, 0.3, 0.5, 0.7, 1.0, 2.0],
                   dtype=np.float32)
    for name, s in specials.items():
        x = s.astype(np.float32)
        for norm in NORMS:
            for emb in (1, 2, 3):
                rr = gpu.rr_counts(x, 1, emb, thr, norm)
                np.testing.assert_array_equal(rr, oracle_mod.rr_counts(x, 1, emb, thr, norm),
                                              err_msg=name)
                det = gpu.det_histograms(x, 1, emb, thr, norm)
                lam = gpu.lam_histograms(x, 1, emb, thr, norm)
                for k, t in enumerate(thr):
                    np.testing.assert_array_equal(
                        det[k], oracle_mod.det_hist(x, 1, emb, t, norm),
                        err_msg=f"{name} emb {emb} DET {t}")
                    np.testing.assert_array_equal(
                        lam[k], oracle_mod.lam_hist(x, 1, emb, t, norm),
                        err_msg=f"{name} emb {emb} LAM {t}")


@pytest.mark.parametrize("norm", NORMS)
def test_rr_level_table_thresholds(gpu, oracle_mod, norm):
    """Float RR passes of more than 8 thresholds count cells by level from a
    bucket table built from the thresholds' limits: negative, zero, tiny,
    infinite and NaN thresholds, repeated ones, limits a few ulps apart
    (fine buckets, or no table), limits spread over sixty decades, and a
    series with NaN, inf and exactly tied distances -- on the row walk
    (emb 2) and the diagonal walk (emb 4, tau 3)."""
    x = workloads.logistic(900, 4).astype(np.float32)
    x[:300] = np.round(x[:300] * 16) / 16
    x[450], x[451], x[700] = np.nan, np.inf, -np.inf
    sets = [
        np.array([-1.0, -0.0, 0.0, 1e-30, 0.05, 0.05, 0.0625, 0.1, np.nextafter(0.1, 1.0),
                  0.2, 0.25, 0.5, np.inf, np.nan], np.float32),
        np.linspace(0.1, 0.1 + 15 * 2 ** -26, 16).astype(np.float32),
        np.geomspace(1e-30, 1e30, 16).astype(np.float32),
        np.full(16, 0.125, np.float32),
        np.linspace(0.0, 0.9, 9).astype(np.float32),
    ]
    for thr in sets:
        for tau, emb in [(1, 2), (3, 4)]:
            np.testing.assert_array_equal(gpu.rr_counts(x, tau, emb, thr, norm),
                                          oracle_mod.rr_counts(x, tau, emb, thr, norm),
                                          err_msg=f"{thr} tau {tau} emb {emb}")


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_rp_matches_oracle(gpu, oracle_mod, dt):
    x = workloads.lorenz_x(600, 3, transient=500).astype(dt)
    for norm in NORMS:
        for (tau, emb, t) in [(1, 3, 0.3), (2, 4, 0.8), (5, 1, 0.0)]:
            got = gpu.rp(x, tau, emb, t, norm)
            np.testing.assert_array_equal(got, oracle_mod.rp(x, tau, emb, t, norm))
    x64 = x.astype(np.float64)
    np.testing.assert_array_equal(gpu.rp(x64, 2, 3, 0.5, 1, out_dtype=np.int32),
                                  oracle_mod.rp_i32(x64, 2, 3, 0.5, 1))


@pytest.mark.parametrize("scale,offset,grid", [(1.0, 0.0, False), (1.0, 0.0, True),
                                               (1e6, 0.0, True), (1e-12, 0.0, False),
                                               (1.0, 1e9, False), (1e100, 0.0, False)])
def test_f64_filter_matches_oracle(gpu, oracle_mod, scale, offset, grid):
    """float64 passes decide cells in float against proven limits and only
    the cells near a threshold in double.  Scales and offsets move the
    bound's relative and absolute parts (offset 1e9 makes most cells
    ambiguous), the grid puts many distances exactly on thresholds, and
    |x| = 1e100 turns the filter off."""
    x0 = workloads.lorenz_x(600, 9, transient=500)
    x0 = x0 / np.std(x0)
    if grid:
        x0 = np.round(x0 * 16) / 16
    x = x0 * scale + offset
    thr = np.array([0.0, 0.0625, 0.125, 0.3, 0.5, 0.75, 1.5]) * scale
    for norm in NORMS:
        for tau, emb in [(1, 3), (2, 5), (1, 1), (3, 4), (33, 4), (1, 8)]:
            np.testing.assert_array_equal(gpu.rr_counts(x, tau, emb, thr, norm),
                                          oracle_mod.rr_counts(x, tau, emb, thr, norm))
            det = gpu.det_histograms(x, tau, emb, thr, norm)
            lam = gpu.lam_histograms(x, tau, emb, thr, norm)
            for k, t in enumerate(thr):
                np.testing.assert_array_equal(det[k], oracle_mod.det_hist(x, tau, emb, t, norm))
                np.testing.assert_array_equal(lam[k], oracle_mod.lam_hist(x, tau, emb, t, norm))
