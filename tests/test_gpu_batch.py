"""Batched submission: many uneven series in one call, identical to plain calls.

Every batch output (RR, DET, LAM for each series, both output conventions,
float32 and float64, emb specialised and generic, more than 16 thresholds)
must equal what the per-series public API returns, bit for bit, and the raw
counts behind them must equal the oracle's.
"""
import numpy as np
import pytest

import accrqa_gb300 as A
from accrqa_gb300 import engine, workloads

pytestmark = pytest.mark.gpu


def _jobs(seed, count):
    rng = np.random.default_rng(seed)
    gens = [workloads.logistic, workloads.lorenz_x, workloads.ar1, workloads.white]
    jobs = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(60), np.log(3000))))
        dt = np.float64 if i % 5 == 4 else np.float32
        x = gens[i % 4](n, int(rng.integers(1 << 30))).astype(dt)
        x = (x / np.std(x.astype(np.float64))).astype(dt)
        tau = int(rng.integers(1, 5))
        emb = int(rng.integers(1, 10))
        if n - (emb - 1) * tau < 2:
            emb = 1
        nthr = int(rng.choice([1, 3, 8, 11, 20]))
        thr = np.sort(rng.uniform(0.05, 1.2, nthr)).astype(dt)
        jobs.append(dict(x=x, tau=tau, emb=emb, norm=int(rng.integers(1, 3)), thresholds=thr,
                         lmin=int(rng.choice([1, 2, 3, 17])), vmin=int(rng.choice([2, 4])),
                         calc_entr=int(rng.integers(0, 2))))
    return jobs


@pytest.mark.parametrize("seed", [1, 2])
def test_batch_equals_plain_calls(gpu, seed):
    jobs = _jobs(seed, 40)
    outs = engine.batch(jobs)
    for j, o in zip(jobs, outs):
        x, thr = j["x"], j["thresholds"]
        D = A.accrqaDistance("euclidean" if j["norm"] == 1 else "maximal")
        t = np.array([j["tau"]], np.intc)
        e = np.array([j["emb"]], np.intc)
        rr = A.RR(x, t, e, thr, D, tidy_data=False).reshape(-1)
        np.testing.assert_array_equal(o["rr"], rr)
        det = A.DET(x, t, e, np.array([j["lmin"]], np.intc), thr, D,
                    calculate_ENTR=bool(j["calc_entr"]), tidy_data=False).reshape(-1, 5)
        np.testing.assert_array_equal(o["det"], det)
        lam = A.LAM(x, t, e, np.array([j["vmin"]], np.intc), thr, D,
                    calculate_ENTR=bool(j["calc_entr"]), tidy_data=False).reshape(-1, 5)
        np.testing.assert_array_equal(o["lam"], lam)


def test_batch_counts_match_oracle(gpu, oracle_mod):
    jobs = _jobs(7, 12)
    outs = engine.batch(jobs, measures=("rr",))
    for j, o in zip(jobs, outs):
        nc = len(j["x"]) - (j["emb"] - 1) * j["tau"]
        cnt = oracle_mod.rr_counts(j["x"], j["tau"], j["emb"], j["thresholds"], j["norm"])
        np.testing.assert_array_equal(o["rr"], oracle_mod.rr_output(cnt, nc, j["x"].dtype))
        assert "det" not in o


RTOL = {np.float32: 1e-6, np.float64: 1e-12}


@pytest.mark.parametrize("measures", [("det", "lam"), ("rr", "det", "lam"), ("lam",)])
def test_batch_lines_match_oracle(gpu, oracle_mod, measures):
    """Batched DET and LAM outputs against the oracle's histograms (their
    measures in the reference's GPU layout and conventions): ratios within
    1e-6 (float32) / 1e-12 (float64), line lengths exact."""
    jobs = _jobs(11, 14)
    outs = engine.batch(jobs, measures=measures)
    for j, o in zip(jobs, outs):
        x, dt = j["x"], j["x"].dtype.type
        for kind in ("det", "lam"):
            if kind not in measures:
                assert kind not in o
                continue
            lm = j["lmin"] if kind == "det" else j["vmin"]
            want = oracle_mod.line_output(x, [j["tau"]], [j["emb"]], [lm], j["thresholds"],
                                          j["norm"], j["calc_entr"], kind == "det").reshape(-1, 5)
            got = np.asarray(o[kind], np.float64)
            w = np.asarray(want, np.float64)
            assert np.array_equal(np.isnan(got), np.isnan(w)), kind
            m = ~np.isnan(w)
            np.testing.assert_allclose(got[m], w[m], rtol=RTOL[dt], atol=0)
            np.testing.assert_array_equal(got[:, 2], w[:, 2])   # longest line
        if "rr" in measures:
            nc = len(x) - (j["emb"] - 1) * j["tau"]
            cnt = oracle_mod.rr_counts(x, j["tau"], j["emb"], j["thresholds"], j["norm"])
            np.testing.assert_array_equal(o["rr"], oracle_mod.rr_output(cnt, nc, x.dtype))


def test_batch_rejects_bad_job(gpu):
    jobs = _jobs(3, 2)
    jobs[1]["tau"] = 0
    with pytest.raises(engine.EngineError):
        engine.batch(jobs)


def test_batch_large_series_from_tile_levels(gpu):
    """Series long enough for the level passes (their DET and LAM walked from
    one store of tile levels, their RR taken from the LAM histograms) mixed
    with short ones: every output equals the plain calls', bit for bit."""
    rng = np.random.default_rng(31)
    jobs = []
    for i, n in enumerate([17000, 23000, 1200, 30000, 2500, 19000]):
        dt = np.float64 if i % 3 == 2 or i == 5 else np.float32
        x = workloads.lorenz_x(n, 100 + i, transient=500).astype(dt)
        x = (x / np.std(x.astype(np.float64))).astype(dt)
        nthr = [3, 8, 11, 20, 5, 16][i]
        jobs.append(dict(x=x, tau=int(rng.integers(1, 4)), emb=int(rng.integers(2, 7)),
                         norm=1 + i % 2,
                         thresholds=np.sort(rng.uniform(0.05, 1.0, nthr)).astype(dt),
                         lmin=2, vmin=2, calc_entr=1 - (i == 3)))
    for measures in (("rr", "det", "lam"), ("rr", "lam"), ("det", "lam")):
        outs = engine.batch(jobs, measures=measures)
        for j, o in zip(jobs, outs):
            D = A.accrqaDistance("euclidean" if j["norm"] == 1 else "maximal")
            t = np.array([j["tau"]], np.intc)
            e = np.array([j["emb"]], np.intc)
            if "rr" in measures:
                np.testing.assert_array_equal(
                    o["rr"], A.RR(j["x"], t, e, j["thresholds"], D, tidy_data=False).reshape(-1))
            if "det" in measures:
                np.testing.assert_array_equal(
                    o["det"], A.DET(j["x"], t, e, np.array([2], np.intc), j["thresholds"], D,
                                    calculate_ENTR=bool(j["calc_entr"]),
                                    tidy_data=False).reshape(-1, 5))
            np.testing.assert_array_equal(
                o["lam"], A.LAM(j["x"], t, e, np.array([2], np.intc), j["thresholds"], D,
                                calculate_ENTR=bool(j["calc_entr"]),
                                tidy_data=False).reshape(-1, 5))
