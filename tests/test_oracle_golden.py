"""The oracle against the reference's golden vectors (CPU only).

  * raw RR counts and DET/LAM histograms produced by the reference's own CPU
    code (tests/golden/ref_histograms.npz) -- bit for bit;
  * the reference's public CPU API outputs on the CRQA grid
    (tests/golden/ref_outputs.json) -- the oracle's measures;
  * the CRQA known answers of the reference's C++ test (tol 1e-4) and the
    expected tables of its R tests (CRQA tol 1e-6, PyRQA tol 1e-3);
  * the analytic constant-series answers of the reference's R tests.
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return json.load(open(os.path.join(GOLD, name)))


@pytest.fixture(scope="module")
def crqa_x():
    return np.load(os.path.join(GOLD, "crqa_input.npy"))


def test_oracle_matches_reference_raw_integers(oracle_mod):
    meta = _load("ref_histograms.json")
    arr = np.load(os.path.join(GOLD, "ref_histograms.npz"))
    assert len(meta["cases"]) == 16
    for c in meta["cases"]:
        k = c["key"]
        x, thr = arr[k + "_x"], arr[k + "_thr"]
        tau, emb, dist = c["tau"], c["emb"], c["dist"]
        np.testing.assert_array_equal(oracle_mod.rr_counts(x, tau, emb, thr, dist),
                                      arr[k + "_rr"], err_msg=k)
        for j, t in enumerate(thr):
            np.testing.assert_array_equal(oracle_mod.det_hist(x, tau, emb, t, dist),
                                          arr[k + "_det"][j], err_msg=f"{k} DET {t}")
            np.testing.assert_array_equal(oracle_mod.lam_hist(x, tau, emb, t, dist),
                                          arr[k + "_lam"][j], err_msg=f"{k} LAM {t}")


def test_oracle_measures_match_reference_api(oracle_mod, crqa_x):
    g = _load("ref_outputs.json")
    taus, embs, lmins, thr = g["taus"], g["embs"], g["lmins"], g["thr"]
    for dist in (1, 2):
        rr = np.array(g["out"][f"RR_{dist}"]).reshape(len(taus), len(embs), len(thr))
        for a, tau in enumerate(taus):
            for b, emb in enumerate(embs):
                nc = len(crqa_x) - (emb - 1) * tau
                cnt = oracle_mod.rr_counts(crqa_x, tau, emb, thr, dist)
                np.testing.assert_allclose(cnt / float(nc * nc), rr[a, b], rtol=1e-15)
        for kind in ("DET", "LAM"):
            # the reference's CPU path computes every measure for both calc_ENTR values;
            # CPU DET packs [tau][emb][thr][lmin], CPU LAM packs [tau][emb][lmin][thr]
            for entr in (1, 0):
                out = np.array(g["out"][f"{kind}_{dist}_{entr}"])
                if kind == "DET":
                    out = out.reshape(len(taus), len(embs), len(thr), len(lmins), 5)
                    out = out.transpose(0, 1, 3, 2, 4)
                else:
                    out = out.reshape(len(taus), len(embs), len(lmins), len(thr), 5)
                for a, tau in enumerate(taus):
                    for b, emb in enumerate(embs):
                        for k, t in enumerate(thr):
                            h = (oracle_mod.det_hist if kind == "DET" else oracle_mod.lam_hist)(
                                crqa_x, tau, emb, t, dist)
                            for c, lm in enumerate(lmins):
                                m = oracle_mod.measures(h, lm, kind == "DET")
                                np.testing.assert_allclose(m, out[a, b, c, k], rtol=1e-13,
                                                           err_msg=f"{kind} {dist} {tau} {emb}")


def test_crqa_known_answers(oracle_mod, crqa_x):
    kat = _load("crqa_kat.json")["cases"]
    for dist in ("1", "2"):
        for row in kat["DET"][dist]:
            tau, emb, lm = int(row["tau"]), int(row["emb"]), int(row["lmin"])
            h = oracle_mod.det_hist(crqa_x, tau, emb, row["thr"], int(dist))
            m = oracle_mod.measures(h, lm, True)
            for i, key in ((0, "CRQA_DET"), (1, "CRQA_L"), (3, "CRQA_ENTR"), (4, "CRQA_RR")):
                assert abs(m[i] - row[key]) <= 1e-4, (dist, row, key, m[i])
        for row in kat["LAM"][dist]:
            tau, emb, vm = int(row["tau"]), int(row["emb"]), int(row["vmin"])
            h = oracle_mod.lam_hist(crqa_x, tau, emb, row["thr"], int(dist))
            m = oracle_mod.measures(h, vm, False)
            for i, key in ((0, "CRQA_LAM"), (1, "CRQA_TT"), (4, "CRQA_RR")):
                assert abs(m[i] - row[key]) <= 1e-4, (dist, row, key, m[i])
        for row in kat["RR"][dist]:
            tau, emb = int(row["tau"]), int(row["emb"])
            nc = len(crqa_x) - (emb - 1) * tau
            c = oracle_mod.rr_counts(crqa_x, tau, emb, [row["thr"]], int(dist))[0]
            assert abs(c / nc / nc - row["CRQA_RR"]) <= 1e-4


def _mean_rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.mean(np.abs(a - b)) / np.mean(np.abs(b)))


@pytest.mark.parametrize("table,tol", [
    ("expected_CRQA_DET_euclidean", 1e-6), ("expected_CRQA_DET_maximal", 1e-6),
    ("expected_CRQA_LAM_euclidean", 1e-6), ("expected_CRQA_LAM_maximal", 1e-6),
    ("expected_CRQA_RR_euclidean", 1e-6), ("expected_CRQA_RR_maximal", 1e-6),
    ("expected_PyRQA_DET_euclidean", 1e-3), ("expected_PyRQA_LAM_euclidean", 1e-3),
    ("expected_PyRQA_RR_euclidean", 1e-3)])
def test_r_fixture_tables(oracle_mod, crqa_x, table, tol):
    """R's expect_equal(tolerance) compares mean relative differences per column."""
    t = _load("r_fixtures.json")["tables"][table]
    dist = 2 if "maximal" in table else 1
    rows = len(t["Delay"])
    got = {k: [] for k in t}
    for r in range(rows):
        tau, emb, thr = int(t["Delay"][r]), int(t["Embedding"][r]), t["Threshold"][r]
        nc = len(crqa_x) - (emb - 1) * tau
        if "_RR_" in table:
            got["RR"].append(oracle_mod.rr_counts(crqa_x, tau, emb, [thr], dist)[0] / nc / nc)
            continue
        det = "_DET_" in table
        lm = int(t["Lmin" if det else "Vmin"][r])
        h = (oracle_mod.det_hist if det else oracle_mod.lam_hist)(crqa_x, tau, emb, thr, dist)
        m = oracle_mod.measures(h, lm, det)
        names = ("DET", "L", "Lmax", "ENTR", "RR") if det else ("LAM", "TT", "TTmax", "ENTR", "RR")
        for i, nm in enumerate(names):
            if nm in got:
                got[nm].append(m[i])
    # test-accRQA_PyRQA.R:27-28 drops L from the PyRQA DET comparison
    skip = {"L"} if table == "expected_PyRQA_DET_euclidean" else set()
    for col in got:
        if got[col] and col not in skip:
            assert _mean_rel(got[col], t[col]) <= tol, (table, col)


@pytest.mark.parametrize("tau", [1, 2])
def test_constant_series_answers(oracle_mod, tau):
    """tests/testthat/test-accRQA_DET.R:84-108 and test-accRQA_LAM.R:89-111."""
    x = np.ones(10)
    for thr in (0.1, 0.2):
        h = oracle_mod.det_hist(x, tau, 1, thr, 2)
        for lm in (2, 3, 4):
            m = oracle_mod.measures(h, lm, True)
            assert m[0] == 1.0 - 2 * sum(range(1, lm)) / 100.0
            assert m[2] == 9.0 and m[4] == 1.0
        hl = oracle_mod.lam_hist(x, tau, 1, thr, 2)
        for vm in (2, 3, 4):
            m = oracle_mod.measures(hl, vm, False)
            assert m[0] == 1.0 and m[4] == 1.0
        assert oracle_mod.rr_counts(x, tau, 1, [thr], 2)[0] == 100


def test_fullsize_series_regenerate():
    """The full-size GPU parity fixtures (tests/golden/fullsize.*) were
    recorded on seeded series: regenerated here they hash the same, so the GPU
    tests compare the engine with the reference on the very same input."""
    import json
    import sys
    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, gold)
    import make_fullsize
    with open(os.path.join(gold, "fullsize.json")) as f:
        table = {c["name"]: c for c in json.load(f)["cases"]}
    for name, build, combos, thr_of, _ in make_fullsize.cases():
        x = build()
        assert make_fullsize.series_sha(x) == table[name]["sha256"], name
        thr = thr_of(x)
        assert [t.tobytes().hex() for t in thr] == table[name]["thresholds_hex"], name
