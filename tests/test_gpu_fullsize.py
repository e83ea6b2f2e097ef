"""GPU parity at the benchmarked sizes, against the reference's own CPU code.

The fixtures in tests/golden/fullsize.{json,npz} hold raw RR counts and full
DET/LAM line-length histograms that the AccRQA reference's CPU implementation
computed on the same seeded series (tests/golden/make_fullsize.py, run from
oracle/_ref; src/AccRQA_CPU_function.cpp:40-46,446-490,587-642):

  * the benchmark's Lorenz series, N = 200,000 float32, Euclidean, (tau, emb)
    = (1, 3) and (8, 8), 4 of its 16 thresholds: RR, DET and LAM;
  * the N = 1e6 roofline workload's shapes at N = 200,000: white noise and
    AR(1) phi = 0.95, tau 1, emb 5, thresholds {0.1, 0.2, 0.5, 1.0} std, in
    float32 and in float64 (float64 through the host entry points, which
    decide cells with the certified float filter): RR and DET.

The engine's integers must equal them bit for bit.  The series are
regenerated here and checked against the recorded SHA-256 first.

An opt-in check at N = 1e6 float64 (ACCRQA_SLOW=1) compares RR and DET with
one threshold against the oracle computed on the host (several minutes).
"""
import json
import os
import sys

import numpy as np
import pytest

from accrqa_gb300 import workloads

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLD)
import make_fullsize  # noqa: E402  (series builders; reads nothing of the reference)

with open(os.path.join(GOLD, "fullsize.json")) as _f:
    TABLE = json.load(_f)
CASES = {c["name"]: c for c in TABLE["cases"]}
BUILDERS = {name: (build, thr_of) for name, build, _, thr_of, _ in make_fullsize.cases()}


@pytest.fixture(scope="module")
def hists():
    return np.load(os.path.join(GOLD, "fullsize.npz"))


def _series(name):
    case = CASES[name]
    x = BUILDERS[name][0]()
    assert make_fullsize.series_sha(x) == case["sha256"], \
        f"{name}: the regenerated series differs from the recorded one"
    thr = np.array([np.frombuffer(bytes.fromhex(h), dtype=x.dtype)[0]
                    for h in case["thresholds_hex"]], dtype=x.dtype)
    np.testing.assert_array_equal(thr, BUILDERS[name][1](x))
    return x, thr


def _dense(hists, key, nc):
    h = np.zeros(nc + 1, dtype=np.uint64)
    h[hists[key + "/len"]] = hists[key + "/cnt"]
    return h


PARAMS = [(c["name"], cb["tau"], cb["emb"]) for c in TABLE["cases"] for cb in c["combos"]]


@pytest.mark.parametrize("name,tau,emb", PARAMS)
def test_fullsize_integers_match_reference(gpu, hists, name, tau, emb):
    x, thr = _series(name)
    combo = next(cb for cb in CASES[name]["combos"] if (cb["tau"], cb["emb"]) == (tau, emb))
    nc = combo["nc"]
    rr = gpu.rr_counts(x, tau, emb, thr, 1)
    np.testing.assert_array_equal(rr, np.array(combo["rr"], dtype=np.uint64))
    kinds = ["det"] + (["lam"] if f"{name}/t{tau}e{emb}/lam/0/len" in hists.files else [])
    for kind in kinds:
        got = (gpu.det_histograms if kind == "det" else gpu.lam_histograms)(x, tau, emb, thr, 1)
        for k in range(len(thr)):
            want = _dense(hists, f"{name}/t{tau}e{emb}/{kind}/{k}", nc)
            bad = np.nonzero(got[k] != want)[0]
            assert bad.size == 0, (kind, k, bad[:5], got[k][bad[:5]], want[bad[:5]])
        if kind == "lam":
            # every recurrent cell lies on exactly one vertical line
            lens = np.arange(nc + 1, dtype=np.uint64)
            np.testing.assert_array_equal((got * lens).sum(axis=1), rr)


@pytest.mark.skipif(os.environ.get("ACCRQA_SLOW") != "1", reason="opt-in: ACCRQA_SLOW=1")
def test_1m_float64_against_oracle(gpu, oracle_mod):
    """N = 1e6 float64 AR(1), tau 1, emb 5, threshold 0.2 std: RR count and
    DET histogram through the float filter against the oracle on the host."""
    base = workloads.ar1(1_000_000, 2024 + 7)
    x = ((base - base.mean()) / base.std()).astype(np.float64)
    thr = np.array([0.2 * float(np.std(x))])
    rr = gpu.rr_counts(x, 1, 5, thr, 1)
    np.testing.assert_array_equal(rr, oracle_mod.rr_counts(x, 1, 5, thr, 1))
    det = gpu.det_histograms(x, 1, 5, thr, 1)
    np.testing.assert_array_equal(det[0], oracle_mod.det_hist(x, 1, 5, thr[0], 1))
