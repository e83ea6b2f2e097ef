"""Serving with continuous batching: each result is the same alone and in the mix.

Requests of mixed size, dtype and measure are submitted from several client
threads while earlier ones are on the GPU; every result must equal the plain
per-series API result bit for bit (float32 and float64 alike), and the
server must have served them in more than one batch.
"""
import threading

import numpy as np
import pytest

import accrqa_gb300 as A
from accrqa_gb300 import engine, workloads

pytestmark = pytest.mark.gpu


def _requests(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(200), np.log(6000))))
        dt = np.float64 if rng.uniform() < 0.2 else np.float32
        x = workloads.ar1(n, int(rng.integers(1 << 30))).astype(dt)
        x = (x / np.std(x.astype(np.float64))).astype(dt)
        nthr = int(rng.integers(1, 17))
        out.append(dict(x=x, tau=int(rng.integers(1, 5)), emb=int(rng.integers(2, 9)),
                        norm=int(rng.integers(1, 3)),
                        thresholds=np.sort(rng.uniform(0.05, 1.0, nthr)).astype(dt),
                        measures=(str(rng.choice(["rr", "det", "lam"])),)))
    return out


def _alone(j):
    D = A.accrqaDistance("euclidean" if j["norm"] == 1 else "maximal")
    t = np.array([j["tau"]], np.intc)
    e = np.array([j["emb"]], np.intc)
    m = j["measures"][0]
    if m == "rr":
        return A.RR(j["x"], t, e, j["thresholds"], D, tidy_data=False).reshape(-1)
    f = A.DET if m == "det" else A.LAM
    return f(j["x"], t, e, np.array([2], np.intc), j["thresholds"], D,
             tidy_data=False).reshape(-1, 5)


def test_results_same_alone_and_in_the_mix(gpu):
    reqs = _requests(11, 60)
    results = [None] * len(reqs)
    with engine.Server(workers=2) as srv:
        def client(idx):
            for i in idx:
                t = srv.submit(reqs[i])
                results[i] = srv.wait(t)

        threads = [threading.Thread(target=client, args=(range(k, len(reqs), 4),))
                   for k in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        batches, served = srv.stats()
    assert served == len(reqs)
    assert batches >= 2
    for j, (o, lat) in zip(reqs, results):
        assert lat >= 0
        np.testing.assert_array_equal(o[j["measures"][0]], _alone(j))


def test_server_rejects_invalid_job(gpu):
    with engine.Server(workers=1) as srv:
        bad = dict(x=np.zeros(10, np.float32), tau=5, emb=5, norm=1,
                   thresholds=np.array([0.1], np.float32))
        with pytest.raises(engine.EngineError):
            srv.submit(bad)


def test_burst_is_batched_on_resident_series(gpu):
    """Many small requests submitted at once: the workers take them in
    batches (fewer batches than requests) on the series admitted to the
    device, and every result equals the plain call's."""
    reqs = _requests(23, 48)
    for r in reqs:   # small series, so that several fit one work quantum
        r["x"] = r["x"][:min(len(r["x"]), 1500)]
    with engine.Server(workers=2) as srv:
        tickets = [srv.submit(r) for r in reqs]
        results = [srv.wait(t) for t in tickets]
        batches, served = srv.stats()
    assert served == len(reqs)
    assert batches < served
    for j, (o, _) in zip(reqs, results):
        np.testing.assert_array_equal(o[j["measures"][0]], _alone(j))
