"""Record full-size golden results from the AccRQA reference's own CPU code.

TEST INFRASTRUCTURE ONLY.  The GPU parity tests at the benchmarked sizes
(tests/test_gpu_fullsize.py) compare the engine's raw integers -- RR counts
and DET/LAM line-length histograms -- bit for bit with the numbers this
script records.  They come from the reference's CPU implementation itself
(oracle/_ref/libaccrqa_ref.so, built from the reference sources by
`make -C oracle ref REF=<tree>`), not from the restatement:

  R_matrix_element (RR counts)        src/AccRQA_CPU_function.cpp:40-46
  rqa_CPU_DET_metric_parallel_mk1     src/AccRQA_CPU_function.cpp:587-642
  rqa_CPU_LAM_metric_parallel         src/AccRQA_CPU_function.cpp:446-490

Cases (seeded generators of accrqa_gb300/workloads.py, regenerated by the
tests and checked against the SHA-256 of the series recorded here):
  lorenz200k  Lorenz x, N = 200,000 float32 z-scored (the benchmark series),
              Euclidean, (tau, emb) = (1, 3) and (8, 8), 4 of the
              benchmark's 16 thresholds (0.05, 0.30, 0.55, 0.80 std);
              RR, DET and LAM.
  white200k / ar1200k  white noise and AR(1) phi = 0.95, N = 200,000
              z-scored, float32 and float64, tau = 1, emb = 5, Euclidean,
              thresholds {0.1, 0.2, 0.5, 1.0} x std (the N = 1e6 roofline
              workload's shapes at N = 200,000); RR and DET.

    ACCRQA_REFERENCE_TREE=<tree> make -C oracle ref REF=<tree>
    python tests/golden/make_fullsize.py        # ~20 min on 8 cores

Output: tests/golden/fullsize.npz (sparse histograms) and fullsize.json
(case table, series hashes, RR counts).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

BENCH_SEED = 2024
BENCH_THR_INDEX = [0, 5, 10, 15]          # of linspace(0.05, 0.8, 16)


def series_sha(x: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def zscore(v: np.ndarray) -> np.ndarray:
    return (v - v.mean()) / v.std()


def cases():
    """(name, series builder, dtype, combos, thresholds builder, measures).
    The builders are deterministic functions of the seeds; the tests call the
    same functions."""
    from accrqa_gb300 import workloads

    def lorenz():
        return workloads.lorenz_x(200_000, BENCH_SEED).astype(np.float32)

    def lorenz_thr(x):
        sd = float(np.std(x.astype(np.float64)))
        return (np.linspace(0.05, 0.8, 16) * sd).astype(np.float32)[BENCH_THR_INDEX]

    def shaped(gen, dt):
        def f():
            return zscore(gen(200_000, BENCH_SEED + 7)).astype(dt)
        return f

    def shaped_thr(x):
        sd = float(np.std(x.astype(np.float64)))
        return (np.array([0.1, 0.2, 0.5, 1.0]) * sd).astype(x.dtype)

    out = [("lorenz200k", lorenz, [(1, 3), (8, 8)], lorenz_thr, ("rr", "det", "lam"))]
    for name, gen in (("white200k", workloads.white), ("ar1200k", workloads.ar1)):
        for dt in (np.float32, np.float64):
            out.append((f"{name}_{np.dtype(dt).name}", shaped(gen, dt), [(1, 5)], shaped_thr,
                        ("rr", "det")))
    return out


def sparse(h: np.ndarray):
    nz = np.nonzero(h)[0]
    return nz.astype(np.int64), h[nz].astype(np.uint64)


def main() -> None:
    from oracle import oracle
    if oracle.ref_lib() is None:
        raise SystemExit("oracle/_ref/libaccrqa_ref.so is missing: run "
                         "`make -C oracle ref REF=<reference tree>` first")
    table = {"generator": "tests/golden/make_fullsize.py", "source": "reference CPU code",
             "threads": oracle.num_threads(), "cases": []}
    arrays = {}
    for name, build, combos, thr_of, measures in cases():
        x = build()
        thr = thr_of(x)
        entry = {"name": name, "n": int(len(x)), "dtype": np.dtype(x.dtype).name,
                 "sha256": series_sha(x), "norm": 1,
                 "thresholds_hex": [t.tobytes().hex() for t in thr],
                 "combos": []}
        for tau, emb in combos:
            c = {"tau": tau, "emb": emb, "nc": int(len(x) - (emb - 1) * tau)}
            t0 = time.time()
            if "rr" in measures:
                c["rr"] = [int(v) for v in oracle.rr_counts(x, tau, emb, thr, 1, use_ref=True)]
            for kind in ("det", "lam"):
                if kind not in measures:
                    continue
                for k, t in enumerate(thr):
                    h = (oracle.det_hist if kind == "det" else oracle.lam_hist)(
                        x, tau, emb, t, 1, use_ref=True)
                    ln, ct = sparse(h)
                    key = f"{name}/t{tau}e{emb}/{kind}/{k}"
                    arrays[key + "/len"] = ln
                    arrays[key + "/cnt"] = ct
            c["seconds"] = round(time.time() - t0, 1)
            entry["combos"].append(c)
            print(f"{name} tau={tau} emb={emb}: {c['seconds']} s", flush=True)
        table["cases"].append(entry)
    np.savez_compressed(os.path.join(HERE, "fullsize.npz"), **arrays)
    with open(os.path.join(HERE, "fullsize.json"), "w") as f:
        json.dump(table, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
