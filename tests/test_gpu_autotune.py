"""GPU: the autotuner picks the balanced walks' chunk granularity, and results
do not depend on it.

accrqa_gb300_autotune times work units per resident warp (RR {4, 8, 16}, DET
and LAM {8, 16, 32}) for three length classes and installs the fastest; the
report must list a valid choice for every walk and class, and the passes
that follow must still equal the oracle bit for bit.
"""
import re

import numpy as np
import pytest

from accrqa_gb300 import workloads

pytestmark = pytest.mark.gpu


def test_autotune_choices_and_parity_after(gpu, oracle_mod):
    report = gpu.autotune()
    classes = report.split(";")
    assert len(classes) == 3, report
    for c in classes:
        for name, cands in (("RR", {4, 8, 16}), ("DET", {8, 16, 32}), ("LAM", {8, 16, 32})):
            m = re.search(rf"\b{name} (\d+) \(", c)
            assert m and int(m.group(1)) in cands, (name, c)
    x = workloads.lorenz_x(20000, 9, transient=500).astype(np.float32)
    x = (x / np.std(x.astype(np.float64))).astype(np.float32)
    thr = np.array([0.1, 0.4], np.float32)
    np.testing.assert_array_equal(gpu.rr_counts(x, 2, 4, thr, 1),
                                  oracle_mod.rr_counts(x, 2, 4, thr, 1))
    det = gpu.det_histograms(x, 2, 4, thr, 1)
    lam = gpu.lam_histograms(x, 2, 4, thr, 1)
    for k, t in enumerate(thr):
        np.testing.assert_array_equal(det[k], oracle_mod.det_hist(x, 2, 4, t, 1))
        np.testing.assert_array_equal(lam[k], oracle_mod.lam_hist(x, 2, 4, t, 1))
