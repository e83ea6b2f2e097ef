"""Device entry points recorded into a CUDA graph and replayed.

A caller that keeps its series on the device can record the RR, DET and LAM
passes (accrqa_gb300_{rr_counts,det_hist,lam_hist}_dev) into a CUDA graph
and replay it.  While its stream is being captured a DET or LAM pass takes no
stream-ordered scratch, so the graph holds no allocation: it walks its lines
whole instead of in chunks (engine.cpp, line_scratch_alloc).  RR needs no
scratch either way.  Every replay must give the eager passes' counts and
histograms bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("norm", [1, 2])
def test_captured_passes_equal_eager(gpu, norm):
    import torch

    from accrqa_gb300 import workloads

    n, tau, emb = 6000, 2, 4
    x = workloads.lorenz_x(n, 11).astype(np.float32)
    thr = (np.linspace(0.05, 0.8, 8) * float(np.std(x.astype(np.float64)))).astype(np.float32)
    nc = n - (emb - 1) * tau
    dx = torch.zeros(n + 128, dtype=torch.float32, device="cuda")
    dx[:n].copy_(torch.from_numpy(x))
    counts = torch.zeros(len(thr), dtype=torch.int64, device="cuda")
    det = torch.zeros((len(thr), nc + 1), dtype=torch.int64, device="cuda")
    lam = torch.zeros((len(thr), nc + 1), dtype=torch.int64, device="cuda")
    dmax = torch.zeros(len(thr), dtype=torch.int32, device="cuda")
    lmax = torch.zeros(len(thr), dtype=torch.int32, device="cuda")

    def passes(stream):
        counts.zero_()
        det.zero_()
        lam.zero_()
        dmax.zero_()
        lmax.zero_()
        gpu.rr_counts_dev(counts.data_ptr(), dx.data_ptr(), 0, n, tau, emb, thr, norm, stream)
        gpu.det_hist_dev(det.data_ptr(), nc + 1, dmax.data_ptr(), dx.data_ptr(), 0, n, tau,
                         emb, thr, norm, stream)
        gpu.lam_hist_dev(lam.data_ptr(), nc + 1, lmax.data_ptr(), dx.data_ptr(), 0, n, tau,
                         emb, thr, norm, stream)

    def snapshot():
        torch.cuda.synchronize()
        return [t.cpu().numpy().copy() for t in (counts, det, lam, dmax, lmax)]

    passes(torch.cuda.current_stream().cuda_stream)
    eager = snapshot()
    assert eager[0].sum() > 0 and eager[1].sum() > 0 and eager[2].sum() > 0

    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        passes(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        for t in (counts, det, lam, dmax, lmax):
            t.fill_(-1)
        graph.replay()
        got = snapshot()
        for name, a, b in zip(("RR", "DET", "LAM", "DET longest", "LAM longest"), got, eager):
            assert np.array_equal(a, b), name
