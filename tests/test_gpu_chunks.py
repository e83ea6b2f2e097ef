"""GPU: chunked line walks equal whole-line walks, and level walks equal
distance walks, bit for bit.

The DET/LAM kernels split lines into equal chunks when the caller gives
scratch for the chunk boundary records, and join the runs that cross chunk
boundaries in a second kernel.  Given plane memory as well, they first store
the threshold levels of every upper-triangle tile and walk the lines from
those (each unordered pair evaluated once).  Here the same pass is enqueued
through the kernel library's C ABI (accrqa_gb300_launch_walk) with and
without scratch and planes, and the histograms and longest-line markers must
be identical -- with a threshold that makes every cell recurrent (every
chunk full, one run per line), one that makes almost none recurrent, and a
spread between; with 4, 8 and 16 slots, series lengths that are and are not
multiples of the 32-cell tiles, and both norms.
"""
import ctypes

import numpy as np
import pytest

from accrqa_gb300 import _lib, engine, workloads

pytestmark = pytest.mark.gpu

MAX_THR = 16
WALK_DET, WALK_LAM = 1, 2


class WalkDesc(ctypes.Structure):
    """accrqa_walk_desc of accrqa_gb300/csrc/engine_abi.h."""
    _fields_ = [
        ("kind", ctypes.c_int32), ("dtype", ctypes.c_int32), ("norm", ctypes.c_int32),
        ("tau", ctypes.c_int32), ("emb", ctypes.c_int32), ("nthr", ctypes.c_int32),
        ("nc", ctypes.c_int64), ("d_x", ctypes.c_void_p),
        ("keys", ctypes.c_uint64 * MAX_THR),
        ("d_counts", ctypes.c_void_p), ("d_hist", ctypes.c_void_p),
        ("hist_stride", ctypes.c_int64), ("d_maxlen", ctypes.c_void_p),
        ("d_xhi", ctypes.c_void_p), ("d_xlo", ctypes.c_void_p),
        ("filter_keys", ctypes.c_uint64 * MAX_THR),
        ("d_scratch", ctypes.c_void_p), ("scratch_bytes", ctypes.c_int64),
        ("d_planes", ctypes.c_void_p), ("planes_bytes", ctypes.c_int64),
        ("planes_ready", ctypes.c_int32), ("pad_", ctypes.c_int32),
    ]


def _walk(torch, lib, kind, dx, dt, n, tau, emb, thr, norm, chunked, levels=False,
          planes=None, ready=False):
    nc = n - (emb - 1) * tau
    keys = engine.threshold_keys(thr, dt, norm)
    hist = torch.zeros((len(thr), nc + 1), dtype=torch.int64, device="cuda")
    mx = torch.zeros(MAX_THR, dtype=torch.int32, device="cuda")
    d = WalkDesc()
    d.kind, d.dtype, d.norm = kind, engine.F32 if dt == np.float32 else engine.F64, norm
    d.tau, d.emb, d.nthr, d.nc = tau, emb, len(thr), nc
    d.d_x = dx.data_ptr()
    for k in range(len(thr)):
        d.keys[k] = int(keys[k])
    d.d_hist, d.hist_stride, d.d_maxlen = hist.data_ptr(), nc + 1, mx.data_ptr()
    scratch = None
    if chunked:
        want = lib.accrqa_gb300_walk_scratch_bytes(ctypes.byref(d))
        assert want > 0, "this size must chunk"
        scratch = torch.empty(want, dtype=torch.uint8, device="cuda")
        d.d_scratch, d.scratch_bytes = scratch.data_ptr(), want
    if levels:
        pb = lib.accrqa_gb300_walk_plane_bytes(ctypes.byref(d))
        assert pb > 0
        if planes is None:
            planes = torch.empty(pb, dtype=torch.uint8, device="cuda")
        d.d_planes, d.planes_bytes = planes.data_ptr(), pb
        d.planes_ready = 1 if ready else 0
    st = torch.cuda.current_stream().cuda_stream
    assert lib.accrqa_gb300_launch_walk(ctypes.byref(d), ctypes.c_void_p(st)) == 0
    torch.cuda.synchronize()
    return hist.cpu().numpy(), mx.cpu().numpy()[:len(thr)]


def _bind(lib):
    for f in (lib.accrqa_gb300_walk_scratch_bytes, lib.accrqa_gb300_walk_plane_bytes):
        f.restype = ctypes.c_int64
        f.argtypes = [ctypes.c_void_p]
    lib.accrqa_gb300_launch_walk.argtypes = [ctypes.c_void_p, ctypes.c_void_p]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("kind", [WALK_DET, WALK_LAM])
@pytest.mark.parametrize("n,tau,emb,norm", [(20000, 1, 3, 1), (9000, 2, 5, 2), (3001, 1, 1, 1)])
def test_chunked_equals_whole(kind, dt, n, tau, emb, norm):
    torch = pytest.importorskip("torch")
    lib = _lib.handle()
    _bind(lib)
    x = workloads.logistic(n, 7 + n).astype(dt)
    # 0: exact matches only; 4.0: beyond the largest distance (all recurrent)
    thr = np.array([0.0, 0.01, 0.05, 0.1, 0.2, 0.3, 0.5, 0.8, 1.2, 4.0], dtype=dt)
    dx = torch.zeros(n + 128, dtype=torch.float32 if dt == np.float32 else torch.float64,
                     device="cuda")
    dx[:n] = torch.from_numpy(x).cuda()
    h0, m0 = _walk(torch, lib, kind, dx, dt, n, tau, emb, thr, norm, chunked=False)
    h1, m1 = _walk(torch, lib, kind, dx, dt, n, tau, emb, thr, norm, chunked=True)
    np.testing.assert_array_equal(h1, h0)
    np.testing.assert_array_equal(m1, m0)
    nc = n - (emb - 1) * tau
    if kind == WALK_LAM:
        assert h0[-1, nc] == nc          # every row one run of nc cells
    else:
        assert h0[-1, 1:].sum() == nc - 1  # every strict-upper diagonal one run


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("kind", [WALK_DET, WALK_LAM])
@pytest.mark.parametrize("nthr", [3, 8, 10])
@pytest.mark.parametrize("n,tau,emb,norm", [(20000, 1, 3, 1), (9000, 2, 5, 2), (3001, 1, 1, 1),
                                            (4096, 3, 4, 2), (97, 1, 2, 1), (33, 1, 1, 2)])
def test_levels_equal_distance_walk(kind, dt, nthr, n, tau, emb, norm):
    torch = pytest.importorskip("torch")
    lib = _lib.handle()
    _bind(lib)
    x = workloads.logistic(n, 11 + n).astype(dt)
    thr = np.array([0.0, 0.01, 0.05, 0.1, 0.2, 0.3, 0.5, 0.8, 1.2, 4.0], dtype=dt)
    thr = thr[np.linspace(0, len(thr) - 1, nthr).astype(int)] if nthr <= len(thr) else thr
    dx = torch.zeros(n + 128, dtype=torch.float32 if dt == np.float32 else torch.float64,
                     device="cuda")
    dx[:n] = torch.from_numpy(x).cuda()
    h0, m0 = _walk(torch, lib, kind, dx, dt, n, tau, emb, thr, norm, chunked=False)
    chunked = n >= 3000   # these sizes split their lines into chunks
    for ch in ([False, True] if chunked else [False]):
        h1, m1 = _walk(torch, lib, kind, dx, dt, n, tau, emb, thr, norm, chunked=ch, levels=True)
        np.testing.assert_array_equal(h1, h0)
        np.testing.assert_array_equal(m1, m0)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n,tau,emb,norm", [(20000, 1, 3, 1), (4096, 3, 4, 2), (97, 1, 2, 1)])
def test_det_from_planes_a_lam_pass_left(dt, n, tau, emb, norm):
    """A DET pass given the planes an earlier LAM pass of the same series
    stored (planes_ready) skips the tile walk and still equals the distance
    walk."""
    torch = pytest.importorskip("torch")
    lib = _lib.handle()
    _bind(lib)
    x = workloads.logistic(n, 13 + n).astype(dt)
    thr = np.array([0.0, 0.05, 0.1, 0.3, 0.8, 4.0], dtype=dt)
    dx = torch.zeros(n + 128, dtype=torch.float32 if dt == np.float32 else torch.float64,
                     device="cuda")
    dx[:n] = torch.from_numpy(x).cuda()
    d = WalkDesc()
    d.kind, d.nc, d.nthr = WALK_LAM, n - (emb - 1) * tau, len(thr)
    planes = torch.empty(lib.accrqa_gb300_walk_plane_bytes(ctypes.byref(d)), dtype=torch.uint8,
                         device="cuda")
    ch = n >= 3000
    hl, _ = _walk(torch, lib, WALK_LAM, dx, dt, n, tau, emb, thr, norm, chunked=ch,
                  levels=True, planes=planes)
    hd, md = _walk(torch, lib, WALK_DET, dx, dt, n, tau, emb, thr, norm, chunked=ch,
                   levels=True, planes=planes, ready=True)
    h0, m0 = _walk(torch, lib, WALK_DET, dx, dt, n, tau, emb, thr, norm, chunked=False)
    np.testing.assert_array_equal(hd, h0)
    np.testing.assert_array_equal(md, m0)
    h1, _ = _walk(torch, lib, WALK_LAM, dx, dt, n, tau, emb, thr, norm, chunked=False)
    np.testing.assert_array_equal(hl, h1)
