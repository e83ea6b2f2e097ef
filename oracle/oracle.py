"""ctypes front-end to the test oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liboracle.so`` (the C restatement of the AccRQA reference
algorithm in ``accrqa_oracle.c``) and, where it was built, the reference's own
CPU code in ``oracle/_ref/libaccrqa_ref.so``.  Only the tests, the smoke check
and the CPU-baseline leg of ``bench.py`` import this module; the product
library never does.

All functions take numpy arrays and return numpy arrays.  Histograms are
``uint64`` arrays of ``nc + 1`` bins, ``nc = n - (emb - 1) * tau``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_u64p = ctypes.POINTER(ctypes.c_uint64)
_i64 = ctypes.c_int64


def build(quiet: bool = True) -> None:
    """Compile liboracle.so, and the reference's own CPU code into _ref/ when
    ACCRQA_REFERENCE_TREE names a reference source tree (skipped otherwise)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True,
                   stdout=out)
    ref_root = os.environ.get("ACCRQA_REFERENCE_TREE", "")
    if ref_root and os.path.isdir(os.path.join(ref_root, "src")):
        subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF={ref_root}"],
                       check=True, stdout=out)


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        _LIB = ctypes.CDLL(path)
    return _LIB


def ref_lib():
    """The reference's own CPU code, or None where it was not built."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libaccrqa_ref.so")
        if not os.path.exists(path):
            return None
        _REF = ctypes.CDLL(path)
    return _REF


def _suffix(x: np.ndarray) -> tuple[str, type]:
    if x.dtype == np.float32:
        return "f32", ctypes.c_float
    if x.dtype == np.float64:
        return "f64", ctypes.c_double
    raise TypeError("series must be float32 or float64")


def nc_of(n: int, tau: int, emb: int) -> int:
    return n - (emb - 1) * tau


def set_threads(n: int) -> None:
    lib().oracle_set_threads(ctypes.c_int(n))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


# --------------------------------------------------------------------------
# Restatement (liboracle.so)
# --------------------------------------------------------------------------
def rr_counts(x, tau, emb, thresholds, dist, use_ref=False):
    x = np.ascontiguousarray(x)
    suf, ct = _suffix(x)
    thr = np.ascontiguousarray(thresholds, dtype=x.dtype)
    out = np.zeros(len(thr), dtype=np.uint64)
    L = ref_lib() if use_ref else lib()
    fn = getattr(L, ("ref_rr_counts_" if use_ref else "oracle_rr_counts_") + suf)
    fn(_ptr(out, ctypes.c_uint64), _ptr(x, ct), _i64(len(x)), ctypes.c_int(tau),
       ctypes.c_int(emb), _ptr(thr, ct), ctypes.c_int(len(thr)),
       ctypes.c_int(dist))
    return out


def _hist(kind, x, tau, emb, threshold, dist, use_ref):
    x = np.ascontiguousarray(x)
    suf, ct = _suffix(x)
    nc = nc_of(len(x), tau, emb)
    out = np.zeros(nc + 1, dtype=np.uint64)
    L = ref_lib() if use_ref else lib()
    fn = getattr(L, ("ref_" if use_ref else "oracle_") + kind + "_hist_" + suf)
    fn(_ptr(out, ctypes.c_uint64), _ptr(x, ct), _i64(len(x)), ctypes.c_int(tau),
       ctypes.c_int(emb), ct(float(threshold)), ctypes.c_int(dist))
    return out


def det_hist(x, tau, emb, threshold, dist, use_ref=False):
    return _hist("det", x, tau, emb, threshold, dist, use_ref)


def lam_hist(x, tau, emb, threshold, dist, use_ref=False):
    return _hist("lam", x, tau, emb, threshold, dist, use_ref)


def rp(x, tau, emb, threshold, dist, use_ref=False):
    x = np.ascontiguousarray(x)
    suf, ct = _suffix(x)
    nc = nc_of(len(x), tau, emb)
    out = np.zeros((nc, nc), dtype=np.int8)
    L = ref_lib() if use_ref else lib()
    fn = getattr(L, ("ref_rp_u8_" if use_ref else "oracle_rp_u8_") + suf)
    fn(out.ctypes.data_as(ctypes.c_void_p), _ptr(x, ct), _i64(len(x)),
       ctypes.c_int(tau), ctypes.c_int(emb), ct(float(threshold)),
       ctypes.c_int(dist))
    return out


def rp_i32(x, tau, emb, threshold, dist):
    x = np.ascontiguousarray(x, dtype=np.float64)
    nc = nc_of(len(x), tau, emb)
    out = np.zeros((nc, nc), dtype=np.int32)
    lib().oracle_rp_i32_f64(out.ctypes.data_as(ctypes.c_void_p),
                            _ptr(x, ctypes.c_double), _i64(len(x)),
                            ctypes.c_int(tau), ctypes.c_int(emb),
                            ctypes.c_double(threshold), ctypes.c_int(dist))
    return out


def det_sample(x, tau, emb, threshold, dist, d_begin, d_end):
    """DET run histogram over diagonals [d_begin, d_end); returns (hist, cells)."""
    x = np.ascontiguousarray(x)
    suf, ct = _suffix(x)
    nc = nc_of(len(x), tau, emb)
    out = np.zeros(nc + 1, dtype=np.uint64)
    fn = getattr(lib(), "oracle_det_sample_" + suf)
    fn.restype = ctypes.c_uint64
    cells = fn(_ptr(out, ctypes.c_uint64), _ptr(x, ct), _i64(len(x)),
               ctypes.c_int(tau), ctypes.c_int(emb), ct(float(threshold)),
               ctypes.c_int(dist), _i64(d_begin), _i64(d_end))
    return out, int(cells)


def rr_sample(x, tau, emb, threshold, dist, r_begin, r_end):
    """Recurrent cells of rows [r_begin, r_end); returns (count, cells)."""
    x = np.ascontiguousarray(x)
    suf, ct = _suffix(x)
    cnt = np.zeros(1, dtype=np.uint64)
    fn = getattr(lib(), "oracle_rr_sample_" + suf)
    fn.restype = ctypes.c_uint64
    cells = fn(_ptr(cnt, ctypes.c_uint64), _ptr(x, ct), _i64(len(x)), ctypes.c_int(tau),
               ctypes.c_int(emb), ct(float(threshold)), ctypes.c_int(dist), _i64(r_begin),
               _i64(r_end))
    return int(cnt[0]), int(cells)


def lam_sample(x, tau, emb, threshold, dist, r_begin, r_end):
    """LAM run histogram + recurrent count over rows [r_begin, r_end)."""
    x = np.ascontiguousarray(x)
    suf, ct = _suffix(x)
    nc = nc_of(len(x), tau, emb)
    out = np.zeros(nc + 1, dtype=np.uint64)
    cnt = np.zeros(1, dtype=np.uint64)
    fn = getattr(lib(), "oracle_lam_sample_" + suf)
    fn.restype = ctypes.c_uint64
    cells = fn(_ptr(out, ctypes.c_uint64), _ptr(cnt, ctypes.c_uint64),
               _ptr(x, ct), _i64(len(x)), ctypes.c_int(tau), ctypes.c_int(emb),
               ct(float(threshold)), ctypes.c_int(dist), _i64(r_begin),
               _i64(r_end))
    return out, int(cnt[0]), int(cells)


# --------------------------------------------------------------------------
# Post-processing restatement and the reference GPU path's output formulas
# --------------------------------------------------------------------------
def measures(hist, lmin, is_det):
    """{DET|LAM, L|TT, Lmax|TTmax, ENTR, RR} from one histogram (doubles)."""
    h = np.ascontiguousarray(hist, dtype=np.uint64)
    out = np.zeros(5, dtype=np.float64)
    L = lib()
    L.oracle_measures(_ptr(out, ctypes.c_double), _ptr(h, ctypes.c_uint64),
                      _i64(len(h)), _i64(lmin), ctypes.c_int(1 if is_det else 0))
    return out


def rr_output(counts, nc, dtype):
    """RR as the reference GPU path writes it: (T)((double)count/(double)nc^2)."""
    return (np.asarray(counts, dtype=np.float64) / float(nc * nc)).astype(dtype)


def line_output(x, taus, embs, lmins, thresholds, dist, calc_entr, is_det):
    """Full DET or LAM output cube [nTau][nEmb][nLmin][nThr][5] as the
    reference's GPU path lays it out (src/AccRQA_functions.cpp:568-595 and
    :391-452), computed from oracle histograms."""
    x = np.ascontiguousarray(x)
    dt = x.dtype
    thr = np.asarray(thresholds, dtype=dt)
    out = np.zeros((len(taus), len(embs), len(lmins), len(thr), 5), dtype=dt)
    boxcar = not (calc_entr == 1 or max(lmins) >= 16)
    for a, tau in enumerate(taus):
        for b, emb in enumerate(embs):
            nc = nc_of(len(x), tau, emb)
            for k, t in enumerate(thr):
                h = (det_hist if is_det else lam_hist)(x, tau, emb, t, dist)
                for c, lm in enumerate(lmins):
                    m = measures(h, lm, is_det)
                    if boxcar:
                        # src/AccRQA-GPU-HST.cu:2438-2449 and :2626-2636: the
                        # boxcar path leaves Lmax/ENTR undefined (NaN in the
                        # output) and normalises RR by (nc-1)^2.
                        m[2] = np.nan
                        m[3] = np.nan
                        with np.errstate(divide="ignore", invalid="ignore"):
                            m[4] = np.float64(m[4] * nc * nc) / np.float64(
                                (nc - 1) * (nc - 1))
                    out[a, b, c, k, :] = m.astype(dt)
    return out


# --------------------------------------------------------------------------
# Reference CPU API (oracle/_ref), for golden-vector generation
# --------------------------------------------------------------------------
def ref_api_det_lam(kind, x, taus, embs, lmins, thresholds, dist, entr):
    x = np.ascontiguousarray(x, dtype=np.float64)
    taus = np.ascontiguousarray(taus, dtype=np.int32)
    embs = np.ascontiguousarray(embs, dtype=np.int32)
    lm = np.ascontiguousarray(lmins, dtype=np.int32)
    thr = np.ascontiguousarray(thresholds, dtype=np.float64)
    out = np.zeros(len(taus) * len(embs) * len(lm) * len(thr) * 5)
    fn = getattr(ref_lib(), f"ref_api_{kind}_f64")
    i32p = ctypes.POINTER(ctypes.c_int)
    err = fn(_ptr(out, ctypes.c_double), _ptr(x, ctypes.c_double),
             ctypes.c_size_t(len(x)), _ptr(taus, ctypes.c_int), len(taus),
             _ptr(embs, ctypes.c_int), len(embs), _ptr(lm, ctypes.c_int),
             len(lm), _ptr(thr, ctypes.c_double), len(thr), dist, entr)
    assert err == 0, err
    return out


def ref_api_rr(x, taus, embs, thresholds, dist):
    x = np.ascontiguousarray(x)
    suf, ct = _suffix(x)
    taus = np.ascontiguousarray(taus, dtype=np.int32)
    embs = np.ascontiguousarray(embs, dtype=np.int32)
    thr = np.ascontiguousarray(thresholds, dtype=x.dtype)
    out = np.zeros(len(taus) * len(embs) * len(thr), dtype=x.dtype)
    fn = getattr(ref_lib(), f"ref_api_RR_{suf}")
    err = fn(_ptr(out, ct), _ptr(x, ct), ctypes.c_size_t(len(x)),
             _ptr(taus, ctypes.c_int), len(taus), _ptr(embs, ctypes.c_int),
             len(embs), _ptr(thr, ct), len(thr), dist)
    assert err == 0, err
    return out
