"""Engine-level entry points of libaccrqa.so (numpy in, numpy out).

These return the integers behind the RQA measures -- recurrent-cell counts
and line-length histograms -- and are what the parity tests compare with the
oracle.  The device-resident variants take raw device pointers (for example
``tensor.data_ptr()``) and a CUDA stream handle.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

F32, F64 = 0, 1
EUCLIDEAN, MAXIMAL = 1, 2
NORMS = {"euclidean": EUCLIDEAN, "maximal": MAXIMAL, 1: EUCLIDEAN, 2: MAXIMAL}


class EngineError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what} failed with AccRQA error {code}: {_lib.last_error()}")
        self.code = code


def _check(code: int, what: str) -> None:
    if code != 0:
        raise EngineError(code, what)


def _dtype_code(x: np.ndarray) -> int:
    if x.dtype == np.float32:
        return F32
    if x.dtype == np.float64:
        return F64
    raise TypeError("series must be float32 or float64")


def _norm(norm) -> int:
    try:
        return NORMS[norm]
    except KeyError:
        raise ValueError(f"unknown norm {norm!r}") from None


def _vp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _u64p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))


def embedded_length(n: int, tau: int, emb: int) -> int:
    return n - (emb - 1) * tau


def device_count() -> int:
    return int(_lib.handle().accrqa_gb300_device_count())


def threshold_keys(thresholds, dtype, norm) -> np.ndarray:
    """Comparison keys the kernels use (see include/accrqa_gb300.h)."""
    thr = np.ascontiguousarray(thresholds, dtype=dtype)
    keys = np.zeros(len(thr), dtype=np.uint64)
    _check(_lib.handle().accrqa_gb300_threshold_keys(
        _u64p(keys), _vp(thr), _dtype_code(thr), len(thr), _norm(norm)),
        "threshold_keys")
    return keys


def rr_counts(x, tau: int, emb: int, thresholds, norm) -> np.ndarray:
    """Full-matrix recurrent-cell count per threshold (uint64)."""
    x = np.ascontiguousarray(x)
    thr = np.ascontiguousarray(thresholds, dtype=x.dtype)
    out = np.zeros(len(thr), dtype=np.uint64)
    _check(_lib.handle().accrqa_gb300_rr_counts(
        _u64p(out), _vp(x), _dtype_code(x), len(x), tau, emb, _vp(thr), len(thr),
        _norm(norm)), "rr_counts")
    return out


def _hist(fn_name, x, tau, emb, thresholds, norm):
    x = np.ascontiguousarray(x)
    thr = np.ascontiguousarray(thresholds, dtype=x.dtype)
    nc = embedded_length(len(x), tau, emb)
    out = np.zeros((len(thr), max(nc, 0) + 1), dtype=np.uint64)
    _check(getattr(_lib.handle(), fn_name)(
        _u64p(out), _vp(x), _dtype_code(x), len(x), tau, emb, _vp(thr), len(thr),
        _norm(norm)), fn_name)
    return out


def det_histograms(x, tau: int, emb: int, thresholds, norm) -> np.ndarray:
    """Diagonal-line histograms [nthr][nc+1] in the reference convention."""
    return _hist("accrqa_gb300_det_histograms", x, tau, emb, thresholds, norm)


def lam_histograms(x, tau: int, emb: int, thresholds, norm) -> np.ndarray:
    """Vertical-line histograms [nthr][nc+1] over the full matrix."""
    return _hist("accrqa_gb300_lam_histograms", x, tau, emb, thresholds, norm)


def rp(x, tau: int, emb: int, threshold: float, norm, out_dtype=np.int8) -> np.ndarray:
    """Recurrence plot [nc][nc] as int8 or int32."""
    x = np.ascontiguousarray(x)
    nc = embedded_length(len(x), tau, emb)
    out = np.zeros((max(nc, 0), max(nc, 0)), dtype=out_dtype)
    ot = 1 if np.dtype(out_dtype) == np.int8 else 2
    _check(_lib.handle().accrqa_gb300_rp(
        _vp(out), ot, _vp(x), _dtype_code(x), len(x), tau, emb, float(threshold),
        _norm(norm)), "rp")
    return out


def rp_bits(x, tau: int, emb: int, threshold: float, norm) -> np.ndarray:
    """Bit-packed recurrence plot: uint32 [nc][ceil(nc/32)], bit c of word w
    of row i = cell (i, 32*w + c)."""
    x = np.ascontiguousarray(x)
    nc = embedded_length(len(x), tau, emb)
    out = np.zeros((max(nc, 0), max((nc + 31) // 32, 0)), dtype=np.uint32)
    _check(_lib.handle().accrqa_gb300_rp_bits(
        _vp(out), _vp(x), _dtype_code(x), len(x), tau, emb, float(threshold), _norm(norm)),
        "rp_bits")
    return out


def rp_bits_dev(d_out: int, d_x: int, dtype_code: int, n: int, tau: int, emb: int,
                threshold: float, norm, stream: int = 0) -> None:
    """Enqueue the bit-packed plot of a device series (>= n + 128 elements)
    into device memory d_out (nc * ceil(nc/32) uint32) on `stream`."""
    _check(_lib.handle().accrqa_gb300_rp_bits_dev(
        ctypes.c_void_p(d_out), ctypes.c_void_p(d_x), dtype_code, n, tau, emb, float(threshold),
        _norm(norm), ctypes.c_void_p(stream)), "rp_bits_dev")


def unpack_rp_bits(bits: np.ndarray, nc: int) -> np.ndarray:
    """int8 [nc][nc] plot from its bit-packed form."""
    b = np.unpackbits(bits.view(np.uint8).reshape(bits.shape[0], -1), axis=1, bitorder="little")
    return b[:, :nc].astype(np.int8)


def measures(hist, lmin: int, is_det: bool) -> np.ndarray:
    """{DET|LAM, L|TT, Lmax|TTmax, ENTR, RR} of one histogram (float64)."""
    h = np.ascontiguousarray(hist, dtype=np.uint64)
    out = np.zeros(5, dtype=np.float64)
    _check(_lib.handle().accrqa_gb300_measures(
        out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), _u64p(h), len(h), lmin,
        1 if is_det else 0), "measures")
    return out


# ---------------------------------------------------------------------------
# Many series in one submission
# ---------------------------------------------------------------------------
class SeriesJob(ctypes.Structure):
    """accrqa_gb300_series_job (include/accrqa_gb300.h)."""
    _fields_ = [("x", ctypes.c_void_p), ("n", ctypes.c_int64), ("dtype", ctypes.c_int32),
                ("tau", ctypes.c_int32), ("emb", ctypes.c_int32), ("norm", ctypes.c_int32),
                ("thresholds", ctypes.c_void_p), ("nthr", ctypes.c_int32),
                ("lmin", ctypes.c_int32), ("vmin", ctypes.c_int32), ("calc_entr", ctypes.c_int32),
                ("rr_out", ctypes.c_void_p), ("det_out", ctypes.c_void_p),
                ("lam_out", ctypes.c_void_p)]


def batch(jobs, measures=("rr", "det", "lam")):
    """Run RR/DET/LAM for many series in one submission.

    jobs: list of dicts with keys x (float32/float64 array), tau, emb, norm,
    thresholds, and optional lmin (2), vmin (2), calc_entr (1).
    Returns a list of dicts {"rr": [nthr], "det": [nthr, 5], "lam": [nthr, 5]}.
    """
    arr = (SeriesJob * len(jobs))()
    keep, outs = [], []
    for i, j in enumerate(jobs):
        x = np.ascontiguousarray(j["x"])
        thr = np.ascontiguousarray(j["thresholds"], dtype=x.dtype)
        o = {}
        if "rr" in measures:
            o["rr"] = np.zeros(len(thr), dtype=x.dtype)
        if "det" in measures:
            o["det"] = np.zeros((len(thr), 5), dtype=x.dtype)
        if "lam" in measures:
            o["lam"] = np.zeros((len(thr), 5), dtype=x.dtype)
        keep += [x, thr]
        outs.append(o)
        arr[i] = SeriesJob(x.ctypes.data, len(x), _dtype_code(x), j["tau"], j["emb"],
                           _norm(j["norm"]), thr.ctypes.data, len(thr), j.get("lmin", 2),
                           j.get("vmin", 2), j.get("calc_entr", 1),
                           o["rr"].ctypes.data if "rr" in o else None,
                           o["det"].ctypes.data if "det" in o else None,
                           o["lam"].ctypes.data if "lam" in o else None)
    f = _lib.handle().accrqa_gb300_batch
    f.argtypes = [ctypes.POINTER(SeriesJob), ctypes.c_int32]
    f.restype = ctypes.c_int
    _check(f(arr, len(jobs)), "batch")
    return outs


def autotune() -> str:
    """Time the balanced walks' chunk granularity on this GPU and install the
    fastest per walk kind and length class (accrqa_gb300_autotune); returns
    the choices."""
    lib = _lib.handle()
    f = lib.accrqa_gb300_autotune
    f.argtypes = [ctypes.c_char_p, ctypes.c_int64]
    f.restype = ctypes.c_int
    buf = ctypes.create_string_buffer(1024)
    _check(f(buf, len(buf)), "autotune")
    return buf.value.decode()


class Server:
    """Continuous-batching request server (accrqa_gb300_server_*).

    submit(job) queues one series (dict as for batch(); "measures" selects
    any of "rr", "det", "lam") and returns a ticket; wait(ticket) returns
    (outputs, latency_ms)."""

    def __init__(self, workers: int = 2, hbm_fraction: float = 0.5):
        lib = _lib.handle()
        lib.accrqa_gb300_server_create.restype = ctypes.c_void_p
        lib.accrqa_gb300_server_create.argtypes = [ctypes.c_int32, ctypes.c_double]
        lib.accrqa_gb300_server_submit.restype = ctypes.c_int64
        lib.accrqa_gb300_server_submit.argtypes = [ctypes.c_void_p, ctypes.POINTER(SeriesJob)]
        lib.accrqa_gb300_server_wait.restype = ctypes.c_int
        lib.accrqa_gb300_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_int64,
                                                 ctypes.POINTER(ctypes.c_double)]
        lib.accrqa_gb300_server_stats.argtypes = [ctypes.c_void_p,
                                                  ctypes.POINTER(ctypes.c_uint64),
                                                  ctypes.POINTER(ctypes.c_uint64)]
        lib.accrqa_gb300_server_destroy.argtypes = [ctypes.c_void_p]
        self._lib = lib
        self._h = lib.accrqa_gb300_server_create(workers, hbm_fraction)
        if not self._h:
            raise EngineError(8, "server_create")
        self._pending = {}

    def submit(self, job) -> int:
        x = np.ascontiguousarray(job["x"])
        thr = np.ascontiguousarray(job["thresholds"], dtype=x.dtype)
        want = job.get("measures", ("rr", "det", "lam"))
        o = {}
        if "rr" in want:
            o["rr"] = np.zeros(len(thr), dtype=x.dtype)
        if "det" in want:
            o["det"] = np.zeros((len(thr), 5), dtype=x.dtype)
        if "lam" in want:
            o["lam"] = np.zeros((len(thr), 5), dtype=x.dtype)
        sj = SeriesJob(x.ctypes.data, len(x), _dtype_code(x), job["tau"], job["emb"],
                       _norm(job["norm"]), thr.ctypes.data, len(thr), job.get("lmin", 2),
                       job.get("vmin", 2), job.get("calc_entr", 1),
                       o["rr"].ctypes.data if "rr" in o else None,
                       o["det"].ctypes.data if "det" in o else None,
                       o["lam"].ctypes.data if "lam" in o else None)
        t = self._lib.accrqa_gb300_server_submit(self._h, ctypes.byref(sj))
        if t < 0:
            raise EngineError(int(-t), "server_submit")
        self._pending[t] = o
        return int(t)

    def wait(self, ticket: int):
        lat = ctypes.c_double(0.0)
        e = self._lib.accrqa_gb300_server_wait(self._h, ticket, ctypes.byref(lat))
        o = self._pending.pop(ticket)
        _check(e, "server_wait")
        return o, lat.value

    def stats(self):
        b, s = ctypes.c_uint64(), ctypes.c_uint64()
        self._lib.accrqa_gb300_server_stats(self._h, ctypes.byref(b), ctypes.byref(s))
        return int(b.value), int(s.value)

    def peak_bytes(self) -> int:
        """Most device bytes the admitted requests held at once."""
        self._lib.accrqa_gb300_server_peak_bytes.restype = ctypes.c_uint64
        self._lib.accrqa_gb300_server_peak_bytes.argtypes = [ctypes.c_void_p]
        return int(self._lib.accrqa_gb300_server_peak_bytes(self._h))

    def close(self):
        if self._h:
            self._lib.accrqa_gb300_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# ---------------------------------------------------------------------------
# Device-resident passes (pointers into device memory, enqueue only)
# ---------------------------------------------------------------------------
def rr_counts_dev(d_counts: int, d_x: int, dtype_code: int, n: int, tau: int, emb: int,
                  thresholds: np.ndarray, norm, stream: int = 0) -> None:
    thr = np.ascontiguousarray(thresholds,
                               dtype=np.float32 if dtype_code == F32 else np.float64)
    _check(_lib.handle().accrqa_gb300_rr_counts_dev(
        ctypes.c_void_p(d_counts), ctypes.c_void_p(d_x), dtype_code, n, tau, emb,
        _vp(thr), len(thr), _norm(norm), ctypes.c_void_p(stream)), "rr_counts_dev")


def _lines_dev(name, d_hist, stride, d_maxlen, d_x, dtype_code, n, tau, emb,
               thresholds, norm, stream):
    thr = np.ascontiguousarray(thresholds,
                               dtype=np.float32 if dtype_code == F32 else np.float64)
    _check(getattr(_lib.handle(), name)(
        ctypes.c_void_p(d_hist), stride, ctypes.c_void_p(d_maxlen), ctypes.c_void_p(d_x),
        dtype_code, n, tau, emb, _vp(thr), len(thr), _norm(norm),
        ctypes.c_void_p(stream)), name)


def det_hist_dev(d_hist, stride, d_maxlen, d_x, dtype_code, n, tau, emb, thresholds,
                 norm, stream=0) -> None:
    _lines_dev("accrqa_gb300_det_hist_dev", d_hist, stride, d_maxlen, d_x, dtype_code,
               n, tau, emb, thresholds, norm, stream)


def lam_hist_dev(d_hist, stride, d_maxlen, d_x, dtype_code, n, tau, emb, thresholds,
                 norm, stream=0) -> None:
    _lines_dev("accrqa_gb300_lam_hist_dev", d_hist, stride, d_maxlen, d_x, dtype_code,
               n, tau, emb, thresholds, norm, stream)


def probe_fp32(mode: int = 1, reps: int = 20) -> float:
    """Measured separately rounded multiply/add rate of the current device in
    operations per second (mode 0 FP32 scalar, 1 packed f32x2, 2 FP64)."""
    out = ctypes.c_double(0.0)
    code = _lib.handle().accrqa_gb300_probe_fp32(int(mode), int(reps), ctypes.byref(out))
    if code:
        raise EngineError(f"rate probe failed: CUDA error {code}")
    return float(out.value)
