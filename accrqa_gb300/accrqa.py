"""Python front-end with the AccRQA reference's interface (src/accrqa).

Same function names, arguments, defaults, output shapes and exceptions as the
reference's ``accrqa`` package (src/accrqa/accrqa.py:22-594): ``RP``, ``RR``,
``DET``, ``LAM`` and ``RR_target``, and the helper classes
``accrqaDistance``, ``accrqaCompPlatform``, ``accrqaError`` and
``accrqaMem``.  Calls go through the same C symbols (``py_accrqa_*`` on
``Mem`` handles) of libaccrqa.so.  ``tidy_data=True`` (the reference's
default) needs pandas, exactly as in the reference.
"""
from __future__ import annotations

import ctypes
import sys
from typing import Optional

import numpy as np

from . import _lib


class accrqaError:
    """Error status passed to the library (src/accrqa/accrqa_error.py)."""

    error_codes = {
        0: "AccRQA: No error",
        1: "AccRQA: Generic runtime error",
        2: "AccRQA: Invalid function argument",
        3: "AccRQA: Unsupported data type(s)",
        4: "AccRQA: Memory allocation failure",
        5: "AccRQA: Memory copy failure",
        6: "AccRQA: Memory location mismatch",
        7: "AccRQA: CUDA not found",
        8: "AccRQA: CUDA device not found",
        9: "AccRQA: Not enough memory on the CUDA device",
        10: "AccRQA: CUDA error",
        11: "AccRQA: Invalid metric type",
    }

    def __init__(self):
        self._error = ctypes.c_int(0)

    def check(self):
        if self._error.value != 0:
            msg = self.error_codes.get(self._error.value, "AccRQA: unknown error")
            detail = _lib.last_error()
            raise RuntimeError(msg + (f" ({detail})" if detail else ""))

    def handle(self):
        return ctypes.byref(self._error)

    @staticmethod
    def handle_type():
        return ctypes.POINTER(ctypes.c_int)


class accrqaDistance:
    """Norm selector (src/accrqa/accrqa_distance.py)."""

    distance_types = {1: "euclidean", 2: "maximal"}

    def __init__(self, distance_type: str):
        rev = {v: k for k, v in self.distance_types.items()}
        if distance_type not in rev:
            raise ValueError(f"Unknown distance type: {distance_type}")
        self._distance = ctypes.c_int(rev[distance_type])

    def get_distance_id(self) -> int:
        return self._distance.value

    def get_distance_name(self) -> str:
        return self.distance_types.get(self._distance.value, "Unknown distance")


class accrqaCompPlatform:
    """Platform selector (src/accrqa/accrqa_compplatform.py)."""

    comp_platforms = {1: "cpu", 1024: "nv_gpu"}

    def __init__(self, comp_platform: str):
        rev = {v: k for k, v in self.comp_platforms.items()}
        if comp_platform not in rev:
            raise ValueError(f"Unknown computational platform: {comp_platform}")
        self._platform = ctypes.c_int(rev[comp_platform])

    def get_platform_id(self) -> int:
        return self._platform.value

    def get_platform_name(self) -> str:
        return self.comp_platforms.get(self._platform.value, "Unknown platform")


class accrqaMem:
    """Mem handle around a numpy array (src/accrqa/accrqa_mem.py)."""

    class Handle(ctypes.Structure):
        pass

    _types = {np.dtype(np.int8): 1, np.dtype(np.int32): 2, np.dtype(np.float32): 4,
              np.dtype(np.float64): 8, np.dtype(np.complex64): 36,
              np.dtype(np.complex128): 40}

    def __init__(self, obj):
        self._handle = None
        lib = _lib.handle()
        create = lib.mem_create_wrapper
        create.restype = accrqaMem.handle_type()
        create.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int32,
                           ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                           accrqaError.handle_type()]
        ro = lib.mem_set_read_only
        ro.argtypes = [accrqaMem.handle_type(), ctypes.c_int32]
        err = accrqaError()
        if not isinstance(obj, np.ndarray):
            raise TypeError("Unknown array type")
        if obj.dtype not in self._types:
            raise TypeError("Unsupported type of numpy array")
        shape = (ctypes.c_int64 * obj.ndim)(*obj.shape)
        strides = (ctypes.c_int64 * obj.ndim)(*obj.strides)
        self._keep = obj
        self._handle = create(obj.ctypes.data_as(ctypes.c_void_p), self._types[obj.dtype], 0,
                              obj.ndim, shape, strides, err.handle())
        ro(self._handle, int(not obj.flags.writeable))
        err.check()

    def __del__(self):
        if getattr(self, "_handle", None):
            f = _lib.handle().mem_free
            f.argtypes = [accrqaMem.handle_type()]
            f(self._handle)
            self._handle = None

    def handle(self):
        return self._handle

    @staticmethod
    def handle_type():
        return ctypes.POINTER(accrqaMem.Handle)


def _pandas():
    return sys.modules.get("pandas")


def _check_common(tidy_data):
    if tidy_data is True and _pandas() is None:
        raise Exception("Error: Pandas required for tidy data format!")
    if not isinstance(tidy_data, bool):
        raise TypeError("tidy_data must be bool (False or True)")


def _ids(distance_type, comp_platform):
    if type(distance_type) is not accrqaDistance:
        raise TypeError("Distance must be an instance of accrqaDistance")
    if type(comp_platform) is not accrqaCompPlatform:
        raise TypeError("Computational platform must be an instance of accrqaCompPlatform")
    return distance_type.get_distance_id(), comp_platform.get_platform_id()


def RP(input_data, tau: int, emb: int, threshold: float, distance_type):
    """Recurrence plot (src/accrqa/accrqa.py:22-83): int8 array [nc, nc]."""
    if tau <= 0 or emb <= 0:
        raise TypeError("Delay and embedding must be greater than zero.")
    if type(input_data) is not np.ndarray:
        raise TypeError("Unknown array type of the input_data")
    nc = input_data.shape[0] - (emb - 1) * tau
    if input_data.shape[0] > 65536:
        print("WARNING: Requested recurrence plot will be large. Large amounts of system "
              "memory is needed and system may crash.")
    out = np.zeros((nc, nc), dtype=np.int8)
    if type(distance_type) is not accrqaDistance:
        raise TypeError("Distance must be an instance of accrqaDistance")
    mo, mi, err = accrqaMem(out), accrqaMem(input_data), accrqaError()
    f = _lib.handle().py_accrqa_RP
    f.argtypes = [accrqaMem.handle_type(), accrqaMem.handle_type(), ctypes.c_int,
                  ctypes.c_int, ctypes.c_double, ctypes.c_int, accrqaError.handle_type()]
    f(mo.handle(), mi.handle(), tau, emb, threshold, distance_type.get_distance_id(),
      err.handle())
    err.check()
    return out


def RR(input_data, tau_values, emb_values, threshold_values, distance_type,
       comp_platform: Optional[accrqaCompPlatform] = accrqaCompPlatform("nv_gpu"),
       tidy_data: Optional[bool] = True):
    """RR per (tau, emb, threshold) (src/accrqa/accrqa.py:85-187)."""
    _check_common(tidy_data)
    nT, nE, nThr = tau_values.shape[0], emb_values.shape[0], threshold_values.shape[0]
    if nT <= 0 or nE <= 0 or nThr <= 0:
        raise TypeError("Number of delays, embedding or thresholds must be greater than zero.")
    if type(input_data) is not np.ndarray:
        raise TypeError("Unknown array type of the input_data")
    out = np.zeros((nT, nE, nThr), dtype=input_data.dtype)
    dist, plt = _ids(distance_type, comp_platform)
    mems = [accrqaMem(a) for a in (out, input_data, tau_values, emb_values, threshold_values)]
    err = accrqaError()
    f = _lib.handle().py_accrqa_RR
    f.argtypes = [accrqaMem.handle_type()] * 5 + [ctypes.c_int, ctypes.c_int,
                                                  accrqaError.handle_type()]
    f(*[m.handle() for m in mems], dist, plt, err.handle())
    err.check()
    if not tidy_data:
        return out
    rows = [{"Delay": t, "Embedding": e, "Threshold": th, "RR": out[a, b, c]}
            for a, t in enumerate(tau_values) for b, e in enumerate(emb_values)
            for c, th in enumerate(threshold_values)]
    return _pandas().DataFrame(rows)


def _lines(name, cols, input_data, tau_values, emb_values, lmin_values, threshold_values,
           distance_type, calculate_ENTR, comp_platform, tidy_data):
    _check_common(tidy_data)
    if not isinstance(calculate_ENTR, bool):
        raise TypeError("calculate_ENTR must be bool (False or True)")
    nT, nE = tau_values.shape[0], emb_values.shape[0]
    nL, nThr = lmin_values.shape[0], threshold_values.shape[0]
    if nT <= 0 or nE <= 0 or nL <= 0 or nThr <= 0:
        raise TypeError("Number of delays, embedding, minimal lengths or thresholds must "
                        "be greater than zero.")
    if type(input_data) is not np.ndarray:
        raise TypeError("Unknown array type")
    out = np.zeros((nT, nE, nL, nThr, 5), dtype=input_data.dtype)
    if type(distance_type) is not accrqaDistance:
        raise TypeError("distance must be an instance of accrqaDistance")
    dist, plt = _ids(distance_type, comp_platform)
    mems = [accrqaMem(a) for a in (out, input_data, tau_values, emb_values, lmin_values,
                                   threshold_values)]
    err = accrqaError()
    f = getattr(_lib.handle(), name)
    f.argtypes = [accrqaMem.handle_type()] * 6 + [ctypes.c_int] * 3 + [
        accrqaError.handle_type()]
    f(*[m.handle() for m in mems], dist, 1 if calculate_ENTR else 0, plt, err.handle())
    err.check()
    if not tidy_data:
        return out
    rows = []
    for a, t in enumerate(tau_values):
        for b, e in enumerate(emb_values):
            for c, lm in enumerate(lmin_values):
                for k, th in enumerate(threshold_values):
                    r = {"Delay": t, "Embedding": e, cols[0]: lm, "Threshold": th}
                    for q, key in enumerate(cols[1:]):
                        r[key] = out[a, b, c, k, q]
                    rows.append(r)
    return _pandas().DataFrame(rows)


def DET(input_data, tau_values, emb_values, lmin_values, threshold_values, distance_type,
        calculate_ENTR: Optional[bool] = True,
        comp_platform: Optional[accrqaCompPlatform] = accrqaCompPlatform("nv_gpu"),
        tidy_data: Optional[bool] = True):
    """DET, L, Lmax, ENTR, RR (src/accrqa/accrqa.py:189-327)."""
    return _lines("py_accrqa_DET", ("Lmin", "DET", "L", "Lmax", "ENTR", "RR"), input_data,
                  tau_values, emb_values, lmin_values, threshold_values, distance_type,
                  calculate_ENTR, comp_platform, tidy_data)


def LAM(input_data, tau_values, emb_values, vmin_values, threshold_values, distance_type,
        calculate_ENTR: Optional[bool] = True,
        comp_platform: Optional[accrqaCompPlatform] = accrqaCompPlatform("nv_gpu"),
        tidy_data: Optional[bool] = True):
    """LAM, TT, TTmax, ENTR, RR (src/accrqa/accrqa.py:329-468)."""
    return _lines("py_accrqa_LAM", ("Vmin", "LAM", "TT", "TTmax", "ENTR", "RR"), input_data,
                  tau_values, emb_values, vmin_values, threshold_values, distance_type,
                  calculate_ENTR, comp_platform, tidy_data)


# Bisection steps RR_target evaluates per RR call (2^4 - 1 = 15 thresholds,
# one pass of the 16-threshold kernels).
_RR_TARGET_DEPTH = 4


def RR_target(input_data, tau: int, emb: int, target_RR: float, distance_type,
              epsilon: Optional[float] = 0.01,
              comp_platform: Optional[accrqaCompPlatform] = accrqaCompPlatform("nv_gpu"),
              max_iter: Optional[int] = 20, threshold_min: Optional[float] = 0,
              threshold_max: Optional[float] = 10):
    """Bisection for the threshold giving target_RR (src/accrqa/accrqa.py:470-594).

    Returns (threshold, RR).  The same bisection steps as the reference, on
    float32 thresholds, evaluated four steps per RR call (see below).
    """
    if type(distance_type) is not accrqaDistance:
        raise TypeError("distance must be an instance of accrqaDistance")
    if type(comp_platform) is not accrqaCompPlatform:
        raise TypeError("Computational platform must be an instance of accrqaCompPlatform")
    if type(input_data) is not np.ndarray:
        raise TypeError("Unknown array type")
    if tau <= 0 or emb <= 0:
        raise TypeError("Delay and embedding must be greater than zero.")
    if target_RR < 0.0 or target_RR > 1.0:
        raise TypeError("target_RR must be between 0 and 1.")
    if epsilon <= 0.0:
        raise TypeError("epsilon must be positive and non-zero.")
    if max_iter <= 0:
        raise TypeError("max_iter must be positive.")
    if threshold_min >= threshold_max:
        raise TypeError("threshold_min must be smaller then threshold_max.")
    taus = np.array([tau], dtype=np.intc)
    embs = np.array([emb], dtype=np.intc)

    def rr_of(thresholds):
        thr = np.asarray(thresholds, dtype=np.float32)
        return RR(input_data, taus, embs, thr.astype(input_data.dtype), distance_type,
                  comp_platform, tidy_data=False).flatten()

    mid = (threshold_max - threshold_min) / 2.0 + threshold_min
    vals = rr_of([threshold_min, mid, threshold_max])
    low_RR, hgh_RR = vals[0], vals[2]
    current_RR = vals[1]
    # The reference evaluates one midpoint per RR call.  Here the next `depth`
    # bisection steps are evaluated speculatively in one call: every midpoint
    # the search can reach from (threshold_min, threshold_max) within `depth`
    # steps (2^depth - 1 thresholds, one 16-slot pass for depth 4), computed
    # with the reference's float arithmetic; the walk down that tree then takes
    # exactly the reference's decisions, so the result is the same.
    iteration = 0
    while iteration < max_iter:
        depth = min(_RR_TARGET_DEPTH, max_iter - iteration)
        nodes = [(threshold_min, threshold_max)]   # breadth-first, heap order
        mids = []
        for k in range((1 << depth) - 1):
            lo, hi = nodes[k]
            m = (hi - lo) / 2.0 + lo
            mids.append(m)
            if 2 * k + 2 < (1 << depth) - 1:
                nodes.append((lo, m))   # child 2k+1: RR >= target, max = mid
                nodes.append((m, hi))   # child 2k+2: RR < target, min = mid
        rrs = rr_of(mids)
        k = 0
        for _ in range(depth):
            iteration += 1
            mid, current_RR = mids[k], rrs[k]
            if abs(current_RR - target_RR) < epsilon:
                return mid, current_RR
            if (hgh_RR - low_RR) < epsilon:
                return mid, current_RR
            if current_RR < target_RR:
                threshold_min = mid
                k = 2 * k + 2
            else:
                threshold_max = mid
                k = 2 * k + 1
    print(f"Warning: Bisection search stopped after {max_iter} iterations")
    mid = (threshold_max - threshold_min) / 2.0 + threshold_min
    return mid, current_RR
