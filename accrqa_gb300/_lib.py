"""Loader of libaccrqa.so (the GB300 RQA engine) for the Python front-end.

The library is looked up in ``ACCRQA_LIB_DIR`` (the variable the reference's
Python package uses) and then in ``accrqa_gb300/lib``.  A missing library is
an error: there is no Python or CPU fallback for the compute path.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_NAME = "libaccrqa.so"
_lock = threading.Lock()
_lib = None


def lib_dir() -> str:
    return os.path.join(_HERE, "lib")


def lib_path() -> str:
    env = os.environ.get("ACCRQA_LIB_DIR")
    if env and os.path.exists(os.path.join(env, LIB_NAME)):
        return os.path.join(env, LIB_NAME)
    return os.path.join(lib_dir(), LIB_NAME)


def handle() -> ctypes.CDLL:
    """The loaded library; raises RuntimeError when it has not been built."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                path = lib_path()
                if not os.path.exists(path):
                    raise RuntimeError(
                        f"{LIB_NAME} not found at {path}: build it with "
                        "`python -m accrqa_gb300.build`")
                lib = ctypes.CDLL(path)
                _declare(lib)
                _lib = lib
    return _lib


def _declare(lib: ctypes.CDLL) -> None:
    c_u64p = ctypes.POINTER(ctypes.c_uint64)
    vp = ctypes.c_void_p
    i32 = ctypes.c_int32
    i64 = ctypes.c_int64
    lib.accrqa_gb300_last_error.restype = ctypes.c_char_p
    lib.accrqa_gb300_version.restype = ctypes.c_int
    lib.accrqa_gb300_device_count.restype = ctypes.c_int
    lib.accrqa_gb300_kernel_launches.restype = ctypes.c_uint64
    lib.accrqa_gb300_transfer_stats.argtypes = [vp, vp, i32]
    lib.accrqa_gb300_transfer_stats.restype = None
    lib.accrqa_gb300_threshold_keys.argtypes = [c_u64p, vp, i32, i32, i32]
    for name in ("accrqa_gb300_rr_counts", "accrqa_gb300_det_histograms",
                 "accrqa_gb300_lam_histograms"):
        f = getattr(lib, name)
        f.argtypes = [c_u64p, vp, i32, i64, i32, i32, vp, i32, i32]
        f.restype = ctypes.c_int
    lib.accrqa_gb300_rp.argtypes = [vp, i32, vp, i32, i64, i32, i32,
                                    ctypes.c_double, i32]
    lib.accrqa_gb300_rp.restype = ctypes.c_int
    lib.accrqa_gb300_measures.argtypes = [ctypes.POINTER(ctypes.c_double), c_u64p,
                                          i64, i64, i32]
    lib.accrqa_gb300_measures.restype = ctypes.c_int
    lib.accrqa_gb300_rr_counts_dev.argtypes = [vp, vp, i32, i64, i32, i32, vp,
                                               i32, i32, vp]
    lib.accrqa_gb300_rr_counts_dev.restype = ctypes.c_int
    for name in ("accrqa_gb300_det_hist_dev", "accrqa_gb300_lam_hist_dev"):
        f = getattr(lib, name)
        f.argtypes = [vp, i64, vp, vp, i32, i64, i32, i32, vp, i32, i32, vp]
        f.restype = ctypes.c_int
    lib.accrqa_gb300_rp_bits.argtypes = [vp, vp, i32, i64, i32, i32, ctypes.c_double, i32]
    lib.accrqa_gb300_rp_bits.restype = ctypes.c_int
    lib.accrqa_gb300_rp_bits_dev.argtypes = [vp, vp, i32, i64, i32, i32, ctypes.c_double, i32, vp]
    lib.accrqa_gb300_rp_bits_dev.restype = ctypes.c_int
    lib.accrqa_gb300_probe_fp32.argtypes = [i32, i32, ctypes.POINTER(ctypes.c_double)]
    lib.accrqa_gb300_probe_fp32.restype = ctypes.c_int


def last_error() -> str:
    return handle().accrqa_gb300_last_error().decode(errors="replace")
