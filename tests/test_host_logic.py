"""Host-side logic of libaccrqa.so that needs no GPU.

  * the library loads and exports every function include/*.h declares;
  * threshold keys reproduce the reference's test (t - f(v)) >= 0 exactly;
  * histogram post-processing equals the oracle's restatement;
  * the Mem handle and the py_accrqa_* validation paths (errors raised before
    any device work) behave like the reference's;
  * the Python front-end raises the reference's TypeErrors.
"""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_c_functions():
    src = open(os.path.join(ROOT, "include", "accrqa_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", src)
    return sorted(set(n for n in names if n not in ("if", "sizeof")))


def test_exports_every_declared_symbol(lib):
    from accrqa_gb300 import lib_path
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path()], capture_output=True,
                         text=True, check=True).stdout
    exported = set(ln.split()[-1] for ln in out.splitlines() if ln.strip())
    decl = _declared_c_functions()
    assert len(decl) >= 55
    missing = [n for n in decl if n not in exported]
    assert not missing, missing
    # C++ overloads of include/accrqa_gb300.hpp (demangled)
    dem = subprocess.run(["nm", "-DC", "--defined-only", lib_path()], capture_output=True,
                         text=True, check=True).stdout
    for sig in ("accrqa_RR(float*, float*, unsigned long, int*, int, int*, int, float*, int",
                "accrqa_RR(double*, double*, unsigned long",
                "accrqa_DET(float*, float*", "accrqa_DET(double*, double*",
                "accrqa_LAM(float*, float*", "accrqa_LAM(double*, double*",
                "accrqa_RP(char*, float*", "accrqa_RP(char*, double*", "accrqa_RP(int*, double*",
                "accrqa_print_error(Accrqa_Error*)",
                "accrqa_RR_output_size_in_elements(int, int, int)",
                "accrqa_DET_output_size_in_elements(int, int, int, int)",
                "accrqa_LAM_output_size_in_elements(int, int, int, int)",
                "accrqa_RP_output_size_in_elements(long, long, long)"):
        assert sig in dem, sig


def _pred32(t, v, norm):
    t, v = np.float32(t), np.float32(v)
    d = np.sqrt(v) if norm == 1 else v
    with np.errstate(invalid="ignore", over="ignore"):
        return bool(np.float32(t - d) >= 0)


def _pred64(t, v, norm):
    d = np.sqrt(np.float64(v)) if norm == 1 else np.float64(v)
    with np.errstate(invalid="ignore", over="ignore"):
        return bool(np.float64(t) - d >= 0)


def test_threshold_keys_are_exact(lib):
    from accrqa_gb300 import engine
    rng = np.random.default_rng(3)
    thr = np.concatenate([rng.uniform(0, 3, 200), [0.0, -0.0, 1e-30, 5e-45, 1e30, 3.4e38],
                          rng.uniform(-1, 0, 5)]).astype(np.float32)
    for norm in (1, 2):
        keys = engine.threshold_keys(thr, np.float32, norm)
        for t, k in zip(thr, keys):
            kv = np.uint32(k).view(np.float32)
            if kv < 0:                                   # never recurrent
                assert not _pred32(t, np.float32(0.0), norm)
                continue
            assert _pred32(t, kv, norm)
            nxt = np.nextafter(kv, np.float32(np.inf))
            if np.isfinite(nxt):
                assert not _pred32(t, nxt, norm)
    thr64 = np.concatenate([rng.uniform(0, 3, 100), [0.0, 1e-300, 1e300]])
    for norm in (1, 2):
        keys = engine.threshold_keys(thr64, np.float64, norm)
        for t, k in zip(thr64, keys):
            assert k > 0
            kv = np.uint64(k - 1).view(np.float64)
            assert _pred64(t, kv, norm)
            nxt = np.nextafter(kv, np.inf)
            if np.isfinite(nxt):
                assert not _pred64(t, nxt, norm)
    # special thresholds
    k = engine.threshold_keys(np.array([np.nan, np.inf, -1.0]), np.float64, 1)
    assert k[0] == 0 and k[2] == 0 and k[1] == np.uint64(np.finfo(np.float64).max.view(np.uint64)) + 1


def test_measures_match_oracle(lib, oracle_mod):
    from accrqa_gb300 import engine
    arr = np.load(os.path.join(ROOT, "tests", "golden", "ref_histograms.npz"))
    for key in [k for k in arr.files if k.endswith("_det") or k.endswith("_lam")]:
        for h in arr[key]:
            for lm in (0, 1, 2, 3, 7, len(h) - 1, len(h), len(h) + 5):
                got = engine.measures(h, lm, key.endswith("_det"))
                want = oracle_mod.measures(h, lm, key.endswith("_det"))
                np.testing.assert_array_equal(got, want, err_msg=f"{key} lmin={lm}")


def test_mem_handle(lib):
    L = lib
    L.mem_create_wrapper.restype = ctypes.c_void_p
    L.mem_create_wrapper.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int32,
                                     ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                     ctypes.POINTER(ctypes.c_int)]
    L.mem_create.restype = ctypes.c_void_p
    L.mem_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int32,
                             ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                             ctypes.POINTER(ctypes.c_int)]
    for f in ("mem_shape_dim", "mem_stride_dim"):
        getattr(L, f).restype = ctypes.c_int64
        getattr(L, f).argtypes = [ctypes.c_void_p, ctypes.c_int32]
    for f in ("mem_num_elements", "mem_type_size"):
        getattr(L, f).restype = ctypes.c_int64
    L.mem_num_elements.argtypes = [ctypes.c_void_p]
    for f in ("mem_num_dims", "mem_is_c_contiguous", "mem_is_read_only", "mem_type",
              "mem_location", "mem_is_complex"):
        getattr(L, f).argtypes = [ctypes.c_void_p]
    L.mem_free.argtypes = [ctypes.c_void_p]
    L.mem_data.restype = ctypes.c_void_p
    L.mem_data.argtypes = [ctypes.c_void_p]
    L.mem_set_read_only.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    L.mem_ref_inc.restype = ctypes.c_void_p
    L.mem_ref_inc.argtypes = [ctypes.c_void_p]
    L.mem_assert_type.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]

    a = np.zeros((3, 4), dtype=np.float32)
    err = ctypes.c_int(0)
    sh = (ctypes.c_int64 * 2)(*a.shape)
    st = (ctypes.c_int64 * 2)(*a.strides)
    m = L.mem_create_wrapper(a.ctypes.data, 4, 0, 2, sh, st, ctypes.byref(err))
    assert err.value == 0
    assert L.mem_num_dims(m) == 2 and L.mem_shape_dim(m, 1) == 4 and L.mem_stride_dim(m, 0) == 16
    assert L.mem_num_elements(m) == 12 and L.mem_is_c_contiguous(m) == 1
    assert L.mem_type(m) == 4 and L.mem_location(m) == 0 and L.mem_data(m) == a.ctypes.data
    assert L.mem_shape_dim(m, 5) == 0 and L.mem_is_complex(m) == 0
    L.mem_set_read_only(m, 1)
    assert L.mem_is_read_only(m) == 1
    t = a.T
    st2 = (ctypes.c_int64 * 2)(*t.strides)
    sh2 = (ctypes.c_int64 * 2)(*t.shape)
    m2 = L.mem_create_wrapper(t.ctypes.data, 4, 0, 2, sh2, st2, ctypes.byref(err))
    assert L.mem_is_c_contiguous(m2) == 0
    b = np.zeros(3, dtype=np.float64)
    m3 = L.mem_create_wrapper(b.ctypes.data, 8, 0, 1, (ctypes.c_int64 * 1)(3), None,
                              ctypes.byref(err))
    e2 = ctypes.c_int(0)
    assert L.mem_assert_type(m, m3, ctypes.byref(e2)) == 1 and e2.value == 3
    assert L.mem_ref_inc(m) == m
    L.mem_free(m)            # drops the extra reference
    assert L.mem_num_dims(m) == 2
    L.mem_free(m)
    L.mem_free(m2)
    L.mem_free(m3)
    owned = L.mem_create(2, 0, 1, (ctypes.c_int64 * 1)(10), None, ctypes.byref(err))
    assert err.value == 0 and L.mem_data(owned)
    L.mem_free(owned)
    bad = L.mem_create_wrapper(a.ctypes.data, 77, 0, 1, sh, None, ctypes.byref(err))
    assert err.value == 3
    L.mem_free(bad)


def _ids():
    import accrqa_gb300 as A
    return A.accrqaDistance("euclidean"), A.accrqaCompPlatform("nv_gpu")


def test_python_frontend_type_errors(lib):
    import accrqa_gb300 as A
    D, P = _ids()
    x = np.random.rand(100).astype(np.float32)
    i1 = np.array([1], np.intc)
    thr = np.array([0.1], np.float32)
    with pytest.raises(TypeError):
        A.RR(x, np.array([], np.intc), i1, thr, D, tidy_data=False)
    with pytest.raises(TypeError):
        A.RR([1.0, 2.0], i1, i1, thr, D, tidy_data=False)
    with pytest.raises(TypeError):
        A.RR(x, i1, i1, thr, "euclidean", tidy_data=False)
    with pytest.raises(TypeError):
        A.DET(x, i1, i1, i1, thr, D, calculate_ENTR="yes", tidy_data=False)
    with pytest.raises(TypeError):
        A.LAM(x, i1, i1, i1, thr, D, comp_platform="gpu", tidy_data=False)
    with pytest.raises(TypeError):
        A.RP(x, 0, 1, 0.1, D)
    with pytest.raises(ValueError):
        A.accrqaDistance("manhattan")
    with pytest.raises(ValueError):
        A.accrqaCompPlatform("tpu")
    with pytest.raises(TypeError):
        A.RR_target(x, 1, 1, 1.5, D)


def test_bindings_validate_before_device_work(lib):
    """Errors the shims raise before any GPU call (identical on CPU-only hosts)."""
    import accrqa_gb300 as A
    D, P = _ids()
    x = np.random.rand(100).astype(np.float32)
    i1 = np.array([1], np.intc)
    # mixed dtypes: ERR_DATA_TYPE
    with pytest.raises(RuntimeError, match="Unsupported data type"):
        A.RR(x, i1, i1, np.array([0.1], np.float64), D, tidy_data=False)
    # non-int tau array: ERR_DATA_TYPE
    with pytest.raises(RuntimeError, match="Unsupported data type"):
        A.DET(x, np.array([1], np.int8), i1, i1, np.array([0.1], np.float32), D,
              tidy_data=False)
    # the CPU platform is not served by this library: ERR_INVALID_ARGUMENT
    with pytest.raises(RuntimeError, match="Invalid function argument"):
        A.RR(x, i1, i1, np.array([0.1], np.float32), D, A.accrqaCompPlatform("cpu"),
             tidy_data=False)
    # invalid distance id straight through the C symbol
    err = A.accrqaError()
    mems = [A.accrqaMem(a) for a in (np.zeros((1, 1, 1), np.float32), x, i1, i1,
                                      np.array([0.1], np.float32))]
    f = A._lib.handle().py_accrqa_RR
    f.argtypes = [A.accrqaMem.handle_type()] * 5 + [ctypes.c_int, ctypes.c_int,
                                                    A.accrqaError.handle_type()]
    f(*[m.handle() for m in mems], 7, 1024, err.handle())
    assert err._error.value == 2
    err2 = A.accrqaError()
    f(*[m.handle() for m in mems], 1, 5, err2.handle())
    assert err2._error.value == 2


def test_output_sizes(lib):
    L = lib
    assert L._FuncPtr(("_Z33accrqa_RR_output_size_in_elementsiii", L))(2, 3, 4) == 24
    assert L._FuncPtr(("_Z34accrqa_DET_output_size_in_elementsiiii", L))(2, 3, 4, 5) == 600
    f = L._FuncPtr(("_Z33accrqa_RP_output_size_in_elementslll", L))
    f.restype = ctypes.c_int64
    f.argtypes = [ctypes.c_int64] * 3
    assert f(100, 2, 3) == 96


def _fake_rr(calls):
    """A monotone stand-in for the RR call (float32 thresholds in, rates out)."""
    def rr(x, taus, embs, thr, D, comp_platform=None, tidy_data=True):
        calls.append(len(thr))
        t = np.asarray(thr, np.float64)
        return np.clip(np.sqrt(t) / 2.5, 0.0, 1.0).reshape(1, 1, -1)
    return rr


@pytest.mark.parametrize("target,eps,max_iter,tmin,tmax", [
    (0.3, 0.01, 20, 0.0, 10.0), (0.3, 1e-9, 20, 0.0, 10.0), (0.71, 1e-7, 7, 0.0, 5.0),
    (0.05, 1e-12, 30, 0.0, 10.0), (0.5, 1e-3, 3, 0.1, 4.0), (0.9, 0.5, 5, 0.0, 1.0)])
def test_rr_target_tree_walk_equals_bisection(monkeypatch, target, eps, max_iter, tmin, tmax):
    import accrqa_gb300 as A
    from accrqa_gb300 import accrqa as mod
    calls = []
    monkeypatch.setattr(mod, "RR", _fake_rr(calls))
    x = np.zeros(100, np.float32)
    D = A.accrqaDistance("euclidean")
    got = A.RR_target(x, 1, 2, target, D, epsilon=eps, max_iter=max_iter,
                      threshold_min=tmin, threshold_max=tmax)
    # the reference's loop, one midpoint per call
    rr = _fake_rr([])
    lo, hi = tmin, tmax
    mid = (hi - lo) / 2.0 + lo
    v = rr(x, 0, 0, np.array([lo, mid, hi], np.float32), D).flatten()
    low, hgh, cur = v[0], v[2], v[1]
    want = None
    for _ in range(1, max_iter + 1):
        mid = (hi - lo) / 2.0 + lo
        cur = rr(x, 0, 0, np.array([mid], np.float32), D).flatten()[0]
        if abs(cur - target) < eps or (hgh - low) < eps:
            want = (mid, cur)
            break
        if cur < target:
            lo = mid
        else:
            hi = mid
    if want is None:
        want = ((hi - lo) / 2.0 + lo, cur)
    assert got[0] == want[0] and got[1] == want[1]
    assert len(calls) <= 1 + -(-max_iter // 4)   # the first call, then one per 4 steps
