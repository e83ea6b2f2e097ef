"""The AccRQA reference's own Python package, unchanged, bound to this library.

The reference's loader (src/accrqa/accrqa_lib.py:16-57) searches
ACCRQA_LIB_DIR for `libaccrqa*`; pointed at accrqa_gb300/lib it must bind
this library's py_accrqa_RR / _DET / _LAM / _RP symbols with the argument
lists its ctypes stubs declare (src/accrqa/accrqa.py:151-171 and the DET, LAM
and RP equivalents), and its documented checks must behave as with its own
library:
  * its TypeErrors (tidy_data, zero-length parameter arrays) come before any
    library call;
  * comp_platform "cpu" makes this library return ERR_INVALID_ARGUMENT, which
    the reference's accrqaError.check() raises as a RuntimeError;
  * without a CUDA device this library returns ERR_CUDA_DEVICE_NOT_FOUND (8),
    a code past the reference's error table (0-6): its check() raises a
    KeyError -- the documented difference.
pandas is absent here; the package needs the name at import (its type
hints), so a stub module stands in for it.  The reference tree is named by
ACCRQA_REFERENCE_TREE or the build recipe's default; where neither exists
(e.g. on a GPU machine) the test skips.
"""
import importlib
import os
import sys
import types

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_src():
    tree = os.environ.get("ACCRQA_REFERENCE_TREE")
    if not tree:
        import __graft_entry__
        tree = __graft_entry__._REFERENCE_TREE
    src = os.path.join(tree, "src")
    return src if os.path.isfile(os.path.join(src, "accrqa", "accrqa_lib.py")) else None


@pytest.fixture(scope="module")
def ref_pkg(lib):
    src = _reference_src()
    if src is None:
        pytest.skip("the reference's source tree is not present")
    saved = {k: sys.modules.get(k) for k in list(sys.modules) if k == "accrqa"
             or k.startswith("accrqa.") or k == "pandas"}
    if "pandas" not in sys.modules:
        try:
            import pandas  # noqa: F401
        except ImportError:
            stub = types.ModuleType("pandas")

            class DataFrame(list):
                pass

            stub.DataFrame = DataFrame
            sys.modules["pandas"] = stub
    old_env = os.environ.get("ACCRQA_LIB_DIR")
    os.environ["ACCRQA_LIB_DIR"] = os.path.join(ROOT, "accrqa_gb300", "lib")
    sys.path.insert(0, src)
    for k in [k for k in sys.modules if k == "accrqa" or k.startswith("accrqa.")]:
        del sys.modules[k]
    try:
        pkg = importlib.import_module("accrqa")
        yield pkg
    finally:
        sys.path.remove(src)
        for k in [k for k in sys.modules if k == "accrqa" or k.startswith("accrqa.")]:
            del sys.modules[k]
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
        if old_env is None:
            os.environ.pop("ACCRQA_LIB_DIR", None)
        else:
            os.environ["ACCRQA_LIB_DIR"] = old_env


def test_loader_binds_this_library(ref_pkg):
    handle = ref_pkg.accrqaLib.handle()
    assert os.path.realpath(handle._name) == os.path.realpath(
        os.path.join(ROOT, "accrqa_gb300", "lib", "libaccrqa.so"))
    for sym in ("py_accrqa_RR", "py_accrqa_DET", "py_accrqa_LAM", "py_accrqa_RP"):
        assert getattr(handle, sym) is not None


def _args(dt=np.float32):
    x = np.sin(np.arange(400) * 0.1).astype(dt)
    return (x, np.array([1], np.intc), np.array([2], np.intc), np.array([2], np.intc),
            np.array([0.1, 0.3], dt))


def test_type_errors_before_any_call(ref_pkg):
    x, taus, embs, lmins, thr = _args()
    D = ref_pkg.accrqaDistance("euclidean")
    with pytest.raises(TypeError):
        ref_pkg.RR(x, taus, embs, thr, D, tidy_data="no")
    with pytest.raises(TypeError):
        ref_pkg.DET(x, taus, embs, lmins, thr[:0], D, tidy_data=False)
    with pytest.raises(TypeError):
        ref_pkg.LAM(x, taus[:0], embs, lmins, thr, D, tidy_data=False)


def test_cpu_platform_is_an_invalid_argument(ref_pkg):
    x, taus, embs, lmins, thr = _args()
    D = ref_pkg.accrqaDistance("maximal")
    cpu = ref_pkg.accrqaCompPlatform("cpu")
    for call in (lambda: ref_pkg.RR(x, taus, embs, thr, D, comp_platform=cpu, tidy_data=False),
                 lambda: ref_pkg.DET(x, taus, embs, lmins, thr, D, comp_platform=cpu,
                                     tidy_data=False),
                 lambda: ref_pkg.LAM(x, taus, embs, lmins, thr, D, comp_platform=cpu,
                                     tidy_data=False)):
        with pytest.raises(RuntimeError, match="Invalid function argument"):
            call()


def test_missing_device_surfaces_past_the_reference_table(ref_pkg):
    from accrqa_gb300 import engine
    if engine.device_count() > 0:
        pytest.skip("a CUDA device is present")
    x, taus, embs, lmins, thr = _args(np.float64)
    D = ref_pkg.accrqaDistance("euclidean")
    with pytest.raises(KeyError) as ei:
        ref_pkg.RR(x, taus, embs, thr, D, tidy_data=False)
    assert ei.value.args[0] == 8   # ERR_CUDA_DEVICE_NOT_FOUND
