"""accrqa_gb300 -- GB300-native recurrence quantification analysis (RQA).

A drop-in for the GPU path of the AccRQA library's ``accrqa_RR``,
``accrqa_DET``, ``accrqa_LAM`` and ``accrqa_RP``: the C/C++ library
``lib/libaccrqa.so`` (hand-written sm_103a kernels behind the reference's C
ABI) plus this Python front-end with the reference's interface.

    from accrqa_gb300 import RR, DET, LAM, RP, accrqaDistance
    from accrqa_gb300 import engine   # raw counts / histograms, device passes
"""
from ._lib import handle as library, lib_path  # noqa: F401
from .accrqa import (RP, RR, DET, LAM, RR_target, accrqaCompPlatform,  # noqa: F401
                     accrqaDistance, accrqaError, accrqaMem)
from . import engine  # noqa: F401

__all__ = ["RP", "RR", "DET", "LAM", "RR_target", "accrqaCompPlatform",
           "accrqaDistance", "accrqaError", "accrqaMem", "engine", "library", "lib_path"]
