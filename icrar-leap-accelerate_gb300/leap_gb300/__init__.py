"""GB300-native LEAP per-direction calibration hot path.

Everything computes through ``_lib/libleap_gb300.so`` (hand-written sm_103a
CUDA behind a C ABI, include/leap_gb300.h).  The library is loaded the first
time one of the names below is used (and that use fails if it has not been
built), so that ``leap_gb300.synth`` and ``leap_gb300.sharding``, which need
no device code, can be imported without mapping it.
"""
from importlib import import_module

_ABI_NAMES = ("LEAP_PRECISION_FP64", "LEAP_PRECISION_MIXED", "LEAP_VIS_C64", "LEAP_VIS_C128", "LIB_PATH")
_CALIBRATOR_NAMES = ("Context", "GpuLeapCalibrator", "InvalidArgument", "LeapError", "MetaData", "build_metadata",
                     "dd_matrix", "evaluate_slice", "phase_matrix", "pseudo_inverse")
__all__ = list(_ABI_NAMES + _CALIBRATOR_NAMES)


def __getattr__(name):
    if name in _ABI_NAMES:
        return getattr(import_module("._abi", __name__), name)
    if name in _CALIBRATOR_NAMES:
        return getattr(import_module(".calibrator", __name__), name)
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
