"""GB300-native LEAP per-direction calibration hot path.

Everything computes through ``_lib/libleap_gb300.so`` (hand-written sm_103a
CUDA behind a C ABI, include/leap_gb300.h); importing the package fails if the
library has not been built.
"""
from ._abi import (LEAP_PRECISION_FP64, LEAP_PRECISION_MIXED, LEAP_VIS_C64, LEAP_VIS_C128,  # noqa: F401
                   LIB_PATH)
from .calibrator import (Context, GpuLeapCalibrator, InvalidArgument, LeapError, MetaData,  # noqa: F401
                         build_metadata, dd_matrix, evaluate_slice, phase_matrix, pseudo_inverse)
