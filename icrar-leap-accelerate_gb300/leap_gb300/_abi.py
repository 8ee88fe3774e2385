"""ctypes binding of the C ABI declared in include/leap_gb300.h.

The shared library is built in-tree by ``icrar-leap-accelerate_gb300/build.py``
into ``leap_gb300/_lib/``.  There is no fallback: if the library is missing or
fails to load, importing this module raises.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libleap_gb300.so")

LEAP_OK = 0
LEAP_ERR_INVALID_ARGUMENT = 1
LEAP_ERR_CUDA = 2
LEAP_ERR_NOT_READY = 3
LEAP_ERR_DEVICE_TIMEOUT = 4
LEAP_ERR_OUT_OF_MEMORY = 5
LEAP_ERR_INTERNAL = 6

LEAP_VIS_C64 = 0
LEAP_VIS_C128 = 1
LEAP_PRECISION_FP64 = 0
LEAP_PRECISION_MIXED = 1
LEAP_MEMORY_HOST = 0
LEAP_MEMORY_DEVICE = 1
LEAP_NOALLOC_SCRATCH_BYTES = 16 * 1024 * 1024
LEAP_OPTION_AUTOTUNE = 1
LEAP_OPTION_TENSOR_CORE_CONTRACTION = 2
LEAP_OPTION_TENSOR_CORE_ROTATION = 3
LEAP_OPTION_GRIDDED_ROTATION = 4
LEAP_OPTION_GRAPH_REPLAY = 5
LEAP_OPTION_GRID_SHARED_GROUPS = 6

# Every entry point include/leap_gb300.h declares, with its ctypes signature.
i32, i64, f64, vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p


class LeapConstants(ctypes.Structure):
    _fields_ = [("nbaselines", ctypes.c_uint32), ("referenceAntenna", ctypes.c_uint32),
                ("channels", ctypes.c_uint32), ("num_pols", ctypes.c_uint32),
                ("stations", ctypes.c_uint32), ("rows", ctypes.c_uint32),
                ("freq_start_hz", f64), ("freq_inc_hz", f64),
                ("phase_centre_ra_rad", f64), ("phase_centre_dec_rad", f64),
                ("dlm_ra", f64), ("dlm_dec", f64)]


class LeapTimings(ctypes.Structure):
    _fields_ = [("rotate_ms", ctypes.c_float), ("solve_ms", ctypes.c_float),
                ("total_ms", ctypes.c_float), ("kernels", ctypes.c_int32), ("calls", ctypes.c_int32)]


class LeapWorkItem(ctypes.Structure):
    _fields_ = [("slot", i32), ("first_direction", i32), ("ndirections", i32), ("reserved", i32)]


SIGNATURES = {
    "leap_create": ([i32, ctypes.POINTER(vp)], i32),
    "leap_destroy": ([vp], None),
    "leap_last_error": ([vp], ctypes.c_char_p),
    "leap_set_metadata": ([vp, ctypes.POINTER(LeapConstants), vp, i32, i32, vp, vp, vp, i32, vp, vp], i32),
    "leap_set_integration": ([vp, i32, i32, vp, vp, i64, i32, i32, i32], i32),
    "leap_build_metadata": ([vp, ctypes.POINTER(LeapConstants), vp, vp, vp, i32, ctypes.POINTER(i32)], i32),
    "leap_get_metadata_matrix": ([vp, i32, vp, i64, ctypes.POINTER(i32), ctypes.POINTER(i32)], i32),
    "leap_set_integration_ms": ([vp, i32, i32, vp, i64, i32, vp, i64, i32, i32, i32], i32),
    "leap_set_integration_ms_async": ([vp, i32, i32, vp, i64, i32, vp, i64, i32, i32, i32], i32),
    "leap_apply_flags": ([vp, i32, vp, i64, i32, i32, i32, ctypes.POINTER(i64)], i32),
    "leap_release_integration": ([vp, i32], i32),
    "leap_calibrate": ([vp, i32, vp, i32, i32, vp], i32),
    "leap_calibrate_async": ([vp, i32, vp, i32, i32, vp, vp], i32),
    "leap_calibrate_batched": ([vp, vp, i32, vp, i32, i32, vp], i32),
    "leap_set_autotune": ([vp, i32], i32),
    "leap_set_option": ([vp, i32, i32], i32),
    "leap_selftest_bounded_wait": ([vp, i32], i32),
    "leap_get_avgdata_device": ([vp, i32, vp, vp], i32),
    "leap_backward": ([vp, i32, vp, i32, vp, vp, vp, vp, vp, vp], i32),
    "leap_get_avgdata": ([vp, i32, vp], i32),
    "leap_rotate_uvw": ([vp, i32, vp, i32, vp], i32),
    "leap_get_timings": ([vp, ctypes.POINTER(LeapTimings)], i32),
    "leap_timing_reset": ([vp], i32),
    "leap_synchronize": ([vp], i32),
    "leap_rotate_average_noalloc": ([i32, vp, vp, i64, i32, i32, i32, f64, f64, vp, i32, vp, vp], i32),
    "leap_noalloc_last_error": ([], ctypes.c_char_p),
    "leap_dd_matrix": ([f64, f64, f64, f64, vp], None),
    "leap_phase_matrix": ([vp, vp, vp, i32, i32, vp, vp, ctypes.POINTER(i32), ctypes.POINTER(i32)], i32),
    "leap_pseudo_inverse": ([vp, i32, i32, vp], i32),
}


def load(path: str = LIB_PATH):
    if not os.path.exists(path):
        raise ImportError(f"LEAP GB300 library not built: {path} (run icrar-leap-accelerate_gb300/build.py)")
    lib = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


lib = load()
