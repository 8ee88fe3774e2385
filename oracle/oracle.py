"""ORACLE — test infrastructure only.

Float64 restatement of LEAP-Accelerate's CPU calibration path, against which
the GPU product's results are compared.  Only the tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may import this module, and only to check
or to time the reference algorithm on the host; nothing shipped calls it.

The per-sample work runs in ``leap_oracle.c`` (built by ``oracle/Makefile``
into ``oracle/_build/``); this module adds the pieces the reference takes from
Eigen and the MeasurementSet layer:

* ``pseudo_inverse``  — ``SVDPseudoInverse`` (LA/math/cpu/matrix_invert.h:49-56):
  thin SVD, tolerance ``max(m, n) * eps * sigma_0``, ``V diag(1/sigma) U^H``.
  numpy's ``svd`` is LAPACK ``gesdd``, the same divide-and-conquer family as
  Eigen's BDCSVD; the pseudoinverse is unique, so both agree to rounding.
* ``metadata``        — ``cpu::MetaData`` construction (LA/model/cpu/MetaData.cc:42-137):
  reference antenna default ``total_antennas - 1`` (:51), filtered baselines =
  flagged(first epoch, ch0, pol0) OR short (LA/ms/MeasurementSet.cc:181-240),
  A1/I1 with the reference antenna (:92), A/I without (:97), pinvs (:111-124).
* ``calibrate``       — ``CpuLeapCalibrator::Calibrate`` (LA/algorithm/cpu/CpuLeapCalibrator.cc:61-145):
  solution loop over ``Slice.Evaluate(timesteps)`` with integration start row
  ``solution * interval * nbl`` (:113-119, which ignores ``Slice.start``).

(LA/ = src/icrar/leap-accelerate/ in the reference project.)
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libleap_oracle.so")
_lib = None
_lib_lock = threading.Lock()

SPEED_OF_LIGHT = 299792458.0  # LA/common/constants.h:35


def build() -> str:
    """Compile leap_oracle.c with the committed Makefile; returns the .so path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        src = os.path.join(_HERE, "leap_oracle.c")
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
            build()
        lib = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER
        i32, i64, f64, vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p
        lib.oracle_phase_matrix.argtypes = [vp, vp, vp, i32, i32, vp, vp, P(i32), P(i32)]
        lib.oracle_phase_matrix.restype = ctypes.c_int
        lib.oracle_dd_matrix.argtypes = [f64, f64, f64, f64, vp]
        lib.oracle_dd_matrix.restype = None
        lib.oracle_rotate_uvw.argtypes = [vp, vp, i64, vp]
        lib.oracle_rotate_uvw.restype = None
        lib.oracle_rotate_visibilities.argtypes = [vp, ctypes.c_int, vp, vp, i64, i32, i32, i32, f64, f64, vp]
        lib.oracle_rotate_visibilities.restype = None
        lib.oracle_solve.argtypes = [vp, i32, vp, i32, i32, vp, vp, vp, i32, vp]
        lib.oracle_solve.restype = None
        lib.oracle_calibrate_interval.argtypes = [vp, ctypes.c_int, vp, i64, i32, i32, i32, f64, f64,
                                                  vp, i32, vp, i32, i32, vp, vp, vp, i32, vp, vp, i32]
        lib.oracle_calibrate_interval.restype = ctypes.c_int
        lib.oracle_calibrate_items.argtypes = [i32, vp, ctypes.c_int, vp, vp, vp, i32, i32, f64, f64, vp, vp,
                                               vp, i32, i32, vp, vp, vp, i32, vp, vp, i32]
        lib.oracle_calibrate_items.restype = ctypes.c_int
        lib.oracle_max_threads.argtypes = []
        lib.oracle_max_threads.restype = ctypes.c_int
        _lib = lib
        return lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class InvalidArgument(ValueError):
    """Raised where the reference throws icrar::invalid_argument_exception."""


# ---------------------------------------------------------------------------
# Small restated pieces
# ---------------------------------------------------------------------------

def channel_wavelength(freq_start_hz: float, freq_inc_hz: float, i: int) -> float:
    """Constants::GetChannelWavelength (LA/model/cpu/MetaData.h:95-98)."""
    return SPEED_OF_LIGHT / (freq_start_hz + i * freq_inc_hz)


def dd_matrix(phase_ra: float, phase_dec: float, ra: float, dec: float) -> np.ndarray:
    """MetaData::GenerateDDMatrix (LA/model/cpu/MetaData.cc:166-203), 3x3 row-major."""
    out = np.zeros(9, dtype=np.float64)
    _load().oracle_dd_matrix(phase_ra, phase_dec, ra, dec, _ptr(out))
    return out.reshape(3, 3)


def phase_matrix(a1: Sequence[int], a2: Sequence[int], fg: Sequence[bool], ref_ant: Optional[int]):
    """PhaseMatrixFunction (LA/algorithm/cpu/PhaseMatrixFunction.cc:35-93).

    Returns (A, I) with A as a float64 (rows x cols) array and I as int32."""
    a1 = np.ascontiguousarray(a1, dtype=np.int32)
    a2 = np.ascontiguousarray(a2, dtype=np.int32)
    fg = np.ascontiguousarray(fg, dtype=np.uint8)
    n = a1.size
    if n == 0:
        # Eigen's maxCoeff on empty input is undefined; the reference reaches the
        # refAnt bounds check first when a reference antenna is given (:46-51).
        raise InvalidArgument("refAnt is out of bounds" if ref_ant is not None else "empty baselines")
    cols_max = int(max(a1.max(), a2.max())) + 1
    A_buf = np.zeros((n + 1) * cols_max, dtype=np.float64)
    I_buf = np.zeros(n, dtype=np.int32)
    rows = ctypes.c_int32(0)
    cols = ctypes.c_int32(0)
    rc = _load().oracle_phase_matrix(_ptr(a1), _ptr(a2), _ptr(fg), n, -1 if ref_ant is None else int(ref_ant),
                                     _ptr(A_buf), _ptr(I_buf), ctypes.byref(rows), ctypes.byref(cols))
    if rc != 0:
        raise InvalidArgument(f"refAnt {ref_ant} is out of bounds or flagged")
    r, c = rows.value, cols.value
    A = A_buf[: r * c].reshape(c, r).T.copy()  # column-major -> (rows, cols)
    return A, I_buf[: r - 1].copy()


def pseudo_inverse(a: np.ndarray, epsilon: float = np.finfo(np.float64).eps) -> np.ndarray:
    """SVDPseudoInverse (LA/math/cpu/matrix_invert.h:49-56).

    The pseudo-inverse is unique; an SVD computes it only to within the SVD's own
    rounding, which depends on the LAPACK build: for the 130,817 x 512 phase matrix of
    a 512-station array, numpy's gesdd is within 2e-13 of the exact pinv on x86-64
    (OpenBLAS) but 1.7e-11 on an aarch64 host, and such a difference moves the
    calibration phases by ~1e-10 rad.  So when A is an integer matrix of full column
    rank (every phase matrix whose stations all have an unflagged baseline) and the
    tolerance rule zeroes no singular value, the SVD result is refined to the exact
    pinv (A^T A)^-1 A^T to within rounding (``_refine_integer_pinv``); otherwise the
    SVD result is returned as the reference computes it."""
    a = np.asarray(a, dtype=np.float64)
    u, s, vt = np.linalg.svd(a, full_matrices=False)
    tol = float(max(a.shape[0], a.shape[1])) * epsilon * abs(s[0])
    keep = np.abs(s) > tol
    inv = np.where(keep, 1.0 / np.where(s == 0, 1.0, s), 0.0)
    m, n = a.shape
    if m >= n and n > 0 and keep.all() and np.array_equal(a, np.round(a)):
        g_inv = (vt.T * (inv * inv)) @ vt  # (A^T A)^-1 from the SVD: V S^-2 V^T
        refined = _refine_integer_pinv(a, g_inv)
        if refined is not None:
            return refined
    return (vt.T * inv) @ u.T


def _split_columns(x: np.ndarray, bits: int):
    """x = hi + lo with hi[:, k] a multiple of 2^(e_k - bits), 2^e_k >= max |x[:, k]| (exact)."""
    amax = np.abs(x).max(axis=0)
    e = np.where(amax > 0, np.ceil(np.log2(np.where(amax > 0, amax, 1.0))), 0.0).astype(np.int64) + 1
    hi = np.ldexp(np.round(np.ldexp(x, bits - e)), e - bits)
    return hi, x - hi


def _refine_integer_pinv(a: np.ndarray, g_inv: np.ndarray, steps: int = 2):
    """Iterative refinement of X = (A^T A)^-1 for an integer A, with residuals computed
    without rounding error: G = A^T A is exact in FP64, and G @ hi (hi: X cut to
    53 - b - 1 significant bits per column, 2^b > the largest row sum of |G|) has every
    partial sum on the grid of hi's last bit and below 2^53 of it, so it is exact.
    Returns X A^T, or None when G's entries are too large for the exact product."""
    g = a.T @ a
    row = float(np.abs(g).sum(axis=1).max())
    if row <= 0 or row >= 2.0 ** 40:
        return None
    b = int(np.ceil(np.log2(row))) + 1
    bits = 52 - b
    x = g_inv
    eye = np.eye(g.shape[0])
    for step in range(steps):
        hi, lo = _split_columns(x, bits)
        r = (eye - g @ hi) - g @ lo
        c = x @ r
        if step + 1 < steps:
            x = x + c
    # The last correction stays apart (X = x + c, a double-FP64 value): the columns of X
    # share a large common part that cancels in X A^T, so c is added after the product.
    return x @ a.T + c @ a.T


# ---------------------------------------------------------------------------
# MetaData
# ---------------------------------------------------------------------------

@dataclass
class OracleMetaData:
    nbaselines: int
    reference_antenna: int
    channels: int
    num_pols: int
    stations: int
    rows: int
    freq_start_hz: float
    freq_inc_hz: float
    phase_centre_ra_rad: float
    phase_centre_dec_rad: float
    A: np.ndarray
    I: np.ndarray
    Ad: np.ndarray
    A1: np.ndarray
    I1: np.ndarray
    Ad1: np.ndarray


def filtered_baselines(obs, minimum_baseline_threshold: float) -> np.ndarray:
    """MeasurementSet::GetFilteredBaselines (LA/ms/MeasurementSet.cc:181-240)."""
    nbl = obs.nbaselines
    flagged = np.asarray(obs.flags[:nbl], dtype=bool)
    short = np.zeros(nbl, dtype=bool)
    if minimum_baseline_threshold > 0.0:
        uv = obs.uvw[:nbl]
        short = np.sqrt(uv[:, 0] * uv[:, 0] + uv[:, 1] * uv[:, 1]) < minimum_baseline_threshold
    return flagged | short


def metadata(obs, reference_antenna: Optional[int] = None, minimum_baseline_threshold: float = 0.0) -> OracleMetaData:
    """cpu::MetaData constructor (LA/model/cpu/MetaData.cc:42-137)."""
    ref = reference_antenna if reference_antenna is not None else obs.total_antennas - 1
    fg = filtered_baselines(obs, minimum_baseline_threshold)
    a1 = obs.antenna1[: obs.nbaselines]
    a2 = obs.antenna2[: obs.nbaselines]
    A1, I1 = phase_matrix(a1, a2, fg, ref)
    A, I = phase_matrix(a1, a2, fg, None)
    return OracleMetaData(
        nbaselines=obs.nbaselines, reference_antenna=ref, channels=obs.channels, num_pols=obs.pols,
        stations=obs.num_stations, rows=obs.rows, freq_start_hz=obs.freq_start_hz,
        freq_inc_hz=obs.freq_inc_hz, phase_centre_ra_rad=obs.phase_centre[0],
        phase_centre_dec_rad=obs.phase_centre[1],
        A=A, I=I, Ad=pseudo_inverse(A), A1=A1, I1=I1, Ad1=pseudo_inverse(A1))


# ---------------------------------------------------------------------------
# Rotation / solve / calibrate
# ---------------------------------------------------------------------------

def _vis_args(vis: np.ndarray):
    if vis.dtype == np.complex64:
        return np.ascontiguousarray(vis), 1
    if vis.dtype == np.complex128:
        return np.ascontiguousarray(vis), 0
    raise TypeError("vis must be complex64 or complex128")


def rotate_visibilities(vis: np.ndarray, uvw: np.ndarray, dd: np.ndarray, nbl: int,
                        freq_start_hz: float, freq_inc_hz: float) -> np.ndarray:
    """RotateVisibilities for one direction; vis is (channels, rows, pols) C-order
    (the reference Integration tensor).  Returns avgData as (nbl, pols) complex128."""
    vis, f32 = _vis_args(vis)
    C, rows, P = vis.shape
    uvw = np.ascontiguousarray(uvw, dtype=np.float64)
    dd = np.ascontiguousarray(dd, dtype=np.float64).reshape(9)
    avg = np.zeros(2 * nbl * P, dtype=np.float64)
    _load().oracle_rotate_visibilities(_ptr(vis), f32, _ptr(uvw), _ptr(dd), rows, C, P, nbl,
                                       freq_start_hz, freq_inc_hz, _ptr(avg))
    return avg.view(np.complex128).reshape(P, nbl).T.copy()


def solve(avg: np.ndarray, md: OracleMetaData) -> np.ndarray:
    """The PhaseRotate solve (CpuLeapCalibrator.cc:159-178) for one direction."""
    nbl, P = avg.shape
    avg_cm = np.ascontiguousarray(avg.T).view(np.float64)  # column-major (nbl x P), interleaved
    A = np.asfortranarray(md.A)
    Ad = np.asfortranarray(md.Ad)
    Ad1 = np.asfortranarray(md.Ad1)
    I1 = np.ascontiguousarray(md.I1, dtype=np.int32)
    S = A.shape[1]
    cal = np.zeros(S, dtype=np.float64)
    _load().oracle_solve(_ptr(avg_cm), nbl, _ptr(A), A.shape[0], S, _ptr(Ad), _ptr(I1), _ptr(Ad1),
                         md.A1.shape[0], _ptr(cal))
    return cal


def calibrate_interval(vis: np.ndarray, uvw: np.ndarray, dds: np.ndarray, md: OracleMetaData,
                       nthreads: int = 0, return_avg: bool = False):
    """All directions of one solution interval.  dds is (D, 3, 3).  Returns cal (D, S)
    and optionally avgData (D, nbl, P)."""
    vis, f32 = _vis_args(vis)
    C, rows, P = vis.shape
    uvw = np.ascontiguousarray(uvw, dtype=np.float64)
    dds = np.ascontiguousarray(dds, dtype=np.float64).reshape(-1, 9)
    D = dds.shape[0]
    A = np.asfortranarray(md.A)
    Ad = np.asfortranarray(md.Ad)
    Ad1 = np.asfortranarray(md.Ad1)
    I1 = np.ascontiguousarray(md.I1, dtype=np.int32)
    S = A.shape[1]
    cal = np.zeros((D, S), dtype=np.float64)
    avg = np.zeros(D * 2 * md.nbaselines * P, dtype=np.float64) if return_avg else None
    rc = _load().oracle_calibrate_interval(
        _ptr(vis), f32, _ptr(uvw), rows, C, P, md.nbaselines, md.freq_start_hz, md.freq_inc_hz,
        _ptr(dds), D, _ptr(A), A.shape[0], S, _ptr(Ad), _ptr(I1), _ptr(Ad1), md.A1.shape[0],
        _ptr(cal), _ptr(avg) if avg is not None else None, int(nthreads))
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    if return_avg:
        avg_c = avg.view(np.complex128).reshape(D, P, md.nbaselines).transpose(0, 2, 1).copy()
        return cal, avg_c
    return cal


def calibrate_items(chunks, md: OracleMetaData, nthreads: int = 0, return_avg: bool = False):
    """Several integration chunks of one array, each with its own directions: `chunks` is a
    list of (vis (channels, rows, pols), uvw (rows, 3), dds (D, 3, 3)).  One (chunk, direction)
    pair per host task.  Returns a list of cal (D, S) (and of avgData (D, nbl, P))."""
    n = len(chunks)
    vis_l, uvw_l, dd_l, cal_l, avg_l = [], [], [], [], []
    f32 = None
    P = None
    for vis, uvw, dds in chunks:
        v, f = _vis_args(vis)
        if f32 is None:
            f32, P = f, v.shape[2]
        if f != f32 or v.shape[2] != P:
            raise TypeError("chunks must share one visibility dtype and pol count")
        vis_l.append(v)
        uvw_l.append(np.ascontiguousarray(uvw, dtype=np.float64))
        dd_l.append(np.ascontiguousarray(dds, dtype=np.float64).reshape(-1, 9))
    A = np.asfortranarray(md.A)
    Ad = np.asfortranarray(md.Ad)
    Ad1 = np.asfortranarray(md.Ad1)
    I1 = np.ascontiguousarray(md.I1, dtype=np.int32)
    S = A.shape[1]
    for d in dd_l:
        cal_l.append(np.zeros((d.shape[0], S), dtype=np.float64))
        avg_l.append(np.zeros(d.shape[0] * 2 * md.nbaselines * P, dtype=np.float64) if return_avg else None)
    ptrs = lambda arrs: (ctypes.c_void_p * n)(*[a.ctypes.data if a is not None else None for a in arrs])
    rows = np.array([v.shape[1] for v in vis_l], dtype=np.int64)
    chans = np.array([v.shape[0] for v in vis_l], dtype=np.int32)
    ndir = np.array([d.shape[0] for d in dd_l], dtype=np.int32)
    rc = _load().oracle_calibrate_items(
        n, ptrs(vis_l), f32, ptrs(uvw_l), _ptr(rows), _ptr(chans), P, md.nbaselines, md.freq_start_hz,
        md.freq_inc_hz, ptrs(dd_l), _ptr(ndir), _ptr(A), A.shape[0], S, _ptr(Ad), _ptr(I1), _ptr(Ad1),
        md.A1.shape[0], ptrs(cal_l), ptrs(avg_l) if return_avg else None, int(nthreads))
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    if return_avg:
        avgs = [a.view(np.complex128).reshape(-1, P, md.nbaselines).transpose(0, 2, 1).copy() for a in avg_l]
        return cal_l, avgs
    return cal_l


def evaluate_slice(start: int, interval: int, end: int, collection_size: int):
    """Slice::Evaluate + Range::GetSize (LA/common/Slice.h:47-54, LA/common/Range.h:40-63)."""
    s = collection_size if start == -1 else start
    i = collection_size if interval == -1 else interval
    e = collection_size if end == -1 else end
    if s < 0 or i < 1 or e < 0:
        raise InvalidArgument("expected a positive integer")
    return s, i, e, (e - s) // i


def calibrate(obs, directions: np.ndarray, solution_interval=(0, -1, -1),
              minimum_baseline_threshold: float = 0.0, reference_antenna: Optional[int] = None,
              nthreads: int = 0, md: Optional[OracleMetaData] = None) -> List[dict]:
    """CpuLeapCalibrator::Calibrate (LA/algorithm/cpu/CpuLeapCalibrator.cc:61-145).

    ``solution_interval`` is an evaluated-at-call (start, interval, end) triple with
    the reference's -1 wildcards.  Returns the CalibrationCollection as a list of
    {"epoch": {"start", "end"}, "calibration": [{"direction", "beamCalibration"}]}."""
    if md is None:
        md = metadata(obs, reference_antenna, minimum_baseline_threshold)
    _, interval, _, solutions = evaluate_slice(*solution_interval, obs.timesteps)
    epochs = obs.epochs
    nbl = obs.nbaselines
    dds = np.stack([dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, float(r), float(d))
                    for r, d in np.asarray(directions, dtype=np.float64).reshape(-1, 2)])
    out = []
    for s in range(solutions):
        r0 = s * interval * nbl
        nrows = interval * nbl
        vis = obs.vis[:, r0:r0 + nrows, :]
        uvw = obs.uvw[r0:r0 + nrows]
        cal = calibrate_interval(vis, uvw, dds, md, nthreads=nthreads)
        out.append({
            "epoch": {"start": float(epochs[s * interval]), "end": float(epochs[(s + 1) * interval - 1])},
            "calibration": [{"direction": [float(x) for x in directions[i]], "beamCalibration": cal[i].tolist()}
                            for i in range(len(directions))],
        })
    return out


def max_threads() -> int:
    return int(_load().oracle_max_threads())
