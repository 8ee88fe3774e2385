"""Python mirror of the reference calibration interface over the C ABI.

``GpuLeapCalibrator.calibrate`` has the argument meaning and error behaviour of
``ILeapCalibrator::Calibrate`` (LA/algorithm/ILeapCalibrator.h:62-68) and the
loop structure of ``CudaLeapCalibrator::Calibrate``
(LA/algorithm/cuda/CudaLeapCalibrator.cu:94-233): MetaData once, then per
solution interval one resident integration and one batched call over all
directions.  ``Context`` exposes the C ABI one entry point per method.

(LA/ = src/icrar/leap-accelerate/ in the reference project.)
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _abi
from ._abi import lib

SPEED_OF_LIGHT = 299792458.0


class LeapError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class InvalidArgument(LeapError, ValueError):
    """Where the reference throws icrar::invalid_argument_exception."""


def _raise(code: int, msg: str):
    if code == _abi.LEAP_ERR_INVALID_ARGUMENT:
        raise InvalidArgument(code, msg)
    raise LeapError(code, msg)


def _check(code: int, ctx=None):
    if code != _abi.LEAP_OK:
        msg = lib.leap_last_error(ctx)
        _raise(code, msg.decode() if msg else "")


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


# ---------------------------------------------------------------------------
# Host set-up maths (the library's own C++ code)
# ---------------------------------------------------------------------------

def dd_matrix(phase_ra: float, phase_dec: float, ra: float, dec: float) -> np.ndarray:
    """MetaData::GenerateDDMatrix (LA/model/cpu/MetaData.cc:166-203)."""
    out = np.zeros(9, dtype=np.float64)
    lib.leap_dd_matrix(phase_ra, phase_dec, ra, dec, _ptr(out))
    return out.reshape(3, 3)


def phase_matrix(a1, a2, fg, ref_ant: Optional[int]) -> Tuple[np.ndarray, np.ndarray]:
    """PhaseMatrixFunction (LA/algorithm/cpu/PhaseMatrixFunction.cc:35-93): (A, I)."""
    a1 = np.ascontiguousarray(a1, dtype=np.int32)
    a2 = np.ascontiguousarray(a2, dtype=np.int32)
    fg = np.ascontiguousarray(fg, dtype=np.uint8)
    n = a1.size
    if a2.size != n or fg.size != n:
        raise InvalidArgument(_abi.LEAP_ERR_INVALID_ARGUMENT, "a1, a2 and fg must be equal size")
    cols_cap = int(max(a1.max(), a2.max())) + 1 if n else 1
    A = np.zeros((n + 1) * cols_cap, dtype=np.float64)
    I = np.zeros(max(n, 1), dtype=np.int32)
    rows, cols = ctypes.c_int32(0), ctypes.c_int32(0)
    _check(lib.leap_phase_matrix(_ptr(a1), _ptr(a2), _ptr(fg), n, -1 if ref_ant is None else int(ref_ant),
                                 _ptr(A), _ptr(I), ctypes.byref(rows), ctypes.byref(cols)))
    r, c = rows.value, cols.value
    return A[: r * c].reshape(c, r).T.copy(), I[: r - 1].copy()


def pseudo_inverse(A: np.ndarray) -> np.ndarray:
    """SVDPseudoInverse (LA/math/cpu/matrix_invert.h:49-56)."""
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    Ad = np.zeros((n, m), dtype=np.float64, order="F")
    _check(lib.leap_pseudo_inverse(_ptr(A), m, n, _ptr(Ad)))
    return np.ascontiguousarray(Ad)


@dataclass
class MetaData:
    """The fields of cpu::MetaData the calibration path uses (LA/model/cpu/MetaData.h:107-127)."""
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

    def constants(self) -> _abi.LeapConstants:
        return _abi.LeapConstants(self.nbaselines, self.reference_antenna, self.channels, self.num_pols,
                                  self.stations, self.rows, self.freq_start_hz, self.freq_inc_hz,
                                  self.phase_centre_ra_rad, self.phase_centre_dec_rad, 0.0, 0.0)


def filtered_baselines(obs, minimum_baseline_threshold: float) -> np.ndarray:
    """MeasurementSet::GetFilteredBaselines (LA/ms/MeasurementSet.cc:181-240)."""
    nbl = obs.nbaselines
    flagged = np.asarray(obs.flags[:nbl], dtype=bool)
    short = np.zeros(nbl, dtype=bool)
    if minimum_baseline_threshold > 0.0:
        uv = obs.uvw[:nbl]
        short = np.sqrt(uv[:, 0] ** 2 + uv[:, 1] ** 2) < minimum_baseline_threshold
    return flagged | short


def build_metadata(obs, reference_antenna: Optional[int] = None, minimum_baseline_threshold: float = 0.0) -> MetaData:
    """cpu::MetaData construction (LA/model/cpu/MetaData.cc:42-137) on the host."""
    ref = reference_antenna if reference_antenna is not None else obs.total_antennas - 1
    fg = filtered_baselines(obs, minimum_baseline_threshold)
    a1 = obs.antenna1[: obs.nbaselines]
    a2 = obs.antenna2[: obs.nbaselines]
    A1, I1 = phase_matrix(a1, a2, fg, ref)
    A, I = phase_matrix(a1, a2, fg, None)
    return MetaData(obs.nbaselines, ref, obs.channels, obs.pols, obs.num_stations, obs.rows,
                    obs.freq_start_hz, obs.freq_inc_hz, obs.phase_centre[0], obs.phase_centre[1],
                    A, I, pseudo_inverse(A), A1, I1, pseudo_inverse(A1))


# ---------------------------------------------------------------------------
# Device context
# ---------------------------------------------------------------------------

def _vis_type(dtype) -> int:
    if dtype == np.complex64:
        return _abi.LEAP_VIS_C64
    if dtype == np.complex128:
        return _abi.LEAP_VIS_C128
    raise InvalidArgument(_abi.LEAP_ERR_INVALID_ARGUMENT, f"unsupported visibility dtype {dtype}")


CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy: the legacy default stream as an explicit handle


def stream_handle(stream: Optional[int]):
    """C-ABI stream argument for a cudaStream_t handle: None selects the context's stream
    (NULL); 0, the legacy default stream (torch's default stream), becomes cudaStreamLegacy."""
    if stream is None:
        return None
    return int(stream) if stream else CUDA_STREAM_LEGACY


class Context:
    """One device, one stream, the resident buffers (leap_create ... leap_destroy)."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        _check(lib.leap_create(device, ctypes.byref(h)))
        self._h = h
        self.device = device
        self.md: Optional[MetaData] = None
        self.slots = {}
        self.autograd_slots = {}  # slot -> (key, vis, uvw) of the differentiable form's last upload
        self._last_slot = None

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib.leap_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, code: int):
        _check(code, self._h)

    def set_metadata(self, md: MetaData):
        k = md.constants()
        A = np.asfortranarray(md.A, dtype=np.float64)
        Ad = np.asfortranarray(md.Ad, dtype=np.float64)
        A1 = np.asfortranarray(md.A1, dtype=np.float64)
        Ad1 = np.asfortranarray(md.Ad1, dtype=np.float64)
        I = np.ascontiguousarray(md.I, dtype=np.int32)
        I1 = np.ascontiguousarray(md.I1, dtype=np.int32)
        if I.size == 0:
            I = np.zeros(1, dtype=np.int32)
        if I1.size == 0:
            I1 = np.zeros(1, dtype=np.int32)
        self._check(lib.leap_set_metadata(self._h, ctypes.byref(k), _ptr(A), A.shape[0], A.shape[1], _ptr(I),
                                          _ptr(Ad), _ptr(A1), A1.shape[0], _ptr(I1), _ptr(Ad1)))
        self.md = md

    def build_metadata(self, obs, reference_antenna: Optional[int] = None, minimum_baseline_threshold: float = 0.0,
                       fetch: bool = True) -> MetaData:
        """MetaData built on the device (leap_build_metadata) from the observation's first-epoch
        baselines; installs it on this context.  With fetch, Ad / Ad1 are copied back and A / I /
        A1 / I1 rebuilt on the host, so the returned MetaData is complete.  The host-path bits
        (1: A, 2: A1) are in ``md.host_path``."""
        ref = reference_antenna if reference_antenna is not None else obs.total_antennas - 1
        fg = np.ascontiguousarray(filtered_baselines(obs, minimum_baseline_threshold), dtype=np.uint8)
        nbl = obs.nbaselines
        a1 = np.ascontiguousarray(obs.antenna1[:nbl], dtype=np.int32)
        a2 = np.ascontiguousarray(obs.antenna2[:nbl], dtype=np.int32)
        k = _abi.LeapConstants(nbl, ref, obs.channels, obs.pols, obs.num_stations, obs.rows, obs.freq_start_hz,
                               obs.freq_inc_hz, obs.phase_centre[0], obs.phase_centre[1], 0.0, 0.0)
        host = ctypes.c_int32(0)
        self._check(lib.leap_build_metadata(self._h, ctypes.byref(k), _ptr(a1), _ptr(a2), _ptr(fg), nbl,
                                            ctypes.byref(host)))
        if fetch:
            A1, I1 = phase_matrix(a1, a2, fg, ref)
            A, I = phase_matrix(a1, a2, fg, None)
            mats = []
            for which in (0, 1):
                r, c = ctypes.c_int32(0), ctypes.c_int32(0)
                self._check(lib.leap_get_metadata_matrix(self._h, which, None, 0, ctypes.byref(r), ctypes.byref(c)))
                out = np.zeros((c.value, r.value), dtype=np.float64)  # column-major S x cols
                self._check(lib.leap_get_metadata_matrix(self._h, which, _ptr(out), out.size, None, None))
                mats.append(out.T.copy())
            md = MetaData(nbl, ref, obs.channels, obs.pols, obs.num_stations, obs.rows, obs.freq_start_hz,
                          obs.freq_inc_hz, obs.phase_centre[0], obs.phase_centre[1], A, I, mats[0], A1, I1, mats[1])
        else:
            md = None
        self.md = md
        if md is not None:
            md.host_path = int(host.value)
        return md

    def set_integration(self, slot: int, vis, uvw):
        """vis: (channels, rows, pols) complex64/complex128 numpy array or CUDA torch tensor
        (a torch complex tensor or its real view); uvw: (rows, 3) float64."""
        self.autograd_slots.pop(slot, None)
        if isinstance(vis, np.ndarray):
            vis = np.ascontiguousarray(vis)
            uvw = np.ascontiguousarray(uvw, dtype=np.float64)
            C, rows, P = vis.shape
            self._check(lib.leap_set_integration(self._h, slot, _vis_type(vis.dtype), _ptr(vis), _ptr(uvw),
                                                 rows, C, P, _abi.LEAP_MEMORY_HOST))
        else:  # torch tensor on the device
            import torch
            assert vis.is_cuda and vis.is_contiguous() and uvw.is_cuda and uvw.is_contiguous()
            # The copy runs on the context's stream: finish torch's pending work on the inputs first.
            torch.cuda.synchronize(vis.device)
            vt = {torch.complex64: _abi.LEAP_VIS_C64, torch.complex128: _abi.LEAP_VIS_C128}[vis.dtype]
            C, rows, P = vis.shape
            self._check(lib.leap_set_integration(self._h, slot, vt, vis.data_ptr(), uvw.data_ptr(), rows, C, P,
                                                 _abi.LEAP_MEMORY_DEVICE))
        self.slots[slot] = (C, rows, P)

    def set_integration_ms(self, slot: int, ms_vis, uvw, start_channel: int = 0, channels: Optional[int] = None,
                           asynchronous: bool = False):
        """Upload from the MeasurementSet's DATA order: ms_vis is (rows, row_channels, pols)
        complex, a numpy array (pageable or not) or a torch tensor (CUDA, or pinned CPU memory);
        channels [start_channel, start_channel + channels) are taken.  Transpose and NaN rule
        run on the device (leap_set_integration_ms)."""
        self.autograd_slots.pop(slot, None)
        if isinstance(ms_vis, np.ndarray):
            ms_vis = np.ascontiguousarray(ms_vis)
            uvw = np.ascontiguousarray(uvw, dtype=np.float64)
            rows, row_channels, P = ms_vis.shape
            vt, vp, up, mem = _vis_type(ms_vis.dtype), _ptr(ms_vis), _ptr(uvw), _abi.LEAP_MEMORY_HOST
        else:
            import torch
            assert ms_vis.is_contiguous() and uvw.is_contiguous() and uvw.dtype == torch.float64
            vt = {torch.complex64: _abi.LEAP_VIS_C64, torch.complex128: _abi.LEAP_VIS_C128}[ms_vis.dtype]
            rows, row_channels, P = ms_vis.shape
            if ms_vis.is_cuda:
                torch.cuda.synchronize(ms_vis.device)
                mem = _abi.LEAP_MEMORY_DEVICE
                assert uvw.is_cuda
            else:
                mem = _abi.LEAP_MEMORY_HOST
                assert not uvw.is_cuda
            vp, up = ms_vis.data_ptr(), uvw.data_ptr()
        C = row_channels - start_channel if channels is None else channels
        fn = lib.leap_set_integration_ms_async if asynchronous else lib.leap_set_integration_ms
        self._check(fn(self._h, slot, vt, vp, row_channels, start_channel, up, rows, C, P, mem))
        self.slots[slot] = (C, rows, P)

    def apply_flags(self, slot: int, flags: np.ndarray, start_channel: int = 0) -> int:
        """Opt-in: zero the (row, channel) groups whose FLAG (rows, row_channels[, pols], MS order)
        is set for any pol; returns the number of groups zeroed (leap_apply_flags)."""
        f = np.ascontiguousarray(flags, dtype=np.uint8)
        if f.ndim == 2:
            f = f[:, :, None]
        rows, row_channels, fp = f.shape
        n = ctypes.c_int64(0)
        self._check(lib.leap_apply_flags(self._h, slot, _ptr(f), row_channels, start_channel, fp,
                                         _abi.LEAP_MEMORY_HOST, ctypes.byref(n)))
        return int(n.value)

    def release_integration(self, slot: int):
        self.autograd_slots.pop(slot, None)
        self._check(lib.leap_release_integration(self._h, slot))
        self.slots.pop(slot, None)

    def calibrate(self, slot: int, dds: np.ndarray, precision: int = _abi.LEAP_PRECISION_FP64) -> np.ndarray:
        dds = np.ascontiguousarray(dds, dtype=np.float64).reshape(-1, 9)
        D = dds.shape[0]
        S = self.md.A.shape[1] if self.md is not None else 1
        cal = np.zeros((D, S), dtype=np.float64)
        self._check(lib.leap_calibrate(self._h, slot, _ptr(dds), D, precision, _ptr(cal)))
        self._last_slot = slot
        return cal

    def calibrate_batched(self, items, dds: np.ndarray, precision: int = _abi.LEAP_PRECISION_MIXED) -> np.ndarray:
        """items: sequence of (slot, first_direction, ndirections); dds: (D, 3, 3)."""
        dds = np.ascontiguousarray(dds, dtype=np.float64).reshape(-1, 9)
        D = dds.shape[0]
        arr = (_abi.LeapWorkItem * len(items))(*[_abi.LeapWorkItem(int(a), int(b), int(c), 0) for a, b, c in items])
        cal = np.zeros((D, self.md.A.shape[1]), dtype=np.float64)
        self._check(lib.leap_calibrate_batched(self._h, arr, len(items), _ptr(dds), D, precision, _ptr(cal)))
        self._last_slot = int(items[0][0])
        return cal

    def set_autotune(self, enable: bool):
        self._check(lib.leap_set_autotune(self._h, int(bool(enable))))

    def set_option(self, option: int, value: int):
        self._check(lib.leap_set_option(self._h, int(option), int(value)))

    def calibrate_async(self, slot: int, dd_ptr: int, ndir: int, precision: int, cal_ptr: int,
                        stream: Optional[int] = None):
        """Device pointers; `stream` is a cudaStream_t handle (torch's Stream.cuda_stream; 0 is the
        legacy default stream), None the context's own stream."""
        self._check(lib.leap_calibrate_async(self._h, slot, dd_ptr, ndir, precision, cal_ptr, stream_handle(stream)))

    def avgdata(self, direction: int) -> np.ndarray:
        """avgData of one direction from the last call, as (nbl, pols) complex128."""
        C, rows, P = self.slots[self._last_slot]
        nbl = self.md.nbaselines
        out = np.zeros(2 * nbl * P, dtype=np.float64)
        self._check(lib.leap_get_avgdata(self._h, direction, _ptr(out)))
        return out.view(np.complex128).reshape(P, nbl).T.copy()

    def rotate_uvw(self, slot: int, dds: np.ndarray) -> np.ndarray:
        dds = np.ascontiguousarray(dds, dtype=np.float64).reshape(-1, 9)
        C, rows, P = self.slots[slot]
        out = np.zeros((dds.shape[0], rows, 3), dtype=np.float64)
        self._check(lib.leap_rotate_uvw(self._h, slot, _ptr(dds), dds.shape[0], _ptr(out)))
        return out

    def timings(self) -> dict:
        t = _abi.LeapTimings()
        self._check(lib.leap_get_timings(self._h, ctypes.byref(t)))
        return {"rotate_ms": t.rotate_ms, "solve_ms": t.solve_ms, "total_ms": t.total_ms, "kernels": t.kernels,
                "calls": t.calls}

    def timing_reset(self):
        self._check(lib.leap_timing_reset(self._h))

    def synchronize(self):
        self._check(lib.leap_synchronize(self._h))


# ---------------------------------------------------------------------------
# ILeapCalibrator mirror
# ---------------------------------------------------------------------------

def evaluate_slice(start: int, interval: int, end: int, collection_size: int):
    """Slice::Evaluate + Range (LA/common/Slice.h:47-54, LA/common/Range.h:40-63)."""
    s = collection_size if start == -1 else start
    i = collection_size if interval == -1 else interval
    e = collection_size if end == -1 else end
    if s < 0 or i < 1 or e < 0:
        raise InvalidArgument(_abi.LEAP_ERR_INVALID_ARGUMENT, "expected a positive integer")
    return s, i, e, (e - s) // i


class GpuLeapCalibrator:
    """ILeapCalibrator::Calibrate over the GB300 path (ComputeImplementation "gb300")."""

    def __init__(self, device: int = 0, precision: int = _abi.LEAP_PRECISION_FP64):
        self.ctx = Context(device)
        self.precision = precision

    def calibrate(self, obs, directions: Sequence[Sequence[float]], solution_interval=(0, -1, -1),
                  minimum_baseline_threshold: float = 0.0, reference_antenna: Optional[int] = None,
                  is_file_system_cache_enabled: bool = False, md: Optional[MetaData] = None) -> List[dict]:
        if md is None:
            md = build_metadata(obs, reference_antenna, minimum_baseline_threshold)
        self.ctx.set_metadata(md)
        _, interval, _, solutions = evaluate_slice(*solution_interval, obs.timesteps)
        nbl = obs.nbaselines
        directions = np.asarray(directions, dtype=np.float64).reshape(-1, 2)
        dds = np.stack([dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in directions])
        out = []
        for s in range(solutions):
            r0 = s * interval * nbl  # start row ignores Slice.start, as CpuLeapCalibrator.cc:116 does
            nrows = interval * nbl
            ms_vis = getattr(obs, "ms_vis", None)
            if ms_vis is not None:  # MeasurementSet order [row][channel][pol]: transposed on the device
                self.ctx.set_integration_ms(0, ms_vis[r0:r0 + nrows], obs.uvw[r0:r0 + nrows])
            else:
                self.ctx.set_integration(0, np.ascontiguousarray(obs.vis[:, r0:r0 + nrows, :]), obs.uvw[r0:r0 + nrows])
            cal = self.ctx.calibrate(0, dds, self.precision)
            out.append({
                "epoch": {"start": float(obs.epochs[s * interval]), "end": float(obs.epochs[(s + 1) * interval - 1])},
                "calibration": [{"direction": [float(x) for x in directions[i]], "beamCalibration": cal[i].tolist()}
                                for i in range(len(directions))],
            })
        return out
