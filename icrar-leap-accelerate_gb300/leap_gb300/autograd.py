"""Differentiable calibration: cal phases as a function of each direction's
(l, m) and of the visibilities, with the gradient from the library's FP64
adjoint kernels (``leap_backward`` in include/leap_gb300.h).

Forward: the directions enter as (l, m) about the phase centre.  The third row
of each direction matrix, the only row the path reads
(LA/algorithm/cpu/CpuLeapCalibrator.cc:191-199), is set to (l, m, n) with
n = sqrt(1 - l^2 - m^2).  The other two rows come from the reference's
MetaData::GenerateDDMatrix (LA/model/cpu/MetaData.cc:166-203) of the same
direction.  One leap_calibrate_async call returns cal (D, S), float64.

Backward: leap_backward recomputes the rotated samples from the visibilities
rather than storing them.  It gives dL/d(l, m, n), chained here to (l, m)
through n(l, m), and dL/dV as complex gradients (dL/dRe + i dL/dIm), the
convention of torch's complex autograd.  The gradients hold on the smooth
branch of every arg(), away from angles at +-pi.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _abi
from .calibrator import Context, dd_matrix, stream_handle

__all__ = ["lm_to_dd", "CalibrateLM", "calibrate_lm"]


def lm_to_dd(lm: np.ndarray, phase_centre) -> np.ndarray:
    """(D, 2) direction cosines -> (D, 3, 3) direction matrices with row 2 = (l, m, n) exactly."""
    lm = np.asarray(lm, dtype=np.float64).reshape(-1, 2)
    ra0, dec0 = phase_centre
    out = np.empty((lm.shape[0], 3, 3))
    for i, (l, m) in enumerate(lm):
        n = np.sqrt(1.0 - l * l - m * m)
        dec = np.arcsin(m * np.cos(dec0) + n * np.sin(dec0))
        ra = ra0 + np.arctan2(l, n * np.cos(dec0) - m * np.sin(dec0))
        dd = dd_matrix(ra0, dec0, ra, dec)
        dd[2] = (l, m, n)
        out[i] = dd
    return out


def _ensure_slot(context: Context, slot: int, vis: torch.Tensor, uvw: torch.Tensor):
    """Make `slot` hold exactly these visibilities and UVWs (re-uploads if anything changed).
    The cache keeps references to both tensors, so their memory cannot be reused by
    other tensors while the slot is recorded as holding them."""
    key = (vis.data_ptr(), tuple(vis.shape), vis.dtype, vis._version, uvw.data_ptr(), tuple(uvw.shape), uvw._version)
    cached = context.autograd_slots.get(slot)
    if cached is None or cached[0] != key:
        context.set_integration(slot, vis, uvw)
        context.autograd_slots[slot] = (key, vis, uvw)


class CalibrateLM(torch.autograd.Function):
    """cal = Calibrate(lm, vis) on one resident integration (see the module docstring)."""

    @staticmethod
    def forward(fctx, lm, vis, uvw, context: Context, slot: int, precision: int):
        if not (lm.is_cuda and vis.is_cuda and uvw.is_cuda):
            raise ValueError("lm, vis and uvw must be CUDA tensors")
        if context.md is None:
            raise ValueError("set the context's metadata first")
        vis_d = vis.detach().contiguous()
        uvw_d = uvw.detach().contiguous().to(torch.float64)
        _ensure_slot(context, slot, vis_d, uvw_d)
        md = context.md
        dd = torch.from_numpy(lm_to_dd(lm.detach().cpu().numpy(), (md.phase_centre_ra_rad, md.phase_centre_dec_rad)))
        dd = dd.reshape(-1).to(vis.device)
        D, S, nbl = lm.shape[0], md.A.shape[1], md.nbaselines
        cal = torch.empty((D, S), dtype=torch.float64, device=vis.device)
        avg0 = torch.empty((D, nbl), dtype=torch.complex128, device=vis.device)
        stream = torch.cuda.current_stream(vis.device).cuda_stream
        context.calibrate_async(slot, dd.data_ptr(), D, precision, cal.data_ptr(), stream)
        context._check(_abi.lib.leap_get_avgdata_device(context.handle, 0, avg0.data_ptr(), stream_handle(stream)))
        fctx.saved = (lm.detach(), vis_d, uvw_d, dd, avg0)
        fctx.context, fctx.slot = context, slot
        return cal

    @staticmethod
    def backward(fctx, grad_cal):
        lm, vis, uvw, dd, avg0 = fctx.saved
        context, slot = fctx.context, fctx.slot
        _ensure_slot(context, slot, vis, uvw)
        D = lm.shape[0]
        g_cal = grad_cal.detach().contiguous().to(torch.float64)
        g_lmn = torch.empty((D, 3), dtype=torch.float64, device=vis.device)
        g_vis = torch.empty_like(vis) if fctx.needs_input_grad[1] else None
        stream = torch.cuda.current_stream(vis.device).cuda_stream
        context._check(_abi.lib.leap_backward(context.handle, slot, dd.data_ptr(), D, avg0.data_ptr(),
                                              g_cal.data_ptr(), vis.data_ptr(), g_lmn.data_ptr(),
                                              g_vis.data_ptr() if g_vis is not None else None,
                                              stream_handle(stream)))
        g_lm = None
        if fctx.needs_input_grad[0]:
            l, m = lm[:, 0], lm[:, 1]
            n = torch.sqrt(1.0 - l * l - m * m)
            g_lm = torch.stack([g_lmn[:, 0] - g_lmn[:, 2] * l / n, g_lmn[:, 1] - g_lmn[:, 2] * m / n], dim=1)
            g_lm = g_lm.to(lm.dtype)
        return g_lm, g_vis, None, None, None, None


def calibrate_lm(context: Context, slot: int, lm: torch.Tensor, vis: torch.Tensor, uvw: torch.Tensor,
                 precision: int = _abi.LEAP_PRECISION_FP64) -> torch.Tensor:
    """Differentiable calibration of directions `lm` (D, 2) against `vis` (C, rows, P) / `uvw` (rows, 3)."""
    return CalibrateLM.apply(lm, vis, uvw, context, slot, precision)
