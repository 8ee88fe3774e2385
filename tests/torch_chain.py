"""Float64 PyTorch restatement of the calibration chain, for autograd checks.

Written from the reference's loops (LA/algorithm/cpu/CpuLeapCalibrator.cc:
RotateVisibilities :181-217, PhaseRotate :147-178), not from this repository's
kernels: rotate every pol-0 sample by exp(-2*pi*i*(w_rot - w)/lambda_c),
sum over channels and timesteps (groups with a NaN in any pol skipped), then
phi1 = arg(avg[I1]) ++ [0], cal1 = Ad1 phi1, dInt[n] = arg(exp(-2*pi*i*(A cal1)[n])
avg[n]) for n < |I| (row n, not I[n]), cal = Ad (dInt ++ [0]) + cal1.
Directions enter as (l, m); the third row of the direction matrix is (l, m, n),
n = sqrt(1 - l^2 - m^2).  Test infrastructure only.
"""
import math

import torch

SPEED_OF_LIGHT = 299792458.0


def chain(lm, vis, uvw, md, nbl, f0, df):
    """Returns cal (D, S), avg0 (D, nbl), phi1 (D, |I1|), dint (D, |I|) as float64/complex128 tensors."""
    dev = vis.device
    C, rows, P = vis.shape
    T = rows // nbl
    u, v, w = uvw[:, 0], uvw[:, 1], uvw[:, 2]
    inv_lambda = (f0 + torch.arange(C, dtype=torch.float64, device=dev) * df) / SPEED_OF_LIGHT
    bad = (torch.isnan(vis.real) | torch.isnan(vis.imag)).any(dim=2)
    v0 = torch.where(bad, torch.zeros((), dtype=vis.dtype, device=dev), vis[:, :, 0])
    avgs = []
    for d in range(lm.shape[0]):
        l, m = lm[d, 0], lm[d, 1]
        n = torch.sqrt(1.0 - l * l - m * m)
        wrot = l * u + m * v + n * w
        shift = -2.0 * math.pi * (wrot - w)
        phase = shift[None, :] * inv_lambda[:, None]
        rot = v0 * torch.exp(1j * phase)
        avgs.append(rot.sum(dim=0).reshape(T, nbl).sum(dim=0))
    avg0 = torch.stack(avgs)
    A = torch.as_tensor(md.A, dtype=torch.float64, device=dev)
    Ad = torch.as_tensor(md.Ad, dtype=torch.float64, device=dev)
    Ad1 = torch.as_tensor(md.Ad1, dtype=torch.float64, device=dev)
    I1 = torch.as_tensor(md.I1, dtype=torch.int64, device=dev)
    I1 = torch.where(I1 < 0, I1 + nbl, I1)
    D = lm.shape[0]
    zero = torch.zeros((D, 1), dtype=torch.float64, device=dev)
    phi1 = torch.angle(avg0[:, I1])
    cal1 = torch.cat([phi1, zero], dim=1) @ Ad1.T
    acal = cal1 @ A.T
    nI = A.shape[0] - 1
    dint = torch.angle(torch.exp(-2j * math.pi * acal[:, :nI]) * avg0[:, :nI])
    cal = torch.cat([dint, zero], dim=1) @ Ad.T + cal1
    return cal, avg0, phi1, dint


def wrapped(x):
    return torch.atan2(torch.sin(x), torch.cos(x))


def loss_per_direction(cal, gain_phase):
    """Sum over antennas of the squared wrapped residual between cal and the injected gain phases."""
    return (wrapped(cal - gain_phase[None, :]) ** 2).sum(dim=1)


def branch_margin(cal, phi1, dint, gain_phase):
    """Per direction: the smallest distance of any arg() output or wrapped residual from +-pi."""
    res = wrapped(cal - gain_phase[None, :])
    parts = [math.pi - res.abs(), math.pi - phi1.abs(), math.pi - dint.abs()]
    return torch.stack([p.min(dim=1).values for p in parts], dim=1).min(dim=1).values
