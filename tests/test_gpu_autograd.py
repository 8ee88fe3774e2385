"""Differentiable form: gradients of a wrapped phase-residual loss with respect
to each direction's (l, m) and to the visibilities, from the library's FP64
adjoint kernels through torch.autograd (leap_gb300.autograd.CalibrateLM).

Checked against (1) a float64 PyTorch autograd re-implementation of the same
chain (tests/torch_chain.py, itself pinned to the oracle on the CPU) and
(2) central finite differences of the FP64 forward with step 1e-7 rad in l and
m, and a directional difference in the visibilities.  Workload: 128 antennas,
8 timesteps, 96 channels, 4 pols, 16 directions, complex<float> visibilities.

The loss is differentiable only on the smooth branch of every arg(): with 8128
dInt angles per direction, a step of 1e-7 rad in l moves some angle across
+-pi in every direction (up to 0.03 rad shifts).  The differences therefore
take the library's avgData at l +- h (the rotate + average stage, smooth in
l and V) and continue each arg() of the solve from its value at the base
point, which is the function whose derivative the adjoint computes.
"""
import numpy as np
import pytest
import torch

import leap_gb300 as lg
from leap_gb300 import synth
from leap_gb300.autograd import calibrate_lm, lm_to_dd

import torch_chain

pytestmark = pytest.mark.gpu



def _workload(ndir=16, timesteps=8, channels=96, stations=128, nan_samples=0):
    if stations == 128:
        obs, _ = synth.mwa_precision(timesteps=timesteps, channels=channels, directions=ndir)
    else:
        obs, _ = synth.small_case(stations=stations, timesteps=timesteps, channels=channels, directions=ndir,
                                  vis_dtype=np.complex64, seed_shift=7)
    _, lm = synth.random_directions(ndir, box_rad=0.1, seed=31)
    lm[0] = (0.01, -0.005) if stations == 128 else lm[0]
    if nan_samples:
        flat = obs.vis.reshape(-1)
        idx = np.random.default_rng(5).integers(0, flat.size, nan_samples)
        flat[idx] = np.nan
    return obs, lm


def _setup(ctx, obs):
    md = lg.build_metadata(obs)
    ctx.set_metadata(md)
    dev = torch.device("cuda:0")
    vis = torch.from_numpy(obs.vis).to(dev)
    uvw = torch.from_numpy(obs.uvw).to(dev)
    gain = torch.from_numpy(np.angle(obs.gains)).to(dev)
    return md, vis, uvw, gain


def _reference(obs, md, lm, vis, uvw, gain):
    lm_r = torch.from_numpy(lm).cuda().requires_grad_()
    vis_r = vis.to(torch.complex128).requires_grad_()
    cal, avg0, phi1, dint = torch_chain.chain(lm_r, vis_r, uvw, md, obs.nbaselines, obs.freq_start_hz,
                                              obs.freq_inc_hz)
    loss = torch_chain.loss_per_direction(cal, gain)
    loss.sum().backward()
    margin = torch_chain.branch_margin(cal.detach(), phi1.detach(), dint.detach(), gain)
    return cal.detach(), loss.detach(), lm_r.grad, vis_r.grad, margin


@pytest.mark.parametrize("nan_samples", [0, 60])
def test_gradients_match_float64_autograd(ctx, nan_samples):
    obs, lm = _workload(nan_samples=nan_samples)
    md, vis, uvw, gain = _setup(ctx, obs)
    lm_t = torch.from_numpy(lm).cuda().requires_grad_()
    vis_t = vis.clone().requires_grad_()
    cal = calibrate_lm(ctx, 0, lm_t, vis_t, uvw, lg.LEAP_PRECISION_FP64)
    loss = torch_chain.loss_per_direction(cal, gain)
    loss.sum().backward()
    cal_r, loss_r, glm_r, gvis_r, margin = _reference(obs, md, lm, vis, uvw, gain)
    # same values, hence the same branch of every arg()
    assert (cal.detach() - cal_r).abs().max() < 1e-10
    assert (loss.detach() - loss_r).abs().max() < 1e-8 * loss_r.abs().max()
    # dL/d(l, m): relative to each direction's gradient scale
    glm = lm_t.grad
    rel = (glm - glm_r).abs().max(dim=1).values / glm_r.abs().max(dim=1).values.clamp_min(1e-30)
    assert rel.max() < 1e-8, rel
    # dL/dV: only pol 0 is non-zero; complex<float> gradient (FP32 rounding)
    gv = vis_t.grad
    assert gv.dtype == torch.complex64
    assert gv[:, :, 1:].abs().max() == 0
    assert ((gv.to(torch.complex128) - gvis_r).abs().max() / gvis_r.abs().max()) < 1e-6
    if nan_samples:
        bad = (torch.isnan(vis.real) | torch.isnan(vis.imag)).any(dim=2)
        assert bad.any() and gv[bad].abs().max() == 0


class SmoothSolve:
    """Host FP64 solve from the library's avgData (pol 0) with every arg() continued
    from its value at a base point (the smooth branch through that point)."""

    def __init__(self, md, gain):
        self.md, self.gain = md, gain.cpu().numpy()
        self.I1 = np.where(md.I1 < 0, md.I1 + md.nbaselines, md.I1)
        self.nI = md.A.shape[0] - 1
        self.base = None

    def loss(self, avg0):
        md, nI = self.md, self.nI
        D = avg0.shape[0]
        z1 = avg0[:, self.I1]
        if self.base is None:
            phi1 = np.angle(z1)
        else:
            phi1 = self.base["phi1"] + np.angle(z1 * np.conj(self.base["z1"]))
        cal1 = np.concatenate([phi1, np.zeros((D, 1))], axis=1) @ md.Ad1.T
        z = np.exp(-2j * np.pi * (cal1 @ md.A.T)[:, :nI]) * avg0[:, :nI]
        if self.base is None:
            dint = np.angle(z)
        else:
            dint = self.base["dint"] + np.angle(z * np.conj(self.base["z"]))
        cal = np.concatenate([dint, np.zeros((D, 1))], axis=1) @ md.Ad.T + cal1
        if self.base is None:
            res = np.angle(np.exp(1j * (cal - self.gain[None, :])))
            self.base = {"phi1": phi1, "z1": z1, "dint": dint, "z": z, "cal": cal, "res": res}
        else:
            res = self.base["res"] + (cal - self.base["cal"])
        return (res ** 2).sum(axis=1), cal


def _avg0(ctx, ndir):
    return np.stack([ctx.avgdata(d)[:, 0] for d in range(ndir)])


def test_lm_gradient_matches_central_differences(ctx):
    obs, lm = _workload()
    md, vis, uvw, gain = _setup(ctx, obs)
    lm_t = torch.from_numpy(lm).cuda().requires_grad_()
    cal = calibrate_lm(ctx, 0, lm_t, vis, uvw, lg.LEAP_PRECISION_FP64)
    torch_chain.loss_per_direction(cal, gain).sum().backward()
    g = lm_t.grad.cpu().numpy()
    ctx.set_integration(0, obs.vis, obs.uvw)
    pc = (md.phase_centre_ra_rad, md.phase_centre_dec_rad)
    solve = SmoothSolve(md, gain)
    ctx.calibrate(0, lm_to_dd(lm, pc))
    L0, cal0 = solve.loss(_avg0(ctx, len(lm)))
    assert np.abs(cal0 - cal.detach().cpu().numpy()).max() < 1e-9
    h = 1e-7
    fd = np.zeros_like(lm)
    for q in range(2):
        lp, lmn = lm.copy(), lm.copy()
        lp[:, q] += h
        lmn[:, q] -= h
        ctx.calibrate(0, lm_to_dd(lp, pc))
        Lp, _ = solve.loss(_avg0(ctx, len(lm)))
        ctx.calibrate(0, lm_to_dd(lmn, pc))
        Lm, _ = solve.loss(_avg0(ctx, len(lm)))
        fd[:, q] = (Lp - Lm) / (2 * h)
    rel = np.abs(fd - g).max(axis=1) / np.abs(g).max(axis=1)
    # most directions agree to 1e-8; the O(h^2) truncation term reaches ~2e-5 where an avgData
    # entry is small (the curvature of arg() grows as 1/|z|^2)
    assert np.median(rel) < 1e-7 and rel.max() < 1e-4, rel


@pytest.mark.parametrize("eps", [1e-4, 1e-5])
def test_vis_gradient_matches_directional_differences(ctx, eps):
    obs, lm = _workload()
    md, vis, uvw, gain = _setup(ctx, obs)
    lm_t = torch.from_numpy(lm).cuda()
    vis_t = vis.clone().requires_grad_()
    cal = calibrate_lm(ctx, 0, lm_t, vis_t, uvw, lg.LEAP_PRECISION_FP64)
    torch_chain.loss_per_direction(cal, gain).sum().backward()
    g = vis_t.grad.to(torch.complex128)
    rng = np.random.default_rng(3)
    dv = torch.from_numpy((rng.standard_normal(obs.vis.shape) + 1j * rng.standard_normal(obs.vis.shape)).astype(
        np.complex64)).cuda()
    vp, vm = vis + eps * dv, vis - eps * dv
    pc = (md.phase_centre_ra_rad, md.phase_centre_dec_rad)
    dds = lm_to_dd(lm, pc)
    solve = SmoothSolve(md, gain)
    ctx.set_integration(0, vis, uvw)
    ctx.calibrate(0, dds)
    solve.loss(_avg0(ctx, len(lm)))
    ctx.set_integration(0, vp, uvw)
    ctx.calibrate(0, dds)
    Lp, _ = solve.loss(_avg0(ctx, len(lm)))
    ctx.set_integration(0, vm, uvw)
    ctx.calibrate(0, dds)
    Lm, _ = solve.loss(_avg0(ctx, len(lm)))
    actual = (vp - vm).to(torch.complex128)  # the perturbation after FP32 rounding
    pred = float((g.real * actual.real + g.imag * actual.imag).sum())
    diff = float(Lp.sum() - Lm.sum())
    # central differences: O(eps^2) truncation (2.7e-2 relative at eps = 1e-3)
    assert abs(diff - pred) <= 1e-3 * abs(pred), (diff, pred)


def test_mixed_forward_gradient_is_close(ctx):
    """With the mixed-precision forward, the adjoint runs at the mixed avgData: the
    gradient agrees with the FP64 one to the forward's own accuracy."""
    obs, lm = _workload()
    md, vis, uvw, gain = _setup(ctx, obs)
    grads = []
    for prec in (lg.LEAP_PRECISION_FP64, lg.LEAP_PRECISION_MIXED):
        lm_t = torch.from_numpy(lm).cuda().requires_grad_()
        torch_chain.loss_per_direction(calibrate_lm(ctx, 0, lm_t, vis, uvw, prec), gain).sum().backward()
        grads.append(lm_t.grad)
    rel = (grads[1] - grads[0]).abs().max(dim=1).values / grads[0].abs().max(dim=1).values
    assert rel.max() < 1e-3, rel


def test_backward_rejects_bad_slot(ctx):
    from leap_gb300 import _abi
    obs, lm = _workload(ndir=2, timesteps=1, channels=8, stations=8)
    md, vis, uvw, gain = _setup(ctx, obs)
    z = torch.zeros(64, dtype=torch.float64, device="cuda")
    rc = _abi.lib.leap_backward(ctx.handle, 12345, z.data_ptr(), 1, z.data_ptr(), z.data_ptr(), None, z.data_ptr(),
                                None, None)
    assert rc == _abi.LEAP_ERR_NOT_READY
