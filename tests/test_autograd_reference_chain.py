"""The float64 PyTorch chain used as the autograd reference: its cal phases
equal the oracle's, and its autograd gradient equals central differences.
CPU only."""
import numpy as np
import torch

import oracle
import leap_gb300 as lg
from leap_gb300 import synth
from leap_gb300.autograd import lm_to_dd

import torch_chain


def _case():
    obs, _ = synth.small_case(stations=10, timesteps=2, channels=6, directions=3, vis_dtype=np.complex128,
                              seed_shift=4)
    _, lm = synth.random_directions(3, box_rad=0.06, seed=21)
    return obs, lm


def test_chain_matches_oracle():
    obs, lm = _case()
    md = lg.build_metadata(obs)
    mdo = oracle.metadata(obs)
    dds = lm_to_dd(lm, obs.phase_centre)
    exp = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo)
    cal, *_ = torch_chain.chain(torch.from_numpy(lm), torch.from_numpy(obs.vis), torch.from_numpy(obs.uvw), md,
                                obs.nbaselines, obs.freq_start_hz, obs.freq_inc_hz)
    assert np.abs(cal.numpy() - exp).max() < 1e-10


def test_chain_autograd_matches_central_differences():
    obs, lm = _case()
    md = lg.build_metadata(obs)
    gain = torch.from_numpy(np.angle(obs.gains))
    vis = torch.from_numpy(obs.vis)
    uvw = torch.from_numpy(obs.uvw)
    args = (vis, uvw, md, obs.nbaselines, obs.freq_start_hz, obs.freq_inc_hz)
    x = torch.from_numpy(lm.copy()).requires_grad_()
    L = torch_chain.loss_per_direction(torch_chain.chain(x, *args)[0], gain).sum()
    L.backward()
    h = 1e-7
    for d in range(lm.shape[0]):
        for q in range(2):
            lp, lmn = lm.copy(), lm.copy()
            lp[d, q] += h
            lmn[d, q] -= h
            Lp = torch_chain.loss_per_direction(torch_chain.chain(torch.from_numpy(lp), *args)[0], gain).sum()
            Lm = torch_chain.loss_per_direction(torch_chain.chain(torch.from_numpy(lmn), *args)[0], gain).sum()
            fd = float(Lp - Lm) / (2 * h)
            g = float(x.grad[d, q])
            assert abs(fd - g) <= 1e-5 * max(1.0, abs(g)), (d, q, fd, g)
