"""The reference's own calibration directions: the nine of its end-to-end
multi-direction run (src/icrar/leap-accelerate-cli/tests/E2EPerformanceTests.cc:65-76),
up to ~1 rad from the phase centre of its MWA test set (the phase centre of the DD
known-answer test, MetaDataTests.cc:146-165), on the 128-antenna array at its full
384 channels.  The phase slopes of such directions span many grid points, so the
gridded kernel's windows take several passes.

Both mixed-form rotate + average kernels (the gridded one forced on, and the
pipelined CUDA-core one) and the FP64 form are checked against the oracle:
FP64 within 1e-10 rad; mixed within 1e-5 rad (or, for a direction that passes an
arg() within 1e-4 of +-pi, within 1e-5 of the oracle's solve with that angle on the
other branch).  The reference's call shape is also run through the calibrator:
Slice(0, 1, 1) and reference antenna 0.
"""
import json
import os

import numpy as np
import pytest

import oracle
import leap_gb300 as lg
from leap_gb300 import synth
from leap_gb300._abi import LEAP_OPTION_GRIDDED_ROTATION
from test_gpu_parity import FP64_CAL_TOL, MIXED_CAL_TOL, _dds, assert_cal_close

pytestmark = pytest.mark.gpu

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))
PHASE_CENTRE = tuple(KATS["dd"]["phase_centre"])
DIRECTIONS = np.asarray(KATS["e2e_directions"]["radec"], dtype=np.float64)


@pytest.fixture(scope="module")
def case():
    obs = synth.mwa_at_phase_centre(PHASE_CENTRE, timesteps=4, channels=384)
    mdo = oracle.metadata(obs)
    return obs, mdo


def test_directions_are_far_from_the_phase_centre(case):
    obs, _ = case
    dd = np.stack([oracle.dd_matrix(*PHASE_CENTRE, r, d) for r, d in DIRECTIONS])
    n = dd[:, 2, 2]  # third row of the direction matrix is (l, m, n)
    assert len(DIRECTIONS) == 9 and np.arccos(n).max() > 0.9


@pytest.mark.parametrize("gridded", [1, 0], ids=["gridded", "pipelined"])
def test_reference_directions_mixed(ctx, case, gridded):
    obs, mdo = case
    md = lg.build_metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = _dds(md, DIRECTIONS)
    ctx.set_option(LEAP_OPTION_GRIDDED_ROTATION, gridded)
    try:
        cal = ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED)
        avg = np.stack([ctx.avgdata(d) for d in range(len(DIRECTIONS))])
    finally:
        ctx.set_option(LEAP_OPTION_GRIDDED_ROTATION, 2)
    cal_o, avg_o = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo, return_avg=True)
    assert np.isfinite(cal).all()
    scale = np.abs(obs.vis).sum(axis=0).reshape(obs.timesteps, obs.nbaselines, 4).sum(axis=0)
    assert (np.abs(avg - avg_o) / np.maximum(scale, 1e-30)[None]).max() < 2e-6
    flipped = assert_cal_close(cal, cal_o, avg_o, mdo, MIXED_CAL_TOL)
    print(f"{'gridded' if gridded else 'pipelined'}: {flipped} of {len(DIRECTIONS)} directions on another branch")
    ctx.release_integration(0)


def test_reference_directions_fp64(ctx, case):
    obs, mdo = case
    md = lg.build_metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = _dds(md, DIRECTIONS)
    cal = ctx.calibrate(0, dds, lg.LEAP_PRECISION_FP64)
    cal_o = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo)
    assert np.abs(cal - cal_o).max() <= FP64_CAL_TOL
    ctx.release_integration(0)


def test_reference_call_shape(case):
    """Calibrate(ms, directions, Slice(0, 1, 1), 0.0, 0, false), the reference's end-to-end call.
    The reference checks the reference antenna's flag by indexing the baseline flags with the
    antenna number (PhaseMatrixFunction.cc:52-57), and baseline 0 here is the flagged
    autocorrelation of antenna 0; so this copy of the observation leaves the autocorrelations
    unflagged (they never enter A, which holds cross baselines only)."""
    import copy
    obs = copy.copy(case[0])
    obs.flags = np.zeros_like(obs.flags)
    cal = lg.GpuLeapCalibrator(0, lg.LEAP_PRECISION_FP64)
    got = cal.calibrate(obs, DIRECTIONS, (0, 1, 1), 0.0, 0)
    exp = oracle.calibrate(obs, DIRECTIONS, (0, 1, 1), 0.0, 0)
    cal.ctx.close()
    assert len(got) == len(exp) == 1
    for gb, eb in zip(got[0]["calibration"], exp[0]["calibration"]):
        assert gb["direction"] == eb["direction"]
        assert np.abs(np.array(gb["beamCalibration"]) - np.array(eb["beamCalibration"])).max() <= FP64_CAL_TOL
