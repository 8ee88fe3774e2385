"""The mixed form's Ad contraction on the tensor cores (3xTF32 tcgen05 MMAs,
FP32 accumulate in tensor memory, K split over CTAs and finished in FP64).

Checked three ways: against the FP32 CUDA-core contraction of the same call
(both are FP32-accurate sums of the same products: within 2e-6 rad), against
the oracle (the mixed-form bar, 1e-5 rad), and through the batched path.
Shapes cover one and several 128-station M tiles, every N tile width
(32/64/128/256 directions) and two N tiles."""
import numpy as np
import pytest

import oracle
import leap_gb300 as lg
from leap_gb300 import synth
from leap_gb300._abi import LEAP_OPTION_TENSOR_CORE_CONTRACTION

pytestmark = pytest.mark.gpu

MIXED_CAL_TOL = 1e-5
TC_VS_CUDA_CORE_TOL = 2e-6


def _dds(md, dirs):
    return np.stack([lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs])


@pytest.mark.parametrize("stations,ndir", [(12, 1), (40, 19), (64, 33), (130, 70), (150, 200), (20, 300)])
def test_tensor_core_contraction_matches_cuda_core_and_oracle(ctx, stations, ndir):
    obs, dirs = synth.small_case(stations=stations, timesteps=2, channels=9, directions=ndir,
                                 vis_dtype=np.complex64, seed_shift=stations + ndir)
    md = lg.build_metadata(obs)
    mdo = oracle.metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = _dds(md, dirs)
    try:
        ctx.set_option(LEAP_OPTION_TENSOR_CORE_CONTRACTION, 1)
        tc = ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED)
        ctx.set_option(LEAP_OPTION_TENSOR_CORE_CONTRACTION, 0)
        cc = ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED)
    finally:
        ctx.set_option(LEAP_OPTION_TENSOR_CORE_CONTRACTION, 1)
    assert np.isfinite(tc).all()
    assert np.abs(tc - cc).max() <= TC_VS_CUDA_CORE_TOL
    cal_o = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo)
    assert np.abs(tc - cal_o).max() <= MIXED_CAL_TOL
    ctx.release_integration(0)


def test_tensor_core_contraction_batched(ctx):
    """Uneven chunks through leap_calibrate_batched with the tensor-core contraction."""
    from test_gpu_batched import make_chunks
    chunks = make_chunks(48, [(2, 30, 40), (1, 50, 9), (3, 12, 100)], seed=5)
    md = lg.build_metadata(chunks[0][0])
    mdo = oracle.metadata(chunks[0][0])
    ctx.set_metadata(md)
    items, dds = [], []
    for slot, (obs, dirs, d0) in enumerate(chunks):
        ctx.set_integration(slot, obs.vis, obs.uvw)
        items.append((slot, d0, len(dirs)))
        dds += [lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs]
    dds = np.stack(dds)
    cal = ctx.calibrate_batched(items, dds, lg.LEAP_PRECISION_MIXED)
    for slot, (obs, dirs, d0) in enumerate(chunks):
        exp = oracle.calibrate_interval(obs.vis, obs.uvw, dds[d0:d0 + len(dirs)], mdo)
        assert np.abs(cal[d0:d0 + len(dirs)] - exp).max() <= MIXED_CAL_TOL, slot
    np.testing.assert_array_equal(cal, ctx.calibrate_batched(items, dds, lg.LEAP_PRECISION_MIXED))
    for slot in range(len(chunks)):
        ctx.release_integration(slot)


def test_unknown_option_is_rejected(ctx):
    with pytest.raises(lg.InvalidArgument):
        ctx.set_option(99, 1)


@pytest.mark.parametrize("stations,timesteps,channels,ndir", [(64, 9, 23, 40), (33, 5, 5, 16), (40, 3, 70, 12),
                                                              (128, 2, 96, 64)])
def test_tensor_core_rotation_matches_cuda_core_and_oracle(ctx, stations, timesteps, channels, ndir):
    """The rotate + average multiply-accumulate as 3xTF32 mma.sync (16 directions per unit) against
    the FP32 CUDA-core kernel and the oracle: partial 32-baseline tiles, partial 16-channel chunks,
    direction counts that are not multiples of 16, several timestep slabs."""
    from leap_gb300._abi import LEAP_OPTION_TENSOR_CORE_ROTATION
    obs, dirs = synth.small_case(stations=stations, timesteps=timesteps, channels=channels, directions=ndir,
                                 vis_dtype=np.complex64, seed_shift=stations + 3)
    md = lg.build_metadata(obs)
    mdo = oracle.metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = _dds(md, dirs)
    out = {}
    try:
        for flag in (1, 0):
            ctx.set_option(LEAP_OPTION_TENSOR_CORE_ROTATION, 2 if flag else 0)
            cal = ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED)
            out[flag] = (cal, np.stack([ctx.avgdata(d) for d in range(ndir)]))
    finally:
        ctx.set_option(LEAP_OPTION_TENSOR_CORE_ROTATION, 1)
    cal_o, avg_o = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo, return_avg=True)
    scale = np.abs(obs.vis).sum(axis=0).reshape(timesteps, obs.nbaselines, 4).sum(axis=0)
    for flag in (1, 0):
        cal, avg = out[flag]
        err = np.abs(avg - avg_o) / np.maximum(scale, 1e-30)[None]
        assert err.max() < 2e-6, (flag, err.max())
        assert np.abs(cal - cal_o).max() <= MIXED_CAL_TOL, flag
    assert np.abs(out[1][0] - out[0][0]).max() <= 5 * TC_VS_CUDA_CORE_TOL
    ctx.release_integration(0)
