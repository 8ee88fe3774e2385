"""Gridded rotate + average (LEAP_OPTION_GRIDDED_ROTATION): the channel sum of every
(row, pol) evaluated at each direction's phase slope through a 2x-oversampled grid,
the grid values as one 3xFP16 tcgen05 product per tile (scaled FP16 hi/lo splits).

Bars, as for the other mixed-form kernels: avgData within 2e-6 of the oracle's
FP64 sums relative to the sum of |terms| of each (baseline, pol); per-antenna cal
phase within 1e-5 rad of the oracle, or of the oracle's solve with angles within
1e-4 rad of +-pi on the other branch (proved per direction, as in the other parity
tests).
"""
import numpy as np
import pytest

import oracle
import leap_gb300 as lg
from leap_gb300 import synth
from leap_gb300._abi import LEAP_OPTION_GRIDDED_ROTATION, LEAP_OPTION_GRID_SHARED_GROUPS
from test_gpu_parity import MIXED_CAL_TOL, _dds, assert_cal_close

pytestmark = pytest.mark.gpu

AVG_TOL = 2e-6


def _gridded(ctx, fn):
    ctx.set_option(LEAP_OPTION_GRIDDED_ROTATION, 1)
    try:
        return fn()
    finally:
        ctx.set_option(LEAP_OPTION_GRIDDED_ROTATION, 2)


def _scale(obs):
    return np.abs(obs.vis).sum(axis=0).reshape(obs.timesteps, obs.nbaselines, obs.pols).sum(axis=0)


def _check(ctx, obs, dirs, avg_tol=AVG_TOL):
    md = lg.build_metadata(obs)
    mdo = oracle.metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = _dds(md, dirs)

    def run():
        cal = ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED)
        return cal, np.stack([ctx.avgdata(d) for d in range(len(dirs))])

    cal, avg = _gridded(ctx, run)
    cal_o, avg_o = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo, return_avg=True)
    err = np.abs(avg - avg_o) / np.maximum(_scale(obs), 1e-30)[None]
    assert np.isfinite(cal).all()
    assert err.max() < avg_tol, err.max()
    assert_cal_close(cal, cal_o, avg_o, mdo, MIXED_CAL_TOL)
    ctx.release_integration(0)
    return cal, cal_o


@pytest.mark.parametrize("stations,timesteps,channels,ndir", [
    (64, 9, 23, 40),    # partial quads of timesteps, partial 16-channel chunk
    (33, 5, 5, 3),      # nbl % 4 != 0, fewer channels than a chunk
    (12, 20, 48, 70),   # two direction groups, several timestep slabs
    (128, 2, 96, 64),   # one full direction group
    (40, 7, 70, 9),
    (24, 6, 200, 36),   # 13 chunks: three full 64-channel segments (middle folds), a last one of one chunk
])
def test_gridded_matches_oracle(ctx, stations, timesteps, channels, ndir):
    obs, dirs = synth.small_case(stations=stations, timesteps=timesteps, channels=channels, directions=ndir,
                                 vis_dtype=np.complex64, seed_shift=stations + 7)
    _check(ctx, obs, dirs)


def test_gridded_multi_pass_windows(ctx):
    """384 channels of 250 kHz on an 800 m array: the grid window of a unit spans
    more than one 64-point pass."""
    obs, dirs = synth.small_case(stations=16, timesteps=6, channels=384, directions=20, vis_dtype=np.complex64,
                                 seed_shift=5)
    _check(ctx, obs, dirs)


def test_gridded_uneven_timesteps_use_separate_loads(ctx):
    """UVWs that jump between neighbouring timesteps: the 4 timesteps of a baseline no
    longer share one grid window, so each loads its own (and windows need several
    passes)."""
    obs, dirs = synth.small_case(stations=20, timesteps=8, channels=96, directions=12, vis_dtype=np.complex64,
                                 seed_shift=9)
    rng = np.random.default_rng(3)
    obs.uvw = obs.uvw * rng.uniform(0.2, 3.0, size=(obs.uvw.shape[0], 1))
    _check(ctx, obs, dirs)


def test_gridded_nan_samples_are_skipped(ctx):
    obs, dirs = synth.small_case(stations=24, timesteps=5, channels=40, directions=10, vis_dtype=np.complex64,
                                 seed_shift=4)
    rng = np.random.default_rng(8)
    idx = rng.integers(0, obs.vis.size // 4, size=300)
    flat = obs.vis.reshape(-1, 4)
    flat[idx, rng.integers(0, 4, size=idx.size)] = np.nan
    md = lg.build_metadata(obs)
    mdo = oracle.metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = _dds(md, dirs)
    cal = _gridded(ctx, lambda: ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED))
    cal_o, avg_o = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo, return_avg=True)
    assert np.isfinite(cal).all()
    assert_cal_close(cal, cal_o, avg_o, mdo, MIXED_CAL_TOL)
    ctx.release_integration(0)


def test_gridded_agrees_with_pipelined_kernel(ctx):
    """Same inputs through the gridded and the FP32 CUDA-core kernels."""
    obs, dirs = synth.small_case(stations=48, timesteps=8, channels=64, directions=24, vis_dtype=np.complex64,
                                 seed_shift=11)
    md = lg.build_metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = _dds(md, dirs)
    ctx.set_option(LEAP_OPTION_GRIDDED_ROTATION, 0)
    ref = ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED)
    got = _gridded(ctx, lambda: ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED))
    assert np.abs(got - ref).max() <= 2 * MIXED_CAL_TOL
    ctx.release_integration(0)


def test_gridded_batched_graph(ctx):
    """Uneven chunks through leap_calibrate_batched (eager run, then the captured graph)."""
    from test_gpu_batched import make_chunks
    chunks = make_chunks(48, [(2, 30, 40), (1, 50, 9), (3, 12, 100), (5, 3, 16)], seed=6)
    md = lg.build_metadata(chunks[0][0])
    mdo = oracle.metadata(chunks[0][0])
    ctx.set_metadata(md)
    items, dds = [], []
    for slot, (obs, dirs, d0) in enumerate(chunks):
        ctx.set_integration(slot, obs.vis, obs.uvw)
        items.append((slot, d0, len(dirs)))
        dds += [lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs]
    dds = np.stack(dds)
    ctx.set_option(LEAP_OPTION_GRIDDED_ROTATION, 1)
    try:
        cal = ctx.calibrate_batched(items, dds, lg.LEAP_PRECISION_MIXED)
        again = ctx.calibrate_batched(items, dds, lg.LEAP_PRECISION_MIXED)
    finally:
        ctx.set_option(LEAP_OPTION_GRIDDED_ROTATION, 2)
    for slot, (obs, dirs, d0) in enumerate(chunks):
        exp, avg_o = oracle.calibrate_interval(obs.vis, obs.uvw, dds[d0:d0 + len(dirs)], mdo, return_avg=True)
        assert_cal_close(cal[d0:d0 + len(dirs)], exp, avg_o, mdo, MIXED_CAL_TOL)
    np.testing.assert_array_equal(cal, again)
    for slot in range(len(chunks)):
        ctx.release_integration(slot)


def test_gridded_option_is_validated(ctx):
    with pytest.raises(lg.InvalidArgument):
        ctx.set_option(LEAP_OPTION_GRIDDED_ROTATION, 3)


def test_gridded_auto_selection(ctx):
    """Default (auto): items of >= 32 directions take the gridded kernel, fewer the
    pipelined one; both agree with the oracle."""
    obs, dirs = synth.small_case(stations=40, timesteps=6, channels=48, directions=40, vis_dtype=np.complex64,
                                 seed_shift=21)
    md = lg.build_metadata(obs)
    mdo = oracle.metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = _dds(md, dirs)
    cal_o, avg_o = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo, return_avg=True)
    for nd in (40, 8):
        cal = ctx.calibrate(0, dds[:nd], lg.LEAP_PRECISION_MIXED)
        assert_cal_close(cal, cal_o[:nd], avg_o[:nd], mdo, MIXED_CAL_TOL)
    ctx.release_integration(0)


@pytest.mark.parametrize("shared", [0, 1], ids=["group_per_unit", "one_product_for_all_groups"])
def test_gridded_direction_groups(ctx, shared):
    """130 directions: three groups of up to 64, each with its own grid product, or all served
    by one product per tile (one-tile units whose sums the slab reduction adds)."""
    obs, dirs = synth.small_case(stations=20, timesteps=9, channels=40, directions=130, vis_dtype=np.complex64,
                                 seed_shift=31)
    ctx.set_option(LEAP_OPTION_GRID_SHARED_GROUPS, shared)
    try:
        _check(ctx, obs, dirs)
    finally:
        ctx.set_option(LEAP_OPTION_GRID_SHARED_GROUPS, 0)


def test_gridded_long_integration_bright_source(ctx):
    """47 timesteps x 384 channels of the 128-antenna array with a bright source, 8 of the
    batched workload's directions: the stencil and accumulation errors of the source's fringe
    add coherently over the timesteps, while the averages of directions away from the source
    do not (with 8-point stencils a chunk of this shape reached 2e-5 rad)."""
    spec = synth.ArraySpec(128, 1500.0)
    obs = synth.make_observation(spec, timesteps=47, channels=384, freq_start_hz=150e6, freq_inc_hz=40e3,
                                 noise_sigma=0.5, source_lm=(0.01, -0.005), vis_dtype=np.complex64,
                                 positions=synth.antenna_positions(spec, 0), seeds=(0, 1, 2))
    dirs, _ = synth.random_directions(256)
    _check(ctx, obs, dirs[::32])
