"""Parity of the CUDA path (through the C ABI) with the oracle.

Tolerances (the bars the calibration path is held to):
  * all-FP64 form: per-antenna cal phase within 1e-10 rad of the oracle, and
    avgData within 1e-11 relative (to the largest |avgData| of the direction);
  * mixed form: per-antenna cal phase within 1e-5 rad of the oracle.
A direction whose solve passes an arg() within the mixed form's error of +-pi may
come out on the other branch of that arg().  Such a direction passes only when the
oracle's own solve, with those angles moved to the other branch, is within the
tolerance of the result (oracle/branch_cuts.py); the count is reported.
"""
import numpy as np
import pytest

import oracle
import branch_cuts
import leap_gb300 as lg
from leap_gb300 import synth

pytestmark = pytest.mark.gpu

FP64_CAL_TOL = 1e-10
FP64_AVG_RTOL = 1e-11
MIXED_CAL_TOL = 1e-5
BRANCH_MARGIN = 1e-4  # angles this close to +-pi may take either branch in the mixed form


def _dds(md, dirs):
    return np.stack([lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs])


def run_case(ctx, obs, dirs, precision, slot=0):
    md = lg.build_metadata(obs)
    mdo = oracle.metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(slot, obs.vis, obs.uvw)
    dds = _dds(md, dirs)
    cal = ctx.calibrate(slot, dds, precision)
    cal_o, avg_o = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo, return_avg=True)
    return md, mdo, dds, cal, cal_o, avg_o


def assert_cal_close(cal, cal_o, avg_o, mdo, tol, margin=BRANCH_MARGIN):
    """Every direction within `tol` of the oracle, or within `tol` of the oracle's solve with
    some of its angles within `margin` of +-pi on the other branch.  Returns the number of
    directions that took another branch."""
    bad, flipped = [], 0
    for d in range(cal.shape[0]):
        err = float(np.abs(cal[d] - cal_o[d]).max())
        if err <= tol:
            continue
        ok, moved, rest = branch_cuts.explain(cal[d], avg_o[d][:, 0], mdo, tol, margin)
        if ok:
            flipped += 1
            print(f"direction {d}: {moved} angle(s) on the other branch, then within {rest:.2e} rad")
        else:
            bad.append((d, err, rest))
    assert not bad, f"directions over tolerance {tol} and not a branch choice: {bad[:5]}"
    return flipped


def test_plain_fp64_askap_small(ctx):
    """36 antennas, 1 timestep, 48 channels, complex<double>: the plain FP64 workload."""
    obs, dirs = synth.askap_small()
    md, mdo, dds, cal, cal_o, avg_o = run_case(ctx, obs, dirs, lg.LEAP_PRECISION_FP64)
    assert np.abs(cal - cal_o).max() <= FP64_CAL_TOL
    avg = ctx.avgdata(0)
    assert np.abs(avg - avg_o[0]).max() <= FP64_AVG_RTOL * np.abs(avg_o[0]).max()


@pytest.mark.parametrize("pols,dtype", [(4, np.complex128), (4, np.complex64), (2, np.complex128), (1, np.complex64)])
@pytest.mark.parametrize("stations,timesteps,channels,ndir", [(5, 1, 3, 1), (9, 3, 7, 5), (40, 2, 33, 19)])
def test_fp64_small_shapes(ctx, pols, dtype, stations, timesteps, channels, ndir):
    obs, dirs = synth.small_case(stations=stations, timesteps=timesteps, channels=channels, pols=pols,
                                 directions=ndir, vis_dtype=dtype, seed_shift=stations + channels)
    md, mdo, dds, cal, cal_o, avg_o = run_case(ctx, obs, dirs, lg.LEAP_PRECISION_FP64)
    assert np.abs(cal - cal_o).max() <= FP64_CAL_TOL
    for d in range(len(dirs)):
        avg = ctx.avgdata(d)
        assert np.abs(avg - avg_o[d]).max() <= FP64_AVG_RTOL * max(np.abs(avg_o[d]).max(), 1.0)


def test_fp64_nan_samples_are_skipped(ctx):
    """A NaN in any pol drops that (row, channel) from every pol (CpuLeapCalibrator.cc:201-214)."""
    obs, dirs = synth.small_case(stations=12, timesteps=3, channels=10, directions=4)
    rng = np.random.default_rng(7)
    vis = obs.vis.copy()
    idx = rng.integers(0, vis.size, 40)
    flat = vis.reshape(-1)
    flat[idx[:20]] = np.nan + 0j
    flat[idx[20:]] = complex(1.0, np.nan)
    obs.vis = vis
    md, mdo, dds, cal, cal_o, avg_o = run_case(ctx, obs, dirs, lg.LEAP_PRECISION_FP64)
    assert np.isfinite(cal).all()
    assert np.abs(cal - cal_o).max() <= FP64_CAL_TOL
    for d in range(len(dirs)):
        assert np.abs(ctx.avgdata(d) - avg_o[d]).max() <= FP64_AVG_RTOL * np.abs(avg_o[d]).max()


def test_fp64_slab_split_many_timesteps(ctx):
    """Enough (timestep, channel) work that the launch splits it into slabs."""
    obs, dirs = synth.small_case(stations=24, timesteps=9, channels=64, directions=3)
    md, mdo, dds, cal, cal_o, avg_o = run_case(ctx, obs, dirs, lg.LEAP_PRECISION_FP64)
    assert np.abs(cal - cal_o).max() <= FP64_CAL_TOL


def test_mixed_precision_reduced_mwa(ctx):
    """128 antennas, 2 timesteps, 96 channels, 24 directions in complex<float>."""
    obs, dirs = synth.mwa_precision(timesteps=2, channels=96, directions=24)
    md, mdo, dds, cal, cal_o, avg_o = run_case(ctx, obs, dirs, lg.LEAP_PRECISION_MIXED)
    assert_cal_close(cal, cal_o, avg_o, mdo, MIXED_CAL_TOL)


def test_mixed_precision_small_shapes(ctx):
    for pols, dtype in [(4, np.complex64), (1, np.complex64), (4, np.complex128)]:
        obs, dirs = synth.small_case(stations=20, timesteps=3, channels=40, pols=pols, directions=7, vis_dtype=dtype)
        md, mdo, dds, cal, cal_o, avg_o = run_case(ctx, obs, dirs, lg.LEAP_PRECISION_MIXED)
        assert_cal_close(cal, cal_o, avg_o, mdo, MIXED_CAL_TOL)


def test_rotate_uvw_matches_oracle(ctx):
    obs, dirs = synth.small_case(stations=10, timesteps=2, channels=2, directions=3)
    md = lg.build_metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(3, obs.vis, obs.uvw)
    dds = _dds(md, dirs)
    got = ctx.rotate_uvw(3, dds)
    for d in range(len(dirs)):
        exp = np.zeros_like(obs.uvw)
        oracle._load().oracle_rotate_uvw(oracle._ptr(np.ascontiguousarray(dds[d])), oracle._ptr(obs.uvw),
                                         obs.uvw.shape[0], oracle._ptr(exp))
        np.testing.assert_allclose(got[d], exp, rtol=0, atol=1e-9)
    ctx.release_integration(3)


@pytest.mark.parametrize("interval", [(0, 1, 1), (0, -1, -1), (0, 1, -1), (0, 2, -1)],
                         ids=["first_timestep", "all_timesteps", "each_timestep", "pairs"])
def test_calibrator_solution_intervals(interval):
    """ILeapCalibrator::Calibrate over solution intervals (PhaseRotateTests.cc:420-428 shapes)."""
    obs, dirs = synth.small_case(stations=16, timesteps=4, channels=12, directions=3)
    cal = lg.GpuLeapCalibrator(0, lg.LEAP_PRECISION_FP64)
    got = cal.calibrate(obs, dirs, interval)
    exp = oracle.calibrate(obs, dirs, interval)
    assert len(got) == len(exp) > 0
    for g, e in zip(got, exp):
        assert g["epoch"] == e["epoch"]
        for gb, eb in zip(g["calibration"], e["calibration"]):
            assert gb["direction"] == eb["direction"]
            assert np.abs(np.array(gb["beamCalibration"]) - np.array(eb["beamCalibration"])).max() <= FP64_CAL_TOL
    cal.ctx.close()


def test_repeat_calls_are_bit_identical(ctx):
    obs, dirs = synth.small_case(stations=30, timesteps=4, channels=50, directions=9, vis_dtype=np.complex64)
    md = lg.build_metadata(obs)
    ctx.set_metadata(md)
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = _dds(md, dirs)
    for prec in (lg.LEAP_PRECISION_FP64, lg.LEAP_PRECISION_MIXED):
        a = ctx.calibrate(0, dds, prec)
        b = ctx.calibrate(0, dds, prec)
        np.testing.assert_array_equal(a, b)


def test_error_paths(ctx):
    fresh = lg.Context(0)
    with pytest.raises(lg.LeapError):
        fresh.calibrate(0, np.eye(3)[None], lg.LEAP_PRECISION_FP64)  # no metadata
    obs, dirs = synth.small_case(stations=6, timesteps=1, channels=2, directions=1)
    fresh.set_metadata(lg.build_metadata(obs))
    with pytest.raises(lg.LeapError):
        fresh.calibrate(5, np.eye(3)[None], lg.LEAP_PRECISION_FP64)  # slot not set
    with pytest.raises(lg.InvalidArgument):
        fresh.set_integration(0, obs.vis[:, :, :3].copy(), obs.uvw)  # 3 pols unsupported
    fresh.set_integration(0, obs.vis, obs.uvw)
    with pytest.raises(lg.InvalidArgument):
        fresh.calibrate(0, np.eye(3)[None], 7)  # unknown precision
    fresh.close()


@pytest.mark.parametrize("stations,timesteps,channels,ndir", [(64, 9, 23, 40), (33, 5, 5, 3), (12, 20, 48, 70)])
def test_mixed_pipelined_edges(ctx, stations, timesteps, channels, ndir):
    """4-pol complex<float> shapes that hit partial 32-baseline tiles, partial
    16-channel chunks, several direction groups and several timestep slabs."""
    obs, dirs = synth.small_case(stations=stations, timesteps=timesteps, channels=channels, directions=ndir,
                                 vis_dtype=np.complex64, seed_shift=stations)
    md, mdo, dds, cal, cal_o, avg_o = run_case(ctx, obs, dirs, lg.LEAP_PRECISION_MIXED)
    assert_cal_close(cal, cal_o, avg_o, mdo, MIXED_CAL_TOL)
    # avgData of the bulk kernel (all pols) against the oracle, relative to the sum of |terms|
    scale = np.abs(obs.vis).sum(axis=0).reshape(timesteps, obs.nbaselines, 4).sum(axis=0)
    for d in range(0, ndir, max(1, ndir // 4)):
        err = np.abs(ctx.avgdata(d) - avg_o[d]) / np.maximum(scale, 1e-30)
        assert err.max() < 2e-6


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_mixed_reference_antenna_rows_are_near_fp64(ctx, dtype):
    """The reference-antenna baselines (pol 0), which the solve reads with weight
    one, are summed with compensated arithmetic: within 1e-9 of the FP64 sums,
    relative to the sum of |terms|."""
    obs, dirs = synth.small_case(stations=40, timesteps=6, channels=70, directions=9, vis_dtype=dtype, seed_shift=2)
    md, mdo, dds, cal, cal_o, avg_o = run_case(ctx, obs, dirs, lg.LEAP_PRECISION_MIXED)
    scale = np.abs(obs.vis[:, :, 0]).sum(axis=0).reshape(obs.timesteps, obs.nbaselines).sum(axis=0)
    for d in range(len(dirs)):
        got = ctx.avgdata(d)[mdo.I1, 0]
        err = np.abs(got - avg_o[d][mdo.I1, 0]) / scale[mdo.I1]
        assert err.max() < 1e-9, (d, err.max())


def test_bounded_wait_timeout_is_reported_and_context_survives(ctx):
    """Failure detection without a fault: a wait that nothing completes gives up after a
    bounded number of polls, the host reads LEAP_ERR_DEVICE_TIMEOUT, and the next call works."""
    from leap_gb300 import _abi
    assert _abi.lib.leap_selftest_bounded_wait(ctx.handle, 1000) == _abi.LEAP_ERR_DEVICE_TIMEOUT
    obs, dirs = synth.small_case(stations=8, timesteps=1, channels=4, directions=2)
    md, mdo, dds, cal, cal_o, avg_o = run_case(ctx, obs, dirs, lg.LEAP_PRECISION_FP64)
    assert np.abs(cal - cal_o).max() <= FP64_CAL_TOL
