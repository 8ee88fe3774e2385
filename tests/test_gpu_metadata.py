"""MetaData build on the device (leap_build_metadata): A / I / A1 / I1 as
PhaseMatrixFunction builds them and both pseudo-inverses on the GPU, against
the host build (exact integer Gram matrix + Jacobi + refinement, itself pinned
to numpy's SVD pseudo-inverse on the CPU)."""
import time

import numpy as np
import pytest

import oracle
import leap_gb300 as lg
from leap_gb300 import synth

pytestmark = pytest.mark.gpu


def _flag(obs, pairs):
    nbl = obs.nbaselines
    a1, a2 = obs.antenna1[:nbl], obs.antenna2[:nbl]
    for p, q in pairs:
        obs.flags[(a1 == p) & (a2 == q)] = 1


def _compare(md_dev, md_host, rtol=1e-12):
    for name in ("A", "I", "A1", "I1"):
        np.testing.assert_array_equal(getattr(md_dev, name), getattr(md_host, name))
    for name in ("Ad", "Ad1"):
        d, h = getattr(md_dev, name), getattr(md_host, name)
        assert d.shape == h.shape
        assert np.abs(d - h).max() <= rtol * np.abs(h).max(), (name, np.abs(d - h).max())


@pytest.mark.parametrize("stations,flag_fraction", [(12, 0.0), (40, 0.1), (128, 0.02)])
def test_device_pinv_matches_host(ctx, stations, flag_fraction):
    obs, dirs = synth.small_case(stations=stations, timesteps=2, channels=4, directions=3, vis_dtype=np.complex64,
                                 seed_shift=stations)
    rng = np.random.default_rng(stations)
    nbl = obs.nbaselines
    cross = np.nonzero(obs.antenna1[:nbl] != obs.antenna2[:nbl])[0]
    refant = obs.total_antennas - 1
    keep_ref = (obs.antenna1[:nbl] != refant) & (obs.antenna2[:nbl] != refant)
    pick = rng.choice(cross[keep_ref[cross]], int(flag_fraction * cross.size), replace=False) if flag_fraction else []
    obs.flags[pick] = 1
    md_host = lg.build_metadata(obs)
    md_dev = ctx.build_metadata(obs)
    assert md_dev.host_path == 0
    _compare(md_dev, md_host)
    # and the calibration through the device-built metadata against the oracle
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = np.stack([lg.dd_matrix(obs.phase_centre[0], obs.phase_centre[1], r, d) for r, d in dirs])
    cal = ctx.calibrate(0, dds, lg.LEAP_PRECISION_FP64)
    exp = oracle.calibrate_interval(obs.vis, obs.uvw, dds, oracle.metadata(obs))
    assert np.abs(cal - exp).max() <= 1e-10


def test_disconnected_array_takes_the_host_path(ctx):
    """Baselines between two halves of the array all flagged: A^T A is singular, the device
    build hands over to the SVD-style host path and gives the host result exactly."""
    obs, _ = synth.small_case(stations=10, timesteps=1, channels=2, directions=1, seed_shift=1)
    _flag(obs, [(p, q) for p in range(5) for q in range(5, 10)])
    # refAnt 2: the reference checks the flag of baseline number refAnt, here (0, 2), unflagged
    md_host = lg.build_metadata(obs, reference_antenna=2)
    md_dev = ctx.build_metadata(obs, reference_antenna=2)
    assert md_dev.host_path == 1  # A singular (antennas 5-9 float free); A1 is a star around antenna 2
    _compare(md_dev, md_host, rtol=1e-12)


def test_unused_antenna_columns_are_zero(ctx):
    """Antennas with every baseline flagged get exact zero rows of Ad (as the SVD gives)."""
    obs, _ = synth.small_case(stations=16, timesteps=1, channels=2, directions=1, seed_shift=2)
    _flag(obs, [(p, 3) for p in range(3)] + [(3, q) for q in range(4, 16)])
    md_dev = ctx.build_metadata(obs)
    assert md_dev.host_path == 0
    assert np.all(md_dev.Ad[3] == 0.0)
    _compare(md_dev, lg.build_metadata(obs))


def test_ska_low_metadata_build_time(ctx):
    """512 stations (130,817 x 512 phase matrix): device build against the host build."""
    obs, _ = synth.ska_low(with_vis=False, timesteps=1, channels=2, directions=1)
    t0 = time.perf_counter()
    ctx.build_metadata(obs, fetch=False)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    md_host = lg.build_metadata(obs)
    t_host = time.perf_counter() - t0
    print(f"SKA-Low metadata: device {t_dev:.3f} s, host {t_host:.3f} s")
    md_dev = ctx.build_metadata(obs)
    _compare(md_dev, md_host, rtol=1e-11)
    assert t_dev < t_host
