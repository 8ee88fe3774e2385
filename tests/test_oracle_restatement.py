"""Cross-check the C oracle against an independent vectorised numpy restatement
of the same reference loops (CpuLeapCalibrator.cc:147-217)."""
import numpy as np
import pytest

import oracle
from leap_gb300 import synth


def numpy_rotate(vis, uvw, dd, nbl, f0, df):
    C, rows, P = vis.shape
    wrot = uvw @ dd[2]
    shift = -2.0 * np.pi * (wrot - uvw[:, 2])                      # [rows]
    lam = oracle.SPEED_OF_LIGHT / (f0 + np.arange(C) * df)         # [C]
    ph = np.exp(1j * (shift[None, :] / lam[:, None]))              # [C, rows]
    rot = vis.astype(np.complex128) * ph[:, :, None]
    ok = ~np.isnan(rot.real).any(axis=2) & ~np.isnan(rot.imag).any(axis=2)
    rot = np.where(ok[:, :, None], rot, 0)
    s = rot.sum(axis=0)                                            # [rows, P]
    return s.reshape(rows // nbl, nbl, P).sum(axis=0)


def numpy_solve(avg, md):
    phi1 = np.append(np.angle(avg[md.I1, 0]), 0.0)
    cal1 = md.Ad1 @ phi1
    acal = md.A @ cal1
    n = md.I.size
    dint = np.angle(np.exp(-2j * np.pi * acal[:n]) * avg[:n, 0])
    return md.Ad @ np.append(dint, 0.0) + cal1


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_oracle_matches_numpy_restatement(dtype):
    obs, dirs = synth.small_case(stations=10, timesteps=3, channels=9, directions=3, vis_dtype=dtype)
    vis = obs.vis.copy()
    vis.reshape(-1)[[5, 77, 300]] = np.nan
    md = oracle.metadata(obs)
    dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs])
    cal, avg = oracle.calibrate_interval(vis, obs.uvw, dds, md, return_avg=True)
    for d in range(len(dirs)):
        a = numpy_rotate(vis, obs.uvw, dds[d], obs.nbaselines, obs.freq_start_hz, obs.freq_inc_hz)
        np.testing.assert_allclose(avg[d], a, rtol=0, atol=1e-11 * np.abs(a).max())
        np.testing.assert_allclose(cal[d], numpy_solve(avg[d], md), rtol=0, atol=1e-12)


def test_dd_third_row_is_lmn():
    for lm in [(0.01, -0.005), (-0.04, 0.03), (0.0, 0.0)]:
        rd = synth.lm_to_radec(np.array([lm[0]]), np.array([lm[1]]))[0]
        dd = oracle.dd_matrix(*synth.PHASE_CENTRE, rd[0], rd[1])
        n = np.sqrt(1 - lm[0] ** 2 - lm[1] ** 2)
        np.testing.assert_allclose(dd[2], [lm[0], lm[1], n], atol=1e-14)


def test_calibrate_items_equals_per_interval_calls():
    """oracle.calibrate_items (one host task per (chunk, direction)) gives exactly the
    results of calibrate_interval chunk by chunk."""
    import oracle
    from leap_gb300 import synth
    obs, dirs = synth.small_case(stations=12, timesteps=3, channels=9, directions=5, vis_dtype=np.complex64)
    mdo = oracle.metadata(obs)
    dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs])
    nbl = obs.nbaselines
    parts = [(slice(0, nbl), slice(0, 2)), (slice(nbl, 3 * nbl), slice(2, 5))]
    chunks = [(obs.vis[:, r], obs.uvw[r], dds[d]) for r, d in parts]
    cals, avgs = oracle.calibrate_items(chunks, mdo, nthreads=3, return_avg=True)
    for (vis, uvw, dd), cal, avg in zip(chunks, cals, avgs):
        exp, exp_avg = oracle.calibrate_interval(vis, uvw, dd, mdo, return_avg=True)
        np.testing.assert_array_equal(cal, exp)
        np.testing.assert_array_equal(avg, exp_avg)
