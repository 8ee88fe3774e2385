"""The branch-cut proof used by the mixed-form parity checks (oracle/branch_cuts.py),
exercised on the CPU with differences planted in oracle results.

* its numpy solve equals the oracle's C solve;
* a result with one dInt angle, or one reference-antenna angle, moved to the other
  side of +-pi is explained as a branch choice, with the number of angles moved;
* a result that differs by anything else (a small error, or a flip of an angle
  that is not near the cut) is not explained.
"""
import numpy as np
import pytest

import oracle
import branch_cuts
from leap_gb300 import synth


def _case(seed_shift=0, stations=24, ndir=6):
    obs, dirs = synth.small_case(stations=stations, timesteps=2, channels=12, directions=ndir, seed_shift=seed_shift)
    mdo = oracle.metadata(obs)
    dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs])
    cal, avg = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo, return_avg=True)
    return mdo, cal, avg


@pytest.mark.parametrize("seed_shift", [0, 3, 9])
def test_numpy_solve_equals_oracle_solve(seed_shift):
    mdo, cal, avg = _case(seed_shift)
    for d in range(cal.shape[0]):
        np.testing.assert_allclose(branch_cuts.solve(avg[d][:, 0], mdo), cal[d], rtol=0, atol=1e-12)
        np.testing.assert_allclose(branch_cuts.solve(avg[d][:, 0], mdo), oracle.solve(avg[d], mdo), rtol=0, atol=1e-12)


def test_identical_result_needs_no_flip():
    mdo, cal, avg = _case()
    ok, moved, err = branch_cuts.explain(cal[0], avg[0][:, 0], mdo, 1e-5, 1e-4)
    assert ok and moved == 0 and err < 1e-12


def test_dint_flip_is_explained_only_inside_the_margin():
    mdo, cal, avg = _case()
    avg0 = avg[0][:, 0]
    _, _, dint = branch_cuts.angles(avg0, mdo)
    n = int(np.argmax(np.abs(dint)))            # the dInt angle closest to +-pi
    dist = np.pi - abs(dint[n])
    shift = np.zeros_like(dint)
    shift[n] = -2 * np.pi if dint[n] > 0 else 2 * np.pi
    flipped = branch_cuts.solve(avg0, mdo, dint_shift=shift)
    np.testing.assert_allclose(flipped - cal[0], shift[n] * mdo.Ad[:, n], atol=1e-12)
    ok, moved, _ = branch_cuts.explain(flipped, avg0, mdo, 1e-5, dist * 1.01)
    assert ok and moved == 1
    # The same flip with a margin that does not reach that angle is an error.
    ok, _, err = branch_cuts.explain(flipped, avg0, mdo, 1e-5, dist * 0.99)
    assert not ok and err > 1e-3
    # A flip plus a small real error is not explained either.
    ok, _, _ = branch_cuts.explain(flipped + 5e-5, avg0, mdo, 1e-5, dist * 1.01)
    assert not ok


def test_two_dint_flips_are_explained():
    mdo, cal, avg = _case(seed_shift=3)
    avg0 = avg[1][:, 0]
    _, _, dint = branch_cuts.angles(avg0, mdo)
    top = np.argsort(-np.abs(dint))[:2]
    shift = np.zeros_like(dint)
    shift[top] = np.where(dint[top] > 0, -2 * np.pi, 2 * np.pi)
    flipped = branch_cuts.solve(avg0, mdo, dint_shift=shift)
    margin = (np.pi - np.abs(dint[top])).max() * 1.01
    ok, moved, _ = branch_cuts.explain(flipped, avg0, mdo, 1e-5, margin)
    assert ok and moved == 2


def test_reference_antenna_flip_is_re_solved():
    mdo, cal, avg = _case(seed_shift=9)
    avg0 = avg[2][:, 0]
    phi1, _, _ = branch_cuts.angles(avg0, mdo)
    k = int(np.argmax(np.abs(phi1)))
    shift = np.zeros_like(phi1)
    shift[k] = -2 * np.pi if phi1[k] > 0 else 2 * np.pi
    flipped = branch_cuts.solve(avg0, mdo, phi1_shift=shift)
    # Not a multiple of one column: every dInt is re-phased.
    assert np.abs(flipped - cal[2] - shift[k] * mdo.Ad1[:, k]).max() > 1e-3
    dist = np.pi - abs(phi1[k])
    ok, moved, _ = branch_cuts.explain(flipped, avg0, mdo, 1e-5, dist * 1.01)
    assert ok and moved >= 1
    ok, _, _ = branch_cuts.explain(flipped, avg0, mdo, 1e-5, dist * 0.99)
    assert not ok


def test_small_error_is_not_explained():
    mdo, cal, avg = _case()
    rng = np.random.default_rng(0)
    bad = cal[3] + rng.uniform(-3e-5, 3e-5, cal.shape[1])
    ok, moved, err = branch_cuts.explain(bad, avg[3][:, 0], mdo, 1e-5, np.pi)
    assert not ok
