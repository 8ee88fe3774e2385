"""ORACLE — test infrastructure only.

Proof that a calibration differs from the oracle's only by the branch of an arg().

The reference's solve (LA/algorithm/cpu/CpuLeapCalibrator.cc:159-178) takes two
sets of angles from avgData:

    phi1[k]  = arg(avg[I1[k], 0])                         k < |I1|   (:161-163)
    dInt[n]  = arg(exp(-2 pi i (A cal1)[n]) avg[n, 0])    n < |I|    (:168-172)

with cal1 = Ad1 (phi1 ++ [0]) and cal = Ad (dInt ++ [0]) + cal1.  An angle that
lies within a form's rounding error of +-pi can come out of another
implementation on the other side of the cut (theta - 2 pi instead of theta, or
the reverse).  That changes the result by a definite amount:

  * one dInt[n] on the other branch moves cal by -+2 pi Ad[:, n];
  * one phi1[k] on the other branch moves cal1 by -+2 pi Ad1[:, k], which
    re-phases every dInt (they then change by a non-integer amount) and so
    moves cal by 2 pi Ad1[:, k] + Ad delta(dInt).

``explain`` re-solves the oracle's own avgData with every such choice of branch
(each near-cut phi1 combination re-solved exactly, then near-cut dInt flips fitted
as integer multiples of 2 pi Ad[:, n]) and accepts a difference only when one of
these alternative solutions lies within the tolerance of the GPU result.  An
angle farther than ``margin`` from +-pi is never flipped, so a real error cannot
pass as a branch choice.

``solve`` restates the oracle's solve in numpy (FP64); ``tests/test_oracle_kats.py``
pins it to ``oracle.solve``.  Only tests and bench.py's parity checks import this.
"""
from __future__ import annotations

import itertools
from typing import Optional, Tuple

import numpy as np


def _i1_rows(mdo) -> np.ndarray:
    """I1 with the VectorRangeSelect wrap-around of negative indices (LA/math/cpu/vector.h:97-104)."""
    i1 = np.asarray(mdo.I1, dtype=np.int64)
    return np.where(i1 < 0, i1 + mdo.nbaselines, i1)


def angles(avg0: np.ndarray, mdo, phi1_shift: Optional[np.ndarray] = None):
    """(phi1 without the appended zero, cal1, dInt) of one direction from avgData column 0."""
    phi1 = np.angle(avg0[_i1_rows(mdo)])
    if phi1_shift is not None:
        phi1 = phi1 + phi1_shift
    cal1 = mdo.Ad1 @ np.append(phi1, 0.0)
    n = mdo.A.shape[0] - 1
    acal = mdo.A[:n] @ cal1
    dint = np.angle(np.exp(-2j * np.pi * acal) * avg0[:n])
    return phi1, cal1, dint


def solve(avg0: np.ndarray, mdo, phi1_shift: Optional[np.ndarray] = None,
          dint_shift: Optional[np.ndarray] = None) -> np.ndarray:
    """cal of one direction (the oracle's solve in numpy), optionally with angles moved by
    multiples of 2 pi (phi1_shift: |I1| entries, dint_shift: |I| entries)."""
    _, cal1, dint = angles(avg0, mdo, phi1_shift)
    if dint_shift is not None:
        dint = dint + dint_shift
    return mdo.Ad @ np.append(dint, 0.0) + cal1


def _other_branch(theta: np.ndarray) -> np.ndarray:
    """The shift that takes an angle to the other side of the +-pi cut."""
    return np.where(theta > 0, -2.0 * np.pi, 2.0 * np.pi)


def explain(cal: np.ndarray, avg0: np.ndarray, mdo, tol: float, margin: float,
            max_phi1_flips: int = 3) -> Tuple[bool, int, float]:
    """Whether `cal` (one direction) equals the oracle solve of `avg0` within `tol` after moving
    some of its near-cut angles (within `margin` of +-pi) to the other branch.

    Returns (explained, number of angles moved, remaining max |difference|)."""
    phi1, _, dint0 = angles(avg0, mdo)
    near_k = np.flatnonzero(np.pi - np.abs(phi1) < margin)
    best = (False, 0, np.inf)
    combos = []
    for r in range(0, min(len(near_k), max_phi1_flips) + 1):
        combos += list(itertools.combinations(near_k.tolist(), r))
    for ks in combos:
        shift1 = np.zeros_like(phi1)
        for k in ks:
            shift1[k] = _other_branch(phi1[k])
        _, cal1, dint = angles(avg0, mdo, shift1)
        base = mdo.Ad @ np.append(dint, 0.0) + cal1
        resid = cal - base
        err = float(np.abs(resid).max())
        if err <= tol:
            return True, len(ks), err
        near_n = np.flatnonzero(np.pi - np.abs(dint) < margin)
        if near_n.size:
            # cal - base = sum_n k_n * s_n * 2 pi Ad[:, n] with k_n in {0, 1} and s_n the shift direction.
            cols = mdo.Ad[:, near_n] * _other_branch(dint[near_n])[None, :]
            coef, *_ = np.linalg.lstsq(cols, resid, rcond=None)
            kint = np.clip(np.rint(coef), 0, 1)
            fit = resid - cols @ kint
            err2 = float(np.abs(fit).max())
            if err2 <= tol:
                return True, len(ks) + int(kint.sum()), err2
            err = min(err, err2)
        if err < best[2]:
            best = (False, 0, err)
    return best
