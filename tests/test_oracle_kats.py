"""Pin the oracle (and the library's host set-up maths) to the reference's own
known-answer tests, from tests/golden/reference_kats.json."""
import json
import os

import numpy as np
import pytest

import oracle
import leap_gb300 as lg

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def _dd_case():
    pc = KATS["dd"]["phase_centre"]
    d = KATS["dd"]["direction"]
    return pc, d, np.array(KATS["dd"]["expected"])


def test_dd_matrix_oracle_matches_reference_kat():
    # MetaDataTests.cc:155-165 asserts EXPECT_DOUBLE_EQ (4 ulps).
    pc, d, exp = _dd_case()
    got = oracle.dd_matrix(pc[0], pc[1], d[0], d[1])
    assert np.all(np.abs(got - exp) <= 4 * np.spacing(np.abs(exp)))


def test_dd_matrix_library_matches_reference_kat():
    pc, d, exp = _dd_case()
    got = lg.dd_matrix(pc[0], pc[1], d[0], d[1])
    assert np.all(np.abs(got - exp) <= 4 * np.spacing(np.abs(exp)))
    np.testing.assert_array_equal(got, oracle.dd_matrix(pc[0], pc[1], d[0], d[1]))


def test_dd_matrix_phase_rotate_kat_is_the_same():
    np.testing.assert_array_equal(np.array(KATS["dd"]["expected_phase_rotate_test"]), np.array(KATS["dd"]["expected"]))


def test_dlm_constants_kat():
    # PhaseRotateTests.cc:206-207: dlm = direction - phase centre (MetaData.cc:208-209).
    c = KATS["constants"]
    d = KATS["dd"]["direction"]
    assert d[0] - c["phase_centre_ra_rad"] == pytest.approx(c["dlm_ra"], abs=4 * np.spacing(abs(c["dlm_ra"])))
    assert d[1] - c["phase_centre_dec_rad"] == pytest.approx(c["dlm_dec"], abs=4 * np.spacing(abs(c["dlm_dec"])))


def test_channel_wavelength_kat():
    c = KATS["constants"]
    lam = oracle.channel_wavelength(c["freq_start_hz"], c["freq_inc_hz"], 0)
    assert lam == pytest.approx(KATS["wavelength0"], abs=4 * np.spacing(KATS["wavelength0"]))


@pytest.mark.parametrize("case", KATS["pinv"], ids=lambda c: c["name"])
def test_pseudo_inverse_kats(case):
    A = np.array(case["A"], dtype=np.float64)
    exp = np.array(case["expected"])
    tol = KATS["pinv_tolerance"]
    for got in (oracle.pseudo_inverse(A), lg.pseudo_inverse(A)):
        np.testing.assert_allclose(got, exp, atol=tol)
        np.testing.assert_allclose(A @ got @ A, A, atol=tol)


def test_pseudo_inverse_library_matches_oracle_on_random_full_rank():
    rng = np.random.default_rng(0)
    for m, n in [(7, 3), (12, 12), (40, 9)]:
        A = rng.standard_normal((m, n))
        np.testing.assert_allclose(lg.pseudo_inverse(A), oracle.pseudo_inverse(A), atol=1e-12)


def test_phase_matrix_empty_input_throws():
    # PhaseRotateTests.cc:248-274
    with pytest.raises(oracle.InvalidArgument):
        oracle.phase_matrix([], [], [], KATS["phase_matrix_empty_input_throws"]["refAnt"])
    with pytest.raises(lg.InvalidArgument):
        lg.phase_matrix([], [], [], KATS["phase_matrix_empty_input_throws"]["refAnt"])


def _toy_baselines(n_ant=6, autos=True):
    a1, a2 = [], []
    for a in range(n_ant):
        for b in range(a if autos else a + 1, n_ant):
            a1.append(a)
            a2.append(b)
    return np.array(a1, np.int32), np.array(a2, np.int32)


def test_phase_matrix_structure_and_ref_row():
    a1, a2 = _toy_baselines(6)
    fg = (a1 == a2).astype(np.uint8)
    fg[3] = 1  # one flagged cross baseline
    # refAnt 0 would be "flagged": the reference checks fg[refAnt], i.e. the flag
    # of the baseline whose index is refAnt (here the flagged autocorrelation (0, 0)).
    for mod in (oracle, lg):
        with pytest.raises(mod.InvalidArgument):
            mod.phase_matrix(a1, a2, fg, 0)
    for ref in (None, 1, 5):
        A, I = oracle.phase_matrix(a1, a2, fg, ref)
        A2, I2 = lg.phase_matrix(a1, a2, fg, ref)
        np.testing.assert_array_equal(A, A2)
        np.testing.assert_array_equal(I, I2)
        assert A.shape[1] == 6
        last = A[-1]
        assert last[0 if ref is None else ref] == 1 and np.count_nonzero(last) == 1
        for k, n in enumerate(I):
            assert a1[n] != a2[n] and not fg[n]
            assert A[k, a1[n]] == 1 and A[k, a2[n]] == -1
            if ref is not None:
                assert ref in (a1[n], a2[n])


def test_phase_matrix_ref_errors():
    a1, a2 = _toy_baselines(4)
    fg = np.zeros(a1.size, np.uint8)
    fg[2] = 1
    # refAnt out of bounds (>= number of baselines) and refAnt "flagged"
    # (the reference indexes the per-baseline flags with the antenna number).
    for mod in (oracle, lg):
        with pytest.raises(mod.InvalidArgument):
            mod.phase_matrix(a1, a2, fg, a1.size)
        with pytest.raises(mod.InvalidArgument):
            mod.phase_matrix(a1, a2, fg, 2)


def test_metadata_reference_antenna_default_and_rows():
    # MetaDataTests.cc:189-212 (TestReferenceAntenna) on a synthetic array.
    from leap_gb300 import synth
    obs, _ = synth.small_case(stations=6, timesteps=1, channels=2)
    for md in (oracle.metadata(obs), lg.build_metadata(obs)):
        k = md.A1.shape[0] - 1
        n = md.A1.shape[1] - 1
        assert md.reference_antenna == obs.total_antennas - 1
        assert md.A1[k, 0] == 0 and md.A1[k, n] == 1
    for ref, col in ((1, 1), (2, 2)):
        md = lg.build_metadata(obs, reference_antenna=ref)
        k = md.A1.shape[0] - 1
        assert md.A1[k, col] == 1 and np.count_nonzero(md.A1[k]) == 1


def test_pinv_identity_properties_synthetic():
    # PhaseMatrixFunctionDataTest: A * Ad * A == A (PhaseRotateTests.cc:368,409).
    from leap_gb300 import synth
    obs, _ = synth.askap_small(with_vis=False)
    md = lg.build_metadata(obs)
    mdo = oracle.metadata(obs)
    np.testing.assert_allclose(md.A @ md.Ad @ md.A, md.A, atol=1e-12)
    np.testing.assert_allclose(md.A1 @ md.Ad1 @ md.A1, md.A1, atol=1e-12)
    np.testing.assert_allclose(md.Ad, mdo.Ad, atol=1e-12)
    np.testing.assert_allclose(md.Ad1, mdo.Ad1, atol=1e-12)


def _exact_phase_pinv(A: np.ndarray) -> np.ndarray:
    """(A^T A)^-1 A^T in exact rational arithmetic, rounded once to FP64."""
    import sympy
    Am = sympy.Matrix(A.astype(int).tolist())
    X = (Am.T * Am).inv() * Am.T
    return np.array([[float(X[i, j]) for j in range(X.shape[1])] for i in range(X.shape[0])])


@pytest.mark.parametrize("stations,keep,ref", [(9, 0.7, 0), (11, 0.85, None), (13, 0.6, None)])
def test_oracle_pinv_of_phase_matrix_is_exact(stations, keep, ref):
    # Full-column-rank phase matrices (0 / +-1 entries) of arrays whose station counts are
    # not powers of two, with flagged baselines: the oracle's pinv must not depend on the
    # LAPACK build, so it equals the exact pinv to within a few ulp of its largest entry,
    # as does the library's.
    rng = np.random.default_rng(stations)
    a1, a2 = np.triu_indices(stations, 1)
    fg = rng.random(a1.size) > keep
    fg[:stations - 1] = False  # every station keeps a baseline
    A, _ = oracle.phase_matrix(a1, a2, fg, ref)
    exact = _exact_phase_pinv(A)
    scale = np.abs(exact).max()
    for got in (oracle.pseudo_inverse(A), lg.pseudo_inverse(A)):
        assert np.abs(got - exact).max() <= 4 * np.finfo(np.float64).eps * scale
