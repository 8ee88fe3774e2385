"""The device visibility generator used by the large benchmark workloads: the
noise-free cube equals the host model of the same observation, and the noise
has the stated per-component variance sigma^2 / 2."""
import numpy as np
import pytest

from leap_gb300 import synth

pytestmark = pytest.mark.gpu


def test_device_model_matches_host_model():
    obs = synth.make_observation(synth.ArraySpec(20, 900.0), timesteps=3, channels=17, freq_start_hz=150e6,
                                 freq_inc_hz=40e3, noise_sigma=0.0, vis_dtype=np.complex64)
    got = synth.device_visibilities(obs, "cuda:0", seed=5).cpu().numpy()
    assert got.shape == obs.vis.shape and got.dtype == np.complex64
    assert np.abs(got - obs.vis).max() < 2e-6


def test_device_noise_statistics_and_determinism():
    obs = synth.make_observation(synth.ArraySpec(24, 900.0), timesteps=4, channels=64, freq_start_hz=150e6,
                                 freq_inc_hz=40e3, noise_sigma=0.8, vis_dtype=np.complex64, with_vis=False)
    a = synth.device_visibilities(obs, "cuda:0", seed=9).cpu().numpy()
    b = synth.device_visibilities(obs, "cuda:0", seed=9).cpu().numpy()
    c = synth.device_visibilities(obs, "cuda:0", seed=10).cpu().numpy()
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    clean = synth.make_observation(synth.ArraySpec(24, 900.0), timesteps=4, channels=64, freq_start_hz=150e6,
                                   freq_inc_hz=40e3, noise_sigma=0.0, vis_dtype=np.complex64).vis
    noise = (a - clean).reshape(-1)
    n = noise.size
    for comp in (noise.real, noise.imag):
        assert abs(comp.mean()) < 5 * 0.8 / np.sqrt(2 * n)
        assert abs(comp.var() / (0.8 ** 2 / 2) - 1.0) < 0.02
