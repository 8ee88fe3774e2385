"""Batched calibration over integration chunks of uneven timestep and channel
counts (leap_calibrate_batched): every direction's cal phases equal the
oracle's for its own chunk (FP64 form within 1e-10 rad, mixed within 1e-5 rad);
a repeated call replays the recorded CUDA graph and returns identical bits."""
import numpy as np
import pytest

import oracle
import leap_gb300 as lg
from leap_gb300 import synth

pytestmark = pytest.mark.gpu


def make_chunks(stations, shapes, seed=0):
    """shapes: [(timesteps, channels, ndirections)]; same array, consecutive timesteps."""
    spec = synth.ArraySpec(stations, 1200.0)
    pos = synth.antenna_positions(spec, 40 + seed)
    gains = np.exp(1j * np.random.default_rng(41 + seed).uniform(-np.pi, np.pi, stations))
    chunks, off, d0 = [], 0, 0
    for i, (T, C, nd) in enumerate(shapes):
        obs = synth.make_observation(spec, timesteps=T, channels=C, freq_start_hz=150e6, freq_inc_hz=40e3,
                                     noise_sigma=0.5, source_lm=(0.01, -0.005), vis_dtype=np.complex64,
                                     seeds=(40 + seed, 41 + seed, 100 + i), timestep_offset=off, positions=pos,
                                     gains=gains)
        dirs, _ = synth.random_directions(nd, seed=200 + i)
        chunks.append((obs, dirs, d0))
        off += T
        d0 += nd
    return chunks


@pytest.mark.parametrize("shapes", [
    [(3, 48, 8), (1, 96, 8), (5, 20, 8), (2, 48, 8)],          # 8 directions per chunk (c3 shape)
    [(2, 40, 11), (4, 17, 3), (1, 64, 36)],                      # uneven direction counts
])
@pytest.mark.parametrize("precision,tol", [(lg.LEAP_PRECISION_MIXED, 1e-5), (lg.LEAP_PRECISION_FP64, 1e-10)])
def test_batched_matches_oracle_per_chunk(ctx, shapes, precision, tol):
    chunks = make_chunks(40, shapes)
    md = lg.build_metadata(chunks[0][0])
    mdo = oracle.metadata(chunks[0][0])
    ctx.set_metadata(md)
    items, dds = [], []
    for slot, (obs, dirs, d0) in enumerate(chunks):
        ctx.set_integration(slot, obs.vis, obs.uvw)
        items.append((slot, d0, len(dirs)))
        dds += [lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs]
    dds = np.stack(dds)
    cal = ctx.calibrate_batched(items, dds, precision)
    for slot, (obs, dirs, d0) in enumerate(chunks):
        exp = oracle.calibrate_interval(obs.vis, obs.uvw, dds[d0:d0 + len(dirs)], mdo)
        err = np.abs(cal[d0:d0 + len(dirs)] - exp).max()
        assert err <= tol, (slot, err)
    again = ctx.calibrate_batched(items, dds, precision)  # replays the graph
    np.testing.assert_array_equal(cal, again)
    for slot in range(len(chunks)):
        ctx.release_integration(slot)


def test_batched_rejects_bad_items(ctx):
    obs, dirs = synth.small_case(stations=8, timesteps=1, channels=4, directions=2)
    ctx.set_metadata(lg.build_metadata(obs))
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = np.stack([np.eye(3)] * 2)
    with pytest.raises(lg.InvalidArgument):
        ctx.calibrate_batched([(0, 1, 2)], dds)  # directions past the end
    with pytest.raises(lg.LeapError):
        ctx.calibrate_batched([(9, 0, 2)], dds)  # slot not set
