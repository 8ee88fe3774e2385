"""MeasurementSet-order ingestion on the device (leap_set_integration_ms): the
resident integration equals the one uploaded in the Integration layout, so
calibrating either gives bit-identical cal phases.  Covers pageable host
memory (staged in pieces), pinned host memory and device memory (read
directly by the transpose kernel), channel subsets, NaN groups, complex<float>
and complex<double>, 1/2/4 pols."""
import numpy as np
import pytest
import torch

import leap_gb300 as lg
from leap_gb300 import synth

pytestmark = pytest.mark.gpu


def _dds(md, dirs):
    return np.stack([lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs])


def _reference(ctx, obs, dds, precision):
    ctx.set_integration(0, obs.vis, obs.uvw)
    return ctx.calibrate(0, dds, precision)


@pytest.mark.parametrize("source", ["pageable", "pinned", "device"])
@pytest.mark.parametrize("dtype,pols", [(np.complex64, 4), (np.complex128, 4), (np.complex64, 2), (np.complex64, 1)])
def test_ms_order_upload_matches(ctx, source, dtype, pols):
    obs, dirs = synth.small_case(stations=30, timesteps=3, channels=37, pols=pols, directions=5, vis_dtype=dtype,
                                 seed_shift=9)
    flat = obs.vis.reshape(-1)
    flat[np.random.default_rng(2).integers(0, flat.size, 25)] = np.nan
    md = lg.build_metadata(obs)
    ctx.set_metadata(md)
    dds = _dds(md, dirs)
    prec = lg.LEAP_PRECISION_MIXED if dtype == np.complex64 and pols == 4 else lg.LEAP_PRECISION_FP64
    exp = _reference(ctx, obs, dds, prec)
    ms = np.ascontiguousarray(obs.vis.transpose(1, 0, 2))  # (rows, channels, pols): MeasurementSet order
    if source == "pageable":
        ctx.set_integration_ms(1, ms, obs.uvw)
    elif source == "pinned":
        ctx.set_integration_ms(1, torch.from_numpy(ms).pin_memory(), torch.from_numpy(obs.uvw))
    else:
        ctx.set_integration_ms(1, torch.from_numpy(ms).cuda(), torch.from_numpy(obs.uvw).cuda())
    got = ctx.calibrate(1, dds, prec)
    np.testing.assert_array_equal(got, exp)
    ctx.release_integration(1)


@pytest.mark.parametrize("source", ["pageable", "pinned"])
def test_ms_order_channel_subset_and_many_pieces(ctx, source):
    """128 antennas x 8 timesteps x 100 channels of which 96 are taken: 203 MB, several staging pieces."""
    obs, dirs = synth.mwa_precision(timesteps=8, channels=100, directions=6)
    md = lg.build_metadata(obs)
    sub = synth.Observation(**{**obs.__dict__, "vis": np.ascontiguousarray(obs.vis[3:99]), "channels": 96,
                               "freq_start_hz": obs.freq_start_hz + 3 * obs.freq_inc_hz})
    md_sub = lg.build_metadata(sub)
    ctx.set_metadata(md_sub)
    dds = _dds(md_sub, dirs)
    exp = _reference(ctx, sub, dds, lg.LEAP_PRECISION_MIXED)
    ms = np.ascontiguousarray(obs.vis.transpose(1, 0, 2))
    if source == "pinned":
        ms = torch.from_numpy(ms).pin_memory()
        uvw = torch.from_numpy(obs.uvw)
    else:
        uvw = obs.uvw
    ctx.set_integration_ms(2, ms, uvw, start_channel=3, channels=96)
    got = ctx.calibrate(2, dds, lg.LEAP_PRECISION_MIXED)
    np.testing.assert_array_equal(got, exp)
    ctx.release_integration(2)


def test_ms_order_rejects_bad_channel_range(ctx):
    obs, _ = synth.small_case(stations=6, timesteps=1, channels=4, directions=1)
    ctx.set_metadata(lg.build_metadata(obs))
    ms = np.ascontiguousarray(obs.vis.transpose(1, 0, 2))
    with pytest.raises(lg.InvalidArgument):
        ctx.set_integration_ms(0, ms, obs.uvw, start_channel=2, channels=3)


@pytest.mark.parametrize("flag_pols", [1, 4])
def test_opt_in_flags_equal_nan_groups(ctx, flag_pols):
    """Flagged groups are zeroed, exactly like NaN groups; no flag changes nothing (the default)."""
    obs, dirs = synth.small_case(stations=22, timesteps=3, channels=19, directions=4, vis_dtype=np.complex64,
                                 seed_shift=5)
    md = lg.build_metadata(obs)
    ctx.set_metadata(md)
    dds = _dds(md, dirs)
    rows, C = obs.rows, obs.channels
    flags = np.zeros((rows, C + 2, flag_pols), dtype=np.uint8)  # MS rows hold 2 more channels than taken
    rng = np.random.default_rng(11)
    pick_r = rng.integers(0, rows, 40)
    pick_c = rng.integers(0, C, 40)
    pick_p = rng.integers(0, flag_pols, 40)
    flags[pick_r, pick_c + 1, pick_p] = 1
    expect_groups = len(set(zip(pick_r.tolist(), pick_c.tolist())))
    ctx.set_integration(0, obs.vis, obs.uvw)
    plain = ctx.calibrate(0, dds, lg.LEAP_PRECISION_FP64)
    assert ctx.apply_flags(0, np.zeros_like(flags), start_channel=1) == 0
    np.testing.assert_array_equal(ctx.calibrate(0, dds, lg.LEAP_PRECISION_FP64), plain)
    assert ctx.apply_flags(0, flags, start_channel=1) == expect_groups
    got = ctx.calibrate(0, dds, lg.LEAP_PRECISION_FP64)
    nan_vis = obs.vis.copy()
    nan_vis[pick_c, pick_r, 0] = np.nan
    ctx.set_integration(1, nan_vis, obs.uvw)
    np.testing.assert_array_equal(got, ctx.calibrate(1, dds, lg.LEAP_PRECISION_FP64))
    assert np.abs(got - plain).max() > 0
    ctx.release_integration(1)


def _device_reads_pageable_memory():
    """cudaDevAttrPageableMemoryAccess and ...UsesHostPageTables of device 0, from the CUDA
    runtime the library loaded."""
    import ctypes
    rt = ctypes.CDLL("libcudart.so.13")
    vals = []
    for attr in (88, 100):
        v = ctypes.c_int(0)
        assert rt.cudaDeviceGetAttribute(ctypes.byref(v), attr, 0) == 0
        vals.append(v.value)
    return all(vals)


def test_async_ingestion_double_buffered(ctx):
    """Chunks uploaded asynchronously into two slots while the other slot is calibrated:
    every chunk's cal phases equal those of a synchronous upload."""
    chunks = []
    for i in range(4):
        obs, dirs = synth.small_case(stations=24, timesteps=2, channels=33, directions=5, vis_dtype=np.complex64,
                                     seed_shift=20 + i)
        chunks.append((obs, dirs))
    md = lg.build_metadata(chunks[0][0])
    ctx.set_metadata(md)
    dds = _dds(md, chunks[0][1])
    exp = []
    for obs, _ in chunks:
        ctx.set_integration(0, obs.vis, obs.uvw)
        exp.append(ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED))
    hosts = [(torch.from_numpy(np.ascontiguousarray(o.vis.transpose(1, 0, 2))).pin_memory(),
              torch.from_numpy(o.uvw).pin_memory()) for o, _ in chunks]
    ctx.set_integration_ms(10, *hosts[0], asynchronous=True)
    for k in range(len(chunks)):
        if k + 1 < len(chunks):
            ctx.set_integration_ms(10 + (k + 1) % 2, *hosts[k + 1], asynchronous=True)
        got = ctx.calibrate(10 + k % 2, dds, lg.LEAP_PRECISION_MIXED)
        np.testing.assert_array_equal(got, exp[k])
    # Pageable memory: read in place on devices that read host page tables (Grace hosts),
    # rejected elsewhere.
    ms_pageable = np.ascontiguousarray(chunks[0][0].vis.transpose(1, 0, 2))
    uvw_pageable = np.ascontiguousarray(chunks[0][0].uvw)
    if _device_reads_pageable_memory():
        ctx.set_integration_ms(12, ms_pageable, uvw_pageable, asynchronous=True)
        np.testing.assert_array_equal(ctx.calibrate(12, dds, lg.LEAP_PRECISION_MIXED), exp[0])
        ctx.release_integration(12)
    else:
        with pytest.raises(lg.InvalidArgument):
            ctx.set_integration_ms(12, ms_pageable, uvw_pageable, asynchronous=True)
    ctx.release_integration(10)
    ctx.release_integration(11)
