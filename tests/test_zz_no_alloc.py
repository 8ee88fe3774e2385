"""The entry point that allocates no device memory (leap_rotate_average_noalloc).

Some callers cannot allocate device memory while they run: code that records a
CUDA graph (no cudaMalloc between capture begin and end), hosts whose device
memory belongs to another runtime's pool and that only hand this library
pre-allocated buffers, and real-time pipelines that cannot take an
allocation's latency.  For them the rotate + average stage keeps its scratch in
a fixed array built into the library.  This test checks, through the C ABI,
that two calls in a row give the avgData of the regular entry point
(leap_calibrate, all-FP64 form) within the FP64 avgData tolerance of the
parity tests, including NaN samples, which this entry point skips itself.

The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

import leap_gb300 as lg
from leap_gb300 import _abi, synth

pytestmark = pytest.mark.gpu

FP64_AVG_RTOL = 1e-11  # same bar as the all-FP64 avgData parity tests


def _regular_avgdata(obs, dds):
    md = lg.build_metadata(obs)
    with lg.Context(0) as ctx:
        ctx.set_metadata(md)
        ctx.set_integration(0, obs.vis, obs.uvw)
        ctx.calibrate(0, dds, lg.LEAP_PRECISION_FP64)
        return np.stack([ctx.avgdata(d) for d in range(dds.shape[0])])  # (D, nbl, P)


@pytest.mark.parametrize("dtype,timesteps,stations,channels,ndir", [
    (np.complex128, 5, 24, 40, 6),    # several timestep slabs
    (np.complex64, 9, 24, 40, 6),
    (np.complex64, 1, 24, 40, 6),     # one timestep: the kernel writes avg_out itself, no slab sum
    (np.complex64, 6, 128, 16, 8),    # 4.2 MB per slab: fewer slabs than the launch wants, to fit 16 MiB
], ids=["c128_slabs", "c64_slabs", "c64_single_slab", "c64_slabs_cut_to_fit"])
def test_no_alloc_entry_point_matches_regular_path(dtype, timesteps, stations, channels, ndir):
    import torch
    obs, dirs = synth.small_case(stations=stations, timesteps=timesteps, channels=channels, pols=4, directions=ndir,
                                 vis_dtype=dtype, seed_shift=5)
    vis = obs.vis.copy()
    vis.reshape(-1)[[3, 1000, min(4321, vis.size - 1)]] = np.nan
    obs.vis = vis
    md = lg.build_metadata(obs)
    dds = np.stack([lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs])
    expected = _regular_avgdata(obs, dds)

    dev = torch.device("cuda:0")
    torch.cuda.set_device(0)
    vis_d = torch.from_numpy(obs.vis).to(dev)
    uvw_d = torch.from_numpy(obs.uvw).to(dev)
    dd_d = torch.from_numpy(dds.reshape(-1).copy()).to(dev)
    D, nbl, P = len(dirs), obs.nbaselines, obs.pols
    out = torch.empty((D, P, nbl, 2), dtype=torch.float64, device=dev)
    vt = _abi.LEAP_VIS_C128 if dtype == np.complex128 else _abi.LEAP_VIS_C64
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out.fill_(float("nan"))
        rc = _abi.lib.leap_rotate_average_noalloc(vt, vis_d.data_ptr(), uvw_d.data_ptr(), obs.rows, obs.channels, P,
                                                  nbl, obs.freq_start_hz, obs.freq_inc_hz, dd_d.data_ptr(), D,
                                                  out.data_ptr(), ctypes.c_void_p(stream))
        assert rc == _abi.LEAP_OK, _abi.lib.leap_noalloc_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        got = (got[..., 0] + 1j * got[..., 1]).transpose(0, 2, 1)  # (D, nbl, P)
        for d in range(D):
            scale = np.abs(expected[d]).max()
            assert np.abs(got[d] - expected[d]).max() <= FP64_AVG_RTOL * scale, f"call {call} direction {d}"


def test_no_alloc_rejects_oversized_channel_count():
    import torch
    dev = torch.device("cuda:0")
    x = torch.zeros(16, dtype=torch.float64, device=dev)
    too_many = _abi.LEAP_NOALLOC_SCRATCH_BYTES // 16 + 1  # wavelengths and reciprocals, 16 B a channel
    rc = _abi.lib.leap_rotate_average_noalloc(_abi.LEAP_VIS_C64, x.data_ptr(), x.data_ptr(), 1, too_many, 1, 1,
                                              1e8, 1e3, x.data_ptr(), 1, x.data_ptr(), None)
    assert rc == _abi.LEAP_ERR_INVALID_ARGUMENT
    assert b"scratch" in _abi.lib.leap_noalloc_last_error()
