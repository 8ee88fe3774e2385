"""Deterministic synthetic observations with the shapes of the benchmark workloads.

No MeasurementSet is available, so every workload is generated: an array of
antennas on the ground, baselines (a <= b, autocorrelations included) in
lexicographic order, rows timestep-major (row = t * nbl + b, as the reference's
MeasurementSet assumes: LA/ms/MeasurementSet.cc:115-130), UVWs from an
hour-angle track, and visibilities

    V_ab(t, nu) = g_a conj(g_b) exp(+2 pi i (u l0 + v m0 + w (n0 - 1)) nu / c) + noise

for every polarisation, with unit-modulus antenna gains of uniform random
phase and complex Gaussian noise (each component N(0, sigma^2 / 2)).

Calibration directions are given as (ra, dec) through the inverse SIN
projection about the phase centre, so that the third row of the reference's
direction matrix (LA/model/cpu/MetaData.cc:166-203) is (l, m, n) and the
reference rotation cancels the model phase in the source direction.

Visibilities are produced directly in the reference Integration layout: a
(channels, rows, pols) C-order array, i.e. the column-major (pol, row, channel)
tensor of LA/model/cpu/Integration.h:73.

Seeds: positions 0, gains 1, noise 2, directions 3, chunk shapes 4.
(LA/ = src/icrar/leap-accelerate/ in the reference project.)
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

SPEED_OF_LIGHT = 299792458.0
EARTH_ROTATION_RAD_S = 7.2921e-5
SITE_LATITUDE_RAD = np.deg2rad(-26.7)
PHASE_CENTRE = (0.0, np.deg2rad(-30.0))
EPOCH0_S = 5.0e9  # arbitrary MJD-seconds origin for the TIME column


@dataclass
class ArraySpec:
    stations: int
    radius_m: float
    layout: str = "uniform"  # "uniform" disc or "loguniform" radial


@dataclass
class Observation:
    """An in-memory stand-in for the MeasurementSet fields the calibration path reads."""
    num_stations: int
    total_antennas: int
    nbaselines: int
    timesteps: int
    channels: int
    pols: int
    freq_start_hz: float
    freq_inc_hz: float
    phase_centre: tuple
    antenna1: np.ndarray      # int32 [nbl] (same for every timestep)
    antenna2: np.ndarray      # int32 [nbl]
    flags: np.ndarray         # uint8 [nbl] FLAG of the first epoch, channel 0, pol 0
    uvw: np.ndarray           # float64 [rows, 3]
    epochs: np.ndarray        # float64 [timesteps]
    vis: Optional[np.ndarray]  # complex [channels, rows, pols]
    gains: np.ndarray         # complex128 [stations]
    positions_enu: np.ndarray  # float64 [stations, 3]
    source_lmn: np.ndarray    # float64 [3]
    noise_sigma: float = 0.0

    @property
    def rows(self) -> int:
        return self.timesteps * self.nbaselines


def antenna_positions(spec: ArraySpec, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    n = spec.stations
    theta = rng.uniform(0.0, 2.0 * np.pi, n)
    if spec.layout == "uniform":
        r = spec.radius_m * np.sqrt(rng.uniform(0.0, 1.0, n))
    elif spec.layout == "loguniform":
        r = np.exp(rng.uniform(np.log(10.0), np.log(spec.radius_m), n))
    else:
        raise ValueError(spec.layout)
    return np.stack([r * np.cos(theta), r * np.sin(theta), np.zeros(n)], axis=1)


def baselines(stations: int, autocorrelations: bool = True):
    a1, a2 = [], []
    for a in range(stations):
        for b in range(a if autocorrelations else a + 1, stations):
            a1.append(a)
            a2.append(b)
    return np.asarray(a1, dtype=np.int32), np.asarray(a2, dtype=np.int32)


def enu_to_uvw(enu: np.ndarray, hour_angle: float, dec: float, lat: float = SITE_LATITUDE_RAD) -> np.ndarray:
    e, n, u = enu[..., 0], enu[..., 1], enu[..., 2]
    x = -np.sin(lat) * n + np.cos(lat) * u
    y = e
    z = np.cos(lat) * n + np.sin(lat) * u
    sh, ch = np.sin(hour_angle), np.cos(hour_angle)
    sd, cd = np.sin(dec), np.cos(dec)
    uu = sh * x + ch * y
    vv = -sd * ch * x + sd * sh * y + cd * z
    ww = cd * ch * x - cd * sh * y + sd * z
    return np.stack([uu, vv, ww], axis=-1)


def lm_to_radec(l: np.ndarray, m: np.ndarray, phase_centre=PHASE_CENTRE) -> np.ndarray:
    """Inverse SIN projection: (l, m) about (ra0, dec0) -> (ra, dec)."""
    ra0, dec0 = phase_centre
    l = np.asarray(l, dtype=np.float64)
    m = np.asarray(m, dtype=np.float64)
    n = np.sqrt(1.0 - l * l - m * m)
    dec = np.arcsin(m * np.cos(dec0) + n * np.sin(dec0))
    ra = ra0 + np.arctan2(l, n * np.cos(dec0) - m * np.sin(dec0))
    return np.stack([ra, dec], axis=-1)


def random_directions(count: int, box_rad: float = 0.1, seed: int = 3, phase_centre=PHASE_CENTRE):
    """(l, m) uniform in a box of side ``box_rad`` centred on the phase centre."""
    rng = np.random.default_rng(seed)
    lm = rng.uniform(-box_rad / 2, box_rad / 2, size=(count, 2))
    return lm_to_radec(lm[:, 0], lm[:, 1], phase_centre), lm


def make_observation(spec: ArraySpec, timesteps: int, channels: int, freq_start_hz: float,
                     freq_inc_hz: float, noise_sigma: float, source_lm=(0.01, -0.005),
                     vis_dtype=np.complex64, pols: int = 4, flag_autos: bool = True,
                     cadence_s: float = 8.0, hour_angle0: float = 0.0, with_vis: bool = True,
                     seeds=(0, 1, 2), timestep_offset: int = 0, positions: Optional[np.ndarray] = None,
                     gains: Optional[np.ndarray] = None, channel_block: int = 16,
                     phase_centre=PHASE_CENTRE) -> Observation:
    pos = antenna_positions(spec, seeds[0]) if positions is None else positions
    S = spec.stations
    if gains is None:
        g_rng = np.random.default_rng(seeds[1])
        gains = np.exp(1j * g_rng.uniform(-np.pi, np.pi, S))
    a1, a2 = baselines(S, True)
    nbl = a1.size
    ra0, dec0 = phase_centre
    rows = timesteps * nbl
    uvw = np.empty((rows, 3), dtype=np.float64)
    for t in range(timesteps):
        ha = hour_angle0 + (t + timestep_offset) * EARTH_ROTATION_RAD_S * cadence_s
        ant_uvw = enu_to_uvw(pos, ha, dec0)
        uvw[t * nbl:(t + 1) * nbl] = ant_uvw[a2] - ant_uvw[a1]
    epochs = EPOCH0_S + (np.arange(timesteps) + timestep_offset) * cadence_s
    flags = (a1 == a2).astype(np.uint8) if flag_autos else np.zeros(nbl, dtype=np.uint8)
    l0, m0 = source_lm
    n0 = np.sqrt(1.0 - l0 * l0 - m0 * m0)
    vis = None
    if with_vis:
        vis = np.empty((channels, rows, pols), dtype=vis_dtype)
        gg = np.tile(gains[a1] * np.conj(gains[a2]), timesteps)
        delay = uvw[:, 0] * l0 + uvw[:, 1] * m0 + uvw[:, 2] * (n0 - 1.0)  # metres
        n_rng = np.random.default_rng(seeds[2])
        scale = noise_sigma / np.sqrt(2.0)
        for c0 in range(0, channels, channel_block):
            c1 = min(channels, c0 + channel_block)
            nu = freq_start_hz + np.arange(c0, c1) * freq_inc_hz
            model = gg[None, :] * np.exp(2j * np.pi * delay[None, :] * (nu[:, None] / SPEED_OF_LIGHT))
            blk = np.repeat(model[:, :, None], pols, axis=2)
            if noise_sigma > 0:
                shape = (c1 - c0, rows, pols)
                blk = blk + scale * (n_rng.standard_normal(shape) + 1j * n_rng.standard_normal(shape))
            vis[c0:c1] = blk.astype(vis_dtype, copy=False)
    return Observation(
        num_stations=S, total_antennas=S, nbaselines=nbl, timesteps=timesteps, channels=channels,
        pols=pols, freq_start_hz=freq_start_hz, freq_inc_hz=freq_inc_hz, phase_centre=tuple(phase_centre),
        antenna1=np.tile(a1, 1), antenna2=np.tile(a2, 1), flags=flags, uvw=uvw, epochs=epochs,
        vis=vis, gains=gains, positions_enu=pos, source_lmn=np.array([l0, m0, n0]), noise_sigma=noise_sigma)


# ---------------------------------------------------------------------------
# Named workloads (sizes of the benchmark configurations)
# ---------------------------------------------------------------------------

def askap_small(with_vis: bool = True) -> tuple:
    """36 antennas in a 3 km disc, 1 timestep, 48 x 1 MHz channels from 700 MHz,
    complex<double>, sigma 0.1, one direction (l, m) = (0.01, -0.005)."""
    obs = make_observation(ArraySpec(36, 3000.0), timesteps=1, channels=48, freq_start_hz=700e6,
                           freq_inc_hz=1e6, noise_sigma=0.1, source_lm=(0.01, -0.005),
                           vis_dtype=np.complex128, with_vis=with_vis)
    dirs = lm_to_radec(np.array([0.01]), np.array([-0.005]))
    return obs, dirs


def mwa_precision(with_vis: bool = True, timesteps: int = 14, channels: int = 384, directions: int = 64) -> tuple:
    """128 antennas in a 1.5 km disc, 14 x 8 s, 384 x 40 kHz from 150 MHz, complex<float>,
    sigma 0.5, 64 directions uniform in a 0.1 rad box (the source is direction 0)."""
    obs = make_observation(ArraySpec(128, 1500.0), timesteps=timesteps, channels=channels,
                           freq_start_hz=150e6, freq_inc_hz=40e3, noise_sigma=0.5,
                           source_lm=(0.01, -0.005), vis_dtype=np.complex64, with_vis=with_vis)
    dirs, lm = random_directions(directions)
    dirs[0] = lm_to_radec(np.array([0.01]), np.array([-0.005]))[0]
    return obs, dirs


def mwa_at_phase_centre(phase_centre, with_vis: bool = True, timesteps: int = 14, channels: int = 384) -> Observation:
    """The 128-antenna array of mwa_precision observed about another phase centre (ra, dec)
    in radians: for calibration directions given as (ra, dec) far from it."""
    return make_observation(ArraySpec(128, 1500.0), timesteps=timesteps, channels=channels,
                            freq_start_hz=150e6, freq_inc_hz=40e3, noise_sigma=0.5, source_lm=(0.01, -0.005),
                            vis_dtype=np.complex64, with_vis=with_vis, phase_centre=phase_centre)


def small_case(stations: int = 8, timesteps: int = 2, channels: int = 6, pols: int = 4, directions: int = 3,
               vis_dtype=np.complex128, noise_sigma: float = 0.3, seed_shift: int = 0) -> tuple:
    """Tiny arrays for element-wise parity tests."""
    obs = make_observation(ArraySpec(stations, 800.0), timesteps=timesteps, channels=channels,
                           freq_start_hz=120e6, freq_inc_hz=250e3, noise_sigma=noise_sigma,
                           source_lm=(0.02, 0.01), vis_dtype=vis_dtype, pols=pols,
                           seeds=(10 + seed_shift, 11 + seed_shift, 12 + seed_shift))
    dirs, _ = random_directions(directions, box_rad=0.08, seed=13 + seed_shift)
    return obs, dirs


@dataclass
class Chunk:
    timesteps: int
    channels: int
    timestep_offset: int


def uneven_chunks(count: int = 32, seed: int = 4, t_range=(1, 64), channel_choices=(48, 96, 384)) -> List[Chunk]:
    """Integration chunks with timesteps uniform in t_range and channels from channel_choices."""
    rng = np.random.default_rng(seed)
    ts = rng.integers(t_range[0], t_range[1] + 1, size=count)
    cs = rng.choice(np.asarray(channel_choices), size=count)
    chunks, off = [], 0
    for t, c in zip(ts, cs):
        chunks.append(Chunk(int(t), int(c), off))
        off += int(t)
    return chunks


def read_leapms(path: str, read_autocorrelations: bool = True) -> Observation:
    """Read a ".leapms" file (the format write_leapms writes) as an Observation whose
    visibilities stay in MeasurementSet order: ``obs.ms_vis`` is (rows, channels, pols)
    and ``obs.vis`` is its (channels, rows, pols) view.  The baseline count follows the
    reference, n(n+1)/2 with autocorrelations (LA/ms/MeasurementSet.cc:149-167)."""
    with open(path, "rb") as f:
        if f.read(8) != b"LEAPMS01":
            raise ValueError(f"{path}: not a .leapms file")
        stations, total, rows, channels, pols, is_double = (int(x) for x in np.fromfile(f, "<u4", 6))
        f0, df, ra0, dec0 = (float(x) for x in np.fromfile(f, "<f8", 4))
        a1 = np.fromfile(f, "<i4", rows)
        a2 = np.fromfile(f, "<i4", rows)
        flags = np.fromfile(f, np.uint8, rows)
        times = np.fromfile(f, "<f8", rows)
        uvw = np.fromfile(f, "<f8", rows * 3).reshape(rows, 3)
        dt = np.complex128 if is_double else np.complex64
        ms_vis = np.fromfile(f, dt, rows * channels * pols).reshape(rows, channels, pols)
    nbl = stations * (stations + 1) // 2 if read_autocorrelations else stations * (stations - 1) // 2
    if rows % nbl:
        raise ValueError(f"{path}: {rows} rows is not a whole number of {nbl}-baseline timesteps")
    T = rows // nbl
    obs = Observation(num_stations=stations, total_antennas=total, nbaselines=nbl, timesteps=T, channels=channels,
                      pols=pols, freq_start_hz=f0, freq_inc_hz=df, phase_centre=(ra0, dec0),
                      antenna1=a1[:nbl].copy(), antenna2=a2[:nbl].copy(), flags=flags[:nbl].copy(), uvw=uvw,
                      epochs=times[::nbl][:T].copy(), vis=ms_vis.transpose(1, 0, 2), gains=np.ones(stations),
                      positions_enu=np.zeros((stations, 3)), source_lmn=np.zeros(3))
    obs.ms_vis = ms_vis
    return obs


def write_leapms(obs: Observation, path: str) -> None:
    """Write an observation as a ".leapms" file for the C++ MeasurementSet stand-in:
    header, per-row ANTENNA1/ANTENNA2/FLAG/TIME/UVW, then DATA in the
    MeasurementSet's own [row][channel][pol] order."""
    nbl, T = obs.nbaselines, obs.timesteps
    rows = nbl * T
    is_double = obs.vis.dtype == np.complex128
    with open(path, "wb") as f:
        f.write(b"LEAPMS01")
        np.array([obs.num_stations, obs.total_antennas, rows, obs.channels, obs.pols, int(is_double)],
                 dtype="<u4").tofile(f)
        np.array([obs.freq_start_hz, obs.freq_inc_hz, obs.phase_centre[0], obs.phase_centre[1]], dtype="<f8").tofile(f)
        np.tile(obs.antenna1[:nbl], T).astype("<i4").tofile(f)
        np.tile(obs.antenna2[:nbl], T).astype("<i4").tofile(f)
        np.tile(np.asarray(obs.flags[:nbl], dtype=np.uint8), T).tofile(f)
        np.repeat(obs.epochs, nbl).astype("<f8").tofile(f)
        np.ascontiguousarray(obs.uvw, dtype="<f8").tofile(f)
        np.ascontiguousarray(obs.vis.transpose(1, 0, 2)).tofile(f)


# ---------------------------------------------------------------------------
# Device-side generation (benchmark sizes: tens of GB of visibilities)
# ---------------------------------------------------------------------------

_SYNTH_LIB = None


def _synth_lib():
    global _SYNTH_LIB
    if _SYNTH_LIB is None:
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libleap_synth.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is not built (run the package build first)")
        lib = ctypes.CDLL(path)
        lib.leap_synth_fill_c64.restype = ctypes.c_int32
        lib.leap_synth_fill_c64.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                            ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_uint64, ctypes.c_void_p]
        _SYNTH_LIB = lib
    return _SYNTH_LIB


def model_delay_and_gains(obs: Observation):
    """Per-row delay u l0 + v m0 + w (n0 - 1) (metres) and per-baseline g_a conj(g_b)."""
    l0, m0, n0 = obs.source_lmn
    delay = obs.uvw[:, 0] * l0 + obs.uvw[:, 1] * m0 + obs.uvw[:, 2] * (n0 - 1.0)
    nbl = obs.nbaselines
    gg = obs.gains[obs.antenna1[:nbl]] * np.conj(obs.gains[obs.antenna2[:nbl]])
    return np.ascontiguousarray(delay), np.ascontiguousarray(gg.astype(np.complex128))


def device_visibilities(obs: Observation, device, seed: int = 2, stream=None):
    """The observation's complex<float> visibility cube (channels, rows, pols),
    generated on the GPU by the same model as make_observation (a different
    noise stream): returns a torch tensor on `device`."""
    import torch
    delay, gg = model_delay_and_gains(obs)
    dev = torch.device(device)
    d_delay = torch.from_numpy(delay).to(dev)
    d_gg = torch.from_numpy(gg.view(np.float64)).to(dev)
    vis = torch.empty((obs.channels, obs.rows, obs.pols), dtype=torch.complex64, device=dev)
    s = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    rc = _synth_lib().leap_synth_fill_c64(vis.data_ptr(), d_delay.data_ptr(), d_gg.data_ptr(), obs.rows,
                                          obs.nbaselines, obs.channels, obs.pols, obs.freq_start_hz,
                                          obs.freq_inc_hz, float(obs.noise_sigma), int(seed), s)
    if rc != 0:
        raise RuntimeError(f"leap_synth_fill_c64 failed with CUDA error {rc}")
    torch.cuda.synchronize(dev)
    return vis


def ska_low(with_vis: bool = True, timesteps: int = 16, channels: int = 384, directions: int = 128) -> tuple:
    """512 stations, log-uniform radial layout to 40 km, 16 x 8 s, 384 x 5.4 kHz from
    100 MHz, complex<float>, sigma 1.0, 128 directions (the source is direction 0)."""
    obs = make_observation(ArraySpec(512, 40000.0, "loguniform"), timesteps=timesteps, channels=channels,
                           freq_start_hz=100e6, freq_inc_hz=5.4e3, noise_sigma=1.0, source_lm=(0.01, -0.005),
                           vis_dtype=np.complex64, with_vis=with_vis)
    dirs, _ = random_directions(directions)
    dirs[0] = lm_to_radec(np.array([0.01]), np.array([-0.005]))[0]
    return obs, dirs


def batched_uneven(chunks: int = 32, directions: int = 256, stations: int = 128,
                   sample_timesteps: Optional[int] = None, direction_ids: Optional[np.ndarray] = None):
    """The batched workload: `chunks` consecutive integration chunks of the
    128-antenna array (timesteps uniform in 1..64, channels from {48, 96, 384},
    seed 4), 150 MHz / 40 kHz, sigma 0.5, and `directions` directions dealt
    round-robin to the chunks (direction j -> chunk j mod chunks).

    With sample_timesteps, each chunk is cut to its first sample_timesteps timesteps
    and its visibilities are generated on the host (a bounded sample of the workload
    for a CPU run).  direction_ids restricts the calibration to those of the
    `directions` directions (each still goes to chunk j mod chunks; a sharded run
    passes its own range).

    Returns (observations, directions (ra, dec) in item order, work items
    [(slot, first_direction, ndirections)], original direction index of each
    item-ordered direction)."""
    spec = ArraySpec(stations, 1500.0)
    pos = antenna_positions(spec, 0)
    gains = np.exp(1j * np.random.default_rng(1).uniform(-np.pi, np.pi, stations))
    shapes = uneven_chunks(chunks, seed=4)
    dirs, _ = random_directions(directions)
    dirs[0] = lm_to_radec(np.array([0.01]), np.array([-0.005]))[0]
    wanted = np.arange(directions) if direction_ids is None else np.asarray(direction_ids)
    obs_list, order, items = [], [], []
    for i, ch in enumerate(shapes):
        t = ch.timesteps if sample_timesteps is None else min(ch.timesteps, sample_timesteps)
        obs_list.append(make_observation(spec, timesteps=t, channels=ch.channels, freq_start_hz=150e6,
                                         freq_inc_hz=40e3, noise_sigma=0.5, source_lm=(0.01, -0.005),
                                         vis_dtype=np.complex64, with_vis=sample_timesteps is not None,
                                         timestep_offset=ch.timestep_offset, positions=pos, gains=gains,
                                         seeds=(0, 1, 2 + i)))
        mine = [int(j) for j in wanted if j % chunks == i]
        if mine:
            items.append((i, len(order), len(mine)))
            order += mine
    return obs_list, dirs[order], items, np.asarray(order)
