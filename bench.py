"""Benchmark of the GB300 LEAP calibration hot path.

Metric: vis-directions/s — one visibility sample (pol, row, channel) phase-
rotated and averaged for one calibration direction, through the whole path
(rotate + average, phase angles, both pseudoinverse contractions).

Workload (default): the precision-form MWA-like array — 128 antennas (8256
baselines with autocorrelations), 14 timesteps at 8 s, 384 channels of 40 kHz
from 150 MHz, 4 pols, complex<float> visibilities, 64 directions; synthetic,
seeded.  The 1.42 GB visibility cube is larger than L2 (129 MB), so no L2 flush
is needed between steps.

  value      inputs resident in HBM, the mixed-precision form, CUDA events on
             the launching stream around exactly --steps calls
  e2e        the public C ABI with host buffers: per step the visibilities in
             MeasurementSet order ([row][channel][pol], page-locked host memory) +
             UVWs go up through leap_set_integration_ms (transposed on the device),
             then leap_calibrate with host dd / cal buffers; the upload of the
             pre-transposed Integration layout (leap_set_integration) is reported
             beside it
  plain_fp64 the all-FP64 form on the same workload
  roofline   the rotate+average kernel against the measured HBM copy bandwidth
  cpu_baseline  the oracle port (C, OpenMP over directions) on a bounded sample

``--impl reference`` times the reference CPU algorithm (the oracle port of
CpuLeapCalibrator, the reference itself cannot be built here) on all host cores.
Multi-GPU (torchrun): each rank calibrates its own directions on its own copy
of the integration (weak scaling, no collective); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "icrar-leap-accelerate_gb300")
sys.path.insert(0, PKG)


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region
    (one `nvidia-smi -lms 200` process for the whole region)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._p = None

    def __enter__(self):
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                        "--format=csv,noheader,nounits", "-lms", "200"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)  # first sample before the timed region starts
        except Exception:
            self._p = None
        return self

    def __exit__(self, *a):
        if self._p is None:
            return
        time.sleep(0.25)
        self._p.terminate()
        try:
            out, _ = self._p.communicate(timeout=5)
        except Exception:
            self._p.kill()
            out, _ = self._p.communicate()
        for line in (out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                self.samples.append(f)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 5 + i and s[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_workload(args, rank: int):
    from leap_gb300 import synth
    obs, dirs = synth.mwa_precision(timesteps=args.timesteps or 14, channels=args.channels, directions=args.directions)
    if rank:
        # Each rank calibrates its own directions (same array and integration).
        _, lm = synth.random_directions(args.directions, seed=3 + 1000 * rank)
        dirs = synth.lm_to_radec(lm[:, 0], lm[:, 1])
    return obs, dirs


def vis_dirs(obs, ndir: int) -> float:
    return float(obs.pols) * obs.rows * obs.channels * ndir


def bench_cpu(obs, dirs, vis_t0, threads: int, budget_s: float):
    """Oracle port on a bounded sample: the first timestep (vis_t0: (channels, nbl, pols))
    and the first directions of the workload, grown towards `budget_s` seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    mdo = oracle.metadata(obs)
    nbl = obs.nbaselines
    vis = np.ascontiguousarray(vis_t0)
    uvw = obs.uvw[:nbl]
    d_s = max(1, min(len(dirs), threads))
    dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs[:d_s]])
    t0 = time.perf_counter()
    oracle.calibrate_interval(vis, uvw, dds, mdo, nthreads=threads)
    dt = time.perf_counter() - t0
    # grow the sample towards the budget (directions are independent)
    reps = max(1, int(budget_s / max(dt, 1e-3)))
    d_s2 = min(len(dirs), d_s * reps)
    if d_s2 > d_s:
        dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs[:d_s2]])
        t0 = time.perf_counter()
        oracle.calibrate_interval(vis, uvw, dds, mdo, nthreads=threads)
        dt = time.perf_counter() - t0
        d_s = d_s2
    # repeat the sample until the budget is spent, so the timing covers ~budget_s of CPU work
    runs, total = 1, dt
    while total < budget_s:
        t0 = time.perf_counter()
        oracle.calibrate_interval(vis, uvw, dds, mdo, nthreads=threads)
        total += time.perf_counter() - t0
        runs += 1
    units = float(obs.pols) * vis.shape[1] * obs.channels * d_s * runs
    return units / total, {"timesteps": 1, "directions": d_s, "seconds": total, "runs": runs}


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    obs, dirs = make_workload(args, 0)
    threads = oracle.max_threads()
    mdo = oracle.metadata(obs)
    nbl = obs.nbaselines
    # Each step: a bounded sample of the workload (1 timestep, `threads` directions).
    vis = np.ascontiguousarray(obs.vis[:, :nbl, :])
    uvw = obs.uvw[:nbl]
    d_s = min(len(dirs), max(1, threads))
    dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs[:d_s]])
    for _ in range(args.warmup):
        oracle.calibrate_interval(vis, uvw, dds, mdo, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.calibrate_interval(vis, uvw, dds, mdo, nthreads=threads)
    dt = (time.perf_counter() - t0) / args.steps
    units = float(obs.pols) * nbl * obs.channels * d_s
    value = units / dt
    line = {
        "impl": "reference", "metric": "vis-directions/s", "value": value, "unit": "vis-directions/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "mwa_precision 128ant/8256bl/14t/384ch/4pol/64dir c64", "sample_per_step":
                   f"1 timestep x {d_s} directions"},
        "cpu_baseline": {"value": value, "unit": "vis-directions/s", "cores": threads, "kind": "port",
                         "sample": f"1 of {obs.timesteps} timesteps, {d_s} of {len(dirs)} directions per step"},
        "e2e": {"value": value, "unit": "vis-directions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def wrapped_max_diff(a, b) -> float:
    return float(np.abs(np.angle(np.exp(1j * (np.asarray(a) - np.asarray(b))))).max())


def branch_margins(ctx, md, D, torch, dev, stream):
    """Per direction of the last calibrate call: the smallest distance from +-pi of any arg()
    in its solve (phi1 at the reference-antenna baselines, dInt at the first |I| rows), from
    that call's own avgData.  An angle within a form's error of +-pi may land on the other
    branch in another form; the cal phases then differ by 2*pi times a column of Ad (or Ad1),
    a different branch rather than an error."""
    from leap_gb300 import _abi
    from leap_gb300.calibrator import stream_handle
    nbl = md.nbaselines
    avg0 = torch.empty((D, nbl), dtype=torch.complex128, device=dev)
    ctx._check(_abi.lib.leap_get_avgdata_device(ctx.handle, 0, avg0.data_ptr(), stream_handle(stream)))
    torch.cuda.synchronize()
    i1 = torch.as_tensor(np.where(md.I1 < 0, md.I1 + nbl, md.I1), dtype=torch.int64, device=dev)
    A = torch.as_tensor(md.A, device=dev)
    Ad1 = torch.as_tensor(md.Ad1, device=dev)
    phi1 = torch.angle(avg0[:, i1])
    cal1 = torch.cat([phi1, torch.zeros((D, 1), dtype=torch.float64, device=dev)], dim=1) @ Ad1.T
    nI = A.shape[0] - 1
    out = []
    for d0 in range(0, D, 16):  # bounded temporaries at 130k baselines
        acal = cal1[d0:d0 + 16] @ A[:nI].T
        dint = torch.angle(torch.exp(-2j * np.pi * acal) * avg0[d0:d0 + 16, :nI])
        m = torch.minimum((np.pi - dint.abs()).min(dim=1).values, (np.pi - phi1[d0:d0 + 16].abs()).min(dim=1).values)
        out.append(m)
    return torch.cat(out).cpu().numpy()


class Workload:
    """One benchmark workload resident on the device: `step(precision)` launches one
    pass of the hot path; `e2e_step()` runs the same through the C ABI with host buffers."""
    name = ""
    config: dict = {}
    units = 0.0           # vis-directions per step
    b_alg = 0.0           # algorithmic HBM bytes per step (vis once per direction)
    f_alg = 0.0           # FP32 FMA-pipe issue slots per step (compute roof)
    traffic = None        # measured DRAM bytes per launch of the bulk kernel, if known
    h2d = 0
    d2h = 0
    kernel_timing = "rotate"  # which leap_timings field times the bulk pass
    checks: dict = {}


def alg_bytes(samples: float, rows: float, ndir: int, nbl: int, pols: int, vis_bytes: int) -> float:
    """Bytes of the bulk pass on the per-direction convention: every direction reads the
    visibilities (vis_bytes each) and 24 B of UVW per row, and writes its FP64 avgData."""
    return ndir * (samples * vis_bytes + rows * 24) + ndir * nbl * pols * 16


def fma_slots(rows: float, channels_x_rows: float, ndir: int, pols: int) -> float:
    return ndir * channels_x_rows * (pols * 4 + 5)


def grid_mma_flops(obs, dds: np.ndarray, taps: int = 10, jw_max: int = 64, stride: int = 48, dirs_per_unit: int = 64):
    """Tensor-core FLOPs of one call of the gridded kernel: the grid windows of its units
    (quad of 4 baselines x all timesteps x up to 64 directions), computed as the kernel
    computes them, times the 3xTF32 MMAs (6 per 16-channel chunk, M = 128, N = 2 jw, K = 8)."""
    C, nbl, T = obs.channels, obs.nbaselines, obs.timesteps
    n, lbase = 2 * C, ((C + taps + 8 + 7) // 8) * 8
    nchunk = (C + 15) // 16
    kb = -(dds[:, 2, :] - np.array([0.0, 0.0, 1.0])) * obs.freq_inc_hz / 299792458.0  # (D, 3) turns per metre
    uvw = obs.uvw.reshape(T, nbl, 3)
    nquad = (nbl + 3) // 4
    flops = 0.0
    for d0 in range(0, dds.shape[0], dirs_per_unit):
        B = np.einsum("tbj,dj->tbd", uvw, kb[d0:d0 + dirs_per_unit])          # turns per channel
        B = B - np.rint(B)
        s = np.floor(B * n).astype(np.int64) - taps // 2 + 1
        pad = nquad * 4 - nbl
        smin = np.pad(s.min(axis=(0, 2)), (0, pad), constant_values=1 << 40).reshape(nquad, 4).min(axis=1)
        smax = np.pad(s.max(axis=(0, 2)), (0, pad), constant_values=-(1 << 40)).reshape(nquad, 4).max(axis=1)
        r0 = ((smin + lbase) >> 3) * 8
        need = smax + 16 + lbase - r0
        single = need <= jw_max
        jw = np.where(single, np.maximum(16, (need + 7) & ~7), jw_max)
        npass = np.where(single, 1, (smax + lbase - r0) // stride + 1)
        ntb = (T + 3) // 4
        flops += float((ntb * npass * nchunk * 6 * 2 * 128 * 2 * jw * 8).sum())
    return flops


def setup_single(args, ctx, lg, torch, local, rank, kind: str):
    """One integration, all directions in one leap_calibrate_async call (MWA or SKA-Low)."""
    from leap_gb300 import synth
    dev = f"cuda:{local}"
    w = Workload()
    if kind == "mwa":
        obs, dirs = make_workload(args, rank)
        vis_host = torch.from_numpy(obs.vis).pin_memory()
        vis_dev = vis_host.to(dev)
        w.cpu_case = (obs, dirs, obs.vis[:, :obs.nbaselines, :])
        w.name = (f"mwa_precision {obs.num_stations}ant/{obs.nbaselines}bl/{obs.timesteps}t/{obs.channels}ch/"
                  f"{obs.pols}pol/{len(dirs)}dir c64")
    else:
        obs, dirs = synth.ska_low(with_vis=False, timesteps=args.timesteps or 16, directions=args.directions or 128)
        if rank:
            _, lm = synth.random_directions(len(dirs), seed=3 + 1000 * rank)
            dirs = synth.lm_to_radec(lm[:, 0], lm[:, 1])
        vis_dev = synth.device_visibilities(obs, dev, seed=2)
        w.cpu_case = (obs, dirs, vis_dev[:, :obs.nbaselines, :].cpu().numpy())
        vis_host = None
        if args.e2e:
            vis_host = torch.empty(vis_dev.shape, dtype=vis_dev.dtype, pin_memory=True)
            vis_host.copy_(vis_dev)
        w.name = (f"ska_low {obs.num_stations}st/{obs.nbaselines}bl/{obs.timesteps}t/{obs.channels}ch/"
                  f"{obs.pols}pol/{len(dirs)}dir c64 (visibilities generated on the device)")
    t0 = time.perf_counter()
    md = ctx.build_metadata(obs)  # on the device (leap_build_metadata); installs it on the context
    w.metadata_s = time.perf_counter() - t0
    uvw_host = torch.from_numpy(obs.uvw).pin_memory()
    ctx.set_integration(0, vis_dev, uvw_host.to(dev))
    del vis_dev
    torch.cuda.empty_cache()
    dds = np.stack([lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs])
    D, S = len(dirs), md.A.shape[1]
    dd_dev = torch.from_numpy(dds.reshape(-1)).to(dev)
    cal_dev = torch.empty((D, S), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream

    def step(p):
        ctx.calibrate_async(0, dd_dev.data_ptr(), D, p, cal_dev.data_ptr(), stream)

    w.step = step
    w.result = lambda: cal_dev.cpu().numpy().copy()
    w.obs, w.dirs, w.md, w.D, w.S = obs, dirs, md, D, S
    w.min_ndir = D
    w.grid_flops = grid_mma_flops(obs, dds)
    w.vis_bytes_resident = obs.rows * obs.channels * obs.pols * 8
    # DRAM traffic of one launch of the gridded kernel, from an ncu capture
    # (dram__bytes_read.sum + dram__bytes_write.sum) of the 4-timestep case of the
    # MWA workload: 101.8 MB read per timestep (the visibilities, once) + 26.9 MB of
    # sum writes, scaled to the timesteps of this run.
    if kind == "mwa" and obs.nbaselines == 8256 and obs.channels == 384 and D == 64:
        w.grid_traffic = 101.80e6 * obs.timesteps + 26.94e6
    w.units = vis_dirs(obs, D)
    w.b_alg = alg_bytes(obs.pols * obs.rows * obs.channels, obs.rows, D, obs.nbaselines, obs.pols, 8)
    w.f_alg = fma_slots(obs.rows, obs.rows * obs.channels, D, obs.pols)
    # DRAM traffic of one launch of the bulk kernel, from an ncu capture
    # (dram__bytes_read.sum + dram__bytes_write.sum) of the 2-timestep case of the
    # MWA workload: 101.7 MB read per timestep (the visibilities, once) + 44.7 MB
    # of partial-sum writes, scaled to the timesteps of this run.
    if kind == "mwa" and obs.nbaselines == 8256 and obs.channels == 384 and D == 64:
        w.traffic = 101.74e6 * obs.timesteps + 44.74e6
    w.config = {"workload": w.name, "precision": args.precision,
                "l2": f"inputs ({obs.vis.nbytes / 1e9 if obs.vis is not None else obs.rows * obs.channels * 32 / 1e9:.2f} GB)"
                      " larger than L2; no flush"}
    if vis_host is not None:
        # The host holds the visibilities in MeasurementSet order, [row][channel][pol]
        # (page-locked); each step ingests them through leap_set_integration_ms, which
        # transposes on the device, then calibrates with host dd / cal buffers.
        ms_host = torch.empty((vis_host.shape[1], vis_host.shape[0], vis_host.shape[2]), dtype=vis_host.dtype,
                              pin_memory=True)
        ms_host.copy_(vis_host.permute(1, 0, 2))
        vis_np = vis_host.numpy()
        uvw_np = uvw_host.numpy()
        cal_host = np.zeros((D, S), dtype=np.float64)
        C, rows, P = vis_np.shape
        prec = lg.LEAP_PRECISION_MIXED if args.precision == "mixed" else lg.LEAP_PRECISION_FP64
        from leap_gb300 import _abi

        def e2e_step():
            ctx._check(_abi.lib.leap_set_integration_ms(ctx.handle, 0, _abi.LEAP_VIS_C64, ms_host.data_ptr(), C, 0,
                                                        uvw_np.ctypes.data, rows, C, P, _abi.LEAP_MEMORY_HOST))
            ctx._check(_abi.lib.leap_calibrate(ctx.handle, 0, dds.ctypes.data, D, prec, cal_host.ctypes.data))

        def e2e_pipelined(n):
            # Double-buffered: the upload of step k+1's visibilities (asynchronous, copy stream) overlaps
            # the calibration of step k; every step still moves its full input and output.
            lib = _abi.lib
            ctx._check(lib.leap_set_integration_ms_async(ctx.handle, 0, _abi.LEAP_VIS_C64, ms_host.data_ptr(), C, 0,
                                                         uvw_host.data_ptr(), rows, C, P, _abi.LEAP_MEMORY_HOST))
            for k in range(n):
                if k + 1 < n:
                    ctx._check(lib.leap_set_integration_ms_async(ctx.handle, (k + 1) % 2, _abi.LEAP_VIS_C64,
                                                                 ms_host.data_ptr(), C, 0, uvw_host.data_ptr(), rows,
                                                                 C, P, _abi.LEAP_MEMORY_HOST))
                ctx._check(lib.leap_calibrate(ctx.handle, k % 2, dds.ctypes.data, D, prec, cal_host.ctypes.data))

        def e2e_layout_step():
            ctx._check(_abi.lib.leap_set_integration(ctx.handle, 0, _abi.LEAP_VIS_C64, vis_np.ctypes.data,
                                                     uvw_np.ctypes.data, rows, C, P, _abi.LEAP_MEMORY_HOST))
            ctx._check(_abi.lib.leap_calibrate(ctx.handle, 0, dds.ctypes.data, D, prec, cal_host.ctypes.data))

        w.e2e_step = e2e_step
        w.e2e_pipelined = e2e_pipelined
        w.e2e_alt = ("integration_layout_upload", e2e_layout_step)
        w.h2d = vis_np.nbytes + uvw_np.nbytes + dds.nbytes
        w.d2h = cal_host.nbytes
    else:
        w.e2e_step = None
    return w


def setup_batched(args, ctx, lg, torch, local, rank):  # noqa: C901
    """32 uneven integration chunks, 256 directions, one leap_calibrate_batched call per step."""
    from leap_gb300 import synth
    dev = f"cuda:{local}"
    w = Workload()
    nd = args.directions or 256
    obs_list, dirs, items, order = synth.batched_uneven(chunks=args.chunks, directions=nd)
    t0 = time.perf_counter()
    md = ctx.build_metadata(obs_list[0])
    w.metadata_s = time.perf_counter() - t0
    spot = None
    hosts = []
    small = min(range(len(obs_list)), key=lambda i: obs_list[i].rows * obs_list[i].channels)
    for i, obs in enumerate(obs_list):
        vis = synth.device_visibilities(obs, dev, seed=2000 + i)
        ctx.set_integration(i, vis, torch.from_numpy(obs.uvw).to(dev))
        if args.e2e:
            vh = torch.empty(vis.shape, dtype=vis.dtype, pin_memory=True)
            vh.copy_(vis)
            hosts.append((vh, torch.from_numpy(obs.uvw).pin_memory()))
        if i == small:
            spot = vis.cpu().numpy()
        del vis
    torch.cuda.empty_cache()
    dds = np.stack([lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs])
    D, S = len(dirs), md.A.shape[1]
    holder = {}

    def step(p):
        holder["cal"] = ctx.calibrate_batched(items, dds, p)

    w.step = step
    w.result = lambda: holder["cal"].copy()
    w.kernel_timing = "total"
    w.obs, w.dirs, w.md, w.D, w.S, w.items, w.dds = obs_list[0], dirs, md, D, S, items, dds
    w.min_ndir = min(it[2] for it in items)
    w.units = sum(float(obs_list[sl].pols) * obs_list[sl].rows * obs_list[sl].channels * n for sl, _, n in items)
    w.b_alg = sum(alg_bytes(4.0 * obs_list[sl].rows * obs_list[sl].channels, obs_list[sl].rows, n,
                            obs_list[sl].nbaselines, 4, 8) for sl, _, n in items)
    w.f_alg = sum(fma_slots(obs_list[sl].rows, obs_list[sl].rows * obs_list[sl].channels, n, 4) for sl, _, n in items)
    samples = sum(4.0 * o.rows * o.channels for o in obs_list)
    w.vis_bytes_resident = samples * 8
    w.name = (f"batched_uneven 128ant/8256bl, {len(obs_list)} chunks (T 1-64, C in 48/96/384; "
              f"{int(sum(o.timesteps for o in obs_list))} timesteps), {D} directions round-robin, 4pol c64 "
              f"({samples * 8 / 1e9:.1f} GB, generated on the device)")
    w.config = {"workload": w.name, "precision": args.precision, "chunks": [[o.timesteps, o.channels] for o in obs_list],
                "l2": "inputs larger than L2; no flush"}
    w.spot = (small, obs_list[small], spot)
    sl, d0, nd = next(it for it in items if it[0] == small)
    w.cpu_case = (obs_list[small], dirs, spot[:, :obs_list[small].nbaselines, :])
    if args.e2e:
        prec = lg.LEAP_PRECISION_MIXED if args.precision == "mixed" else lg.LEAP_PRECISION_FP64
        from leap_gb300 import _abi

        def e2e_step():
            for i, (vh, uh) in enumerate(hosts):
                C, rows, P = vh.shape
                ctx._check(_abi.lib.leap_set_integration(ctx.handle, i, _abi.LEAP_VIS_C64, vh.data_ptr(),
                                                         uh.data_ptr(), rows, C, P, _abi.LEAP_MEMORY_HOST))
            ctx.calibrate_batched(items, dds, prec)

        w.e2e_step = e2e_step
        w.h2d = sum(vh.numel() * 8 + uh.numel() * 8 for vh, uh in hosts) + dds.nbytes
        w.d2h = D * S * 8
    else:
        w.e2e_step = None
    return w


def setup_differentiable(args, ctx, lg, torch, local, rank):
    """Forward + backward of the differentiable form: 128 antennas, 8 timesteps, 96 channels,
    16 directions, complex<float>; loss = sum of squared wrapped residuals to the gain phases,
    gradients with respect to every direction's (l, m) and the visibilities."""
    from leap_gb300 import synth
    from leap_gb300.autograd import calibrate_lm
    dev = f"cuda:{local}"
    w = Workload()
    nd = args.directions or 16
    obs, _ = synth.mwa_precision(timesteps=8, channels=96, directions=nd)
    _, lm = synth.random_directions(nd, seed=31 + 1000 * rank)
    md = lg.build_metadata(obs)
    ctx.set_metadata(md)
    vis = torch.from_numpy(obs.vis).to(dev).requires_grad_()
    uvw = torch.from_numpy(obs.uvw).to(dev)
    gain = torch.from_numpy(np.angle(obs.gains)).to(dev)
    lm_t = torch.from_numpy(lm).to(dev).requires_grad_()
    holder = {}

    def step(p):
        lm_t.grad = None
        vis.grad = None
        cal = calibrate_lm(ctx, 0, lm_t, vis, uvw, p)
        res = torch.atan2(torch.sin(cal - gain[None, :]), torch.cos(cal - gain[None, :]))
        (res * res).sum().backward()
        holder["cal"] = cal

    w.step = step
    w.result = lambda: holder["cal"].detach().cpu().numpy()
    w.kernel_timing = "events"
    w.extra_launches = 8  # leap_backward: 2 transposed contractions, cal1, 2 avgData, (l, m, n) + reduce, vis
    w.obs, w.dirs, w.md, w.D, w.S = obs, None, md, nd, md.A.shape[1]
    w.min_ndir = nd
    w.units = vis_dirs(obs, nd)
    w.b_alg = alg_bytes(4.0 * obs.rows * obs.channels, obs.rows, nd, obs.nbaselines, 4, 8)
    w.f_alg = fma_slots(obs.rows, obs.rows * obs.channels, nd, 4)
    w.name = (f"differentiable {obs.num_stations}ant/{obs.nbaselines}bl/{obs.timesteps}t/{obs.channels}ch/4pol/"
              f"{nd}dir c64: forward + FP64 adjoint (d/d(l,m) and d/dV)")
    w.config = {"workload": w.name, "precision": args.precision, "l2": "inputs (203 MB) larger than L2; no flush"}
    w.e2e_step = None
    dirs = synth.lm_to_radec(lm[:, 0], lm[:, 1])
    w.dirs = dirs
    w.cpu_case = (obs, dirs, obs.vis[:, :obs.nbaselines, :])
    return w


def run_gpu(args, rank: int, world: int):
    import torch
    import leap_gb300 as lg
    from leap_gb300 import _abi

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    ctx = lg.Context(local)
    if args.tc_rotation >= 0:
        ctx.set_option(_abi.LEAP_OPTION_TENSOR_CORE_ROTATION, args.tc_rotation)
    if args.gridded >= 0:
        ctx.set_option(_abi.LEAP_OPTION_GRIDDED_ROTATION, args.gridded)
    # A dedicated stream: the calls and the timing events go on the same (non-null) stream.
    bstream = torch.cuda.Stream(device=f"cuda:{local}")
    torch.cuda.set_stream(bstream)
    if args.workload == "batched":
        w = setup_batched(args, ctx, lg, torch, local, rank)
    elif args.workload == "differentiable":
        w = setup_differentiable(args, ctx, lg, torch, local, rank)
    else:
        w = setup_single(args, ctx, lg, torch, local, rank, args.workload)
    prec = lg.LEAP_PRECISION_MIXED if args.precision == "mixed" else lg.LEAP_PRECISION_FP64
    lib = _abi.lib

    def timed(p, steps, warmup):
        for _ in range(warmup):
            w.step(p)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        lib.leap_timing_reset(ctx.handle)
        e0.record()
        for _ in range(steps):
            w.step(p)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        t = _abi.LeapTimings()
        ctx._check(lib.leap_get_timings(ctx.handle, t))
        if w.kernel_timing == "total":
            # blocking host calls: the device time of each call, from its own events
            ms = t.total_ms / max(1, t.calls)
        if dist:
            tt = torch.tensor([ms], device=f"cuda:{local}")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            dist.barrier()
            ms = float(tt.item())
        return ms, t

    with ClockSampler(local) as clk:
        ms, tim = timed(prec, args.steps, args.warmup)
    clocks = clk.summary()
    value = w.units * world / (ms / 1e3)
    cal_main = w.result()
    gpu_launches = (int(tim.kernels) + getattr(w, "extra_launches", 0)) * args.steps

    # The rotate + average kernel this run used (the library's choice for LEAP_OPTION_GRIDDED_ROTATION).
    gridded = prec == lg.LEAP_PRECISION_MIXED and (
        args.gridded == 1 or (args.gridded in (-1, 2) and args.tc_rotation != 2 and w.min_ndir >= 32))
    alt_kernel = None
    if gridded and args.gridded != 1 and args.workload in ("mwa", "ska_low"):
        # The same call through the FP32 CUDA-core pipelined kernel, for comparison.
        ctx.set_option(_abi.LEAP_OPTION_GRIDDED_ROTATION, 0)
        ms_alt, _ = timed(prec, max(1, min(args.steps, 5)), 2)
        cal_alt = w.result()
        ctx.set_option(_abi.LEAP_OPTION_GRIDDED_ROTATION, 2)
        alt_kernel = {"kernel": "rotate_average_mixed_pipe (FP32 CUDA cores, compensated sums)", "ms_per_step": ms_alt,
                      "value": w.units * world / (ms_alt / 1e3),
                      "max_cal_diff_vs_gridded_rad": wrapped_max_diff(cal_main, cal_alt)}

    checks = {}
    plain = None
    if not args.skip_plain and prec == lg.LEAP_PRECISION_MIXED:
        ms64, _ = timed(lg.LEAP_PRECISION_FP64, max(1, min(args.steps, 3)), 1)
        cal64 = w.result()
        per_dir = np.abs(np.angle(np.exp(1j * (cal_main - cal64)))).max(axis=1)
        margin = branch_margins(ctx, w.md, w.D, torch, f"cuda:{local}", torch.cuda.current_stream().cuda_stream)
        near = margin < 1e-5
        plain = {"value": w.units * world / (ms64 / 1e3), "ms_per_step": ms64, "dtype": "f64",
                 "mixed_vs_fp64_max_cal_err_rad": float(per_dir[~near].max()) if (~near).any() else None,
                 "mixed_vs_fp64_cal_err_rad_median_p99": ([float(np.median(per_dir[~near])),
                                                           float(np.percentile(per_dir[~near], 99))]
                                                          if (~near).any() else None),
                 "directions_near_branch_cut": int(near.sum()),
                 "max_cal_err_rad_incl_branch_cut_directions": float(per_dir.max()),
                 "speedup_mixed_over_fp64": ms64 / ms,
                 "note": "directions whose FP64 solve has an arg() within 1e-5 rad of +-pi are counted apart: "
                         "the mixed form may put that angle on the other branch, which moves cal by 2*pi "
                         "times one column of Ad"}

    if rank == 0 and getattr(w, "spot", None) is not None and not args.skip_cpu:
        # Full-size spot check: the smallest chunk's directions against the oracle.
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        slot, obs_s, vis_s = w.spot
        sl, d0, nd = next(it for it in w.items if it[0] == slot)
        exp = oracle.calibrate_interval(vis_s, obs_s.uvw, w.dds[d0:d0 + nd], oracle.metadata(obs_s),
                                        nthreads=oracle.max_threads())
        checks["oracle_chunk"] = {"slot": slot, "timesteps": obs_s.timesteps, "channels": obs_s.channels,
                                  "directions": nd, "max_cal_err_rad": wrapped_max_diff(cal_main[d0:d0 + nd], exp)}

    e2e = None
    if w.e2e_step is not None:
        for _ in range(max(1, min(args.warmup, 2))):
            w.e2e_step()
        if dist:
            dist.barrier()
        e2e_steps = args.steps if args.workload == "mwa" else max(1, min(args.steps, 3))
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            w.e2e_step()
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        if dist:
            tt = torch.tensor([e2e_s], device=f"cuda:{local}")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            e2e_s = float(tt.item())
        e2e = {"value": w.units * world / e2e_s, "unit": "vis-directions/s", "h2d_bytes_per_step": int(w.h2d),
               "d2h_bytes_per_step": int(w.d2h), "ms_per_step": e2e_s * 1e3, "steps": e2e_steps,
               "mode": "serial: upload, then calibrate, each step"}
        pipe = getattr(w, "e2e_pipelined", None)
        if pipe is not None:
            pipe(2)
            if dist:
                dist.barrier()
            t0 = time.perf_counter()
            pipe(e2e_steps)
            pl_s = (time.perf_counter() - t0) / e2e_steps
            if dist:
                tt = torch.tensor([pl_s], device=f"cuda:{local}")
                dist.all_reduce(tt, op=dist.ReduceOp.MAX)
                pl_s = float(tt.item())
            e2e["serial"] = {"value": e2e["value"], "ms_per_step": e2e["ms_per_step"]}
            e2e.update({"value": w.units * world / pl_s, "ms_per_step": pl_s * 1e3,
                        "mode": "double-buffered: step k+1's upload overlaps step k's calibration; every step moves "
                                "its full input (host -> device) and result (device -> host)"})
        alt = getattr(w, "e2e_alt", None)
        if alt is not None:
            name, fn = alt
            fn()
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                fn()
            e2e[name] = {"value": w.units * world / ((time.perf_counter() - t0) / e2e_steps),
                         "ms_per_step": (time.perf_counter() - t0) / e2e_steps * 1e3}

    peaks = _peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    if w.kernel_timing == "rotate":
        k_ms = tim.rotate_ms / max(1, tim.calls)
        k_name = ("rotate_average (mixed: gridded kernel, 3xTF32 tcgen05 grid product + 10-point interpolation per "
                  "direction; compensated reference-antenna pass)" if gridded else
                  "rotate_average (mixed: persistent TMA-pipelined kernel + compensated reference-antenna pass)")
    elif w.kernel_timing == "events":
        k_ms = ms
        k_name = "whole forward + backward step"
    else:
        k_ms = ms
        k_name = "whole batched call (graph replay)"
    achieved = w.b_alg / (k_ms / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": w.traffic, "kernel": k_name, "kernel_ms": k_ms,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6.8 TB/s (of fallback)",
            "note": "B_alg counts the visibilities once per direction; the kernel reads them once for all directions",
            "compute": {"fp32_issue_per_s": w.f_alg / (k_ms / 1e3), "fp32_peak_fma_per_s": 3.6e13,
                        "frac": w.f_alg / (k_ms / 1e3) / 3.6e13}}
    if gridded and getattr(w, "grid_flops", None):
        # Tensor pipe: the kernel's 3xTF32 MMA FLOPs (from its grid windows) against the TF32
        # rate, half the measured dense BF16 rate.
        tf32_peak = (peaks["bf16_tflops"] / 2 if peaks and "bf16_tflops" in peaks else 950.0) * 1e12
        roof["compute"] = {"tensor_tf32_flops_per_s": w.grid_flops / (k_ms / 1e3), "tf32_peak_flops_per_s": tf32_peak,
                           "frac": w.grid_flops / (k_ms / 1e3) / tf32_peak, "mma_flops_per_call": w.grid_flops,
                           "peak_source": "half of MEASURED_PEAKS.json bf16_tflops (of measured)" if peaks else
                                          "half of the 1.9 PFLOP/s bf16 fallback (of fallback)"}
        roof["note"] = ("B_alg counts the visibilities once per direction (the reference's per-direction loop); the "
                        "gridded kernel reads them once for all directions (hbm_read_once_frac)")
    if hasattr(w, "vis_bytes_resident"):
        roof["hbm_read_once_frac"] = w.vis_bytes_resident / (k_ms / 1e3) / 1e9 / peak
    if gridded and getattr(w, "grid_traffic", None):
        roof["traffic"] = w.grid_traffic
    elif gridded:
        roof["traffic"] = None
    if roof["traffic"]:
        # the DRAM bytes the kernel actually moves (ncu-measured traffic) over its event time
        roof["dram_traffic_frac"] = roof["traffic"] / (k_ms / 1e3) / 1e9 / peak

    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        thr = oracle.max_threads()
        c_obs, c_dirs, c_vis = w.cpu_case
        v, samp = bench_cpu(c_obs, c_dirs, c_vis, thr, args.cpu_budget)
        v1, samp1 = bench_cpu(c_obs, c_dirs, c_vis, 1, args.cpu_budget / 5)
        cpu = {"value": v, "unit": "vis-directions/s", "cores": thr, "kind": "port",
               "sample": f"1 timestep ({c_obs.nbaselines} baselines x {c_obs.channels} channels) x "
                         f"{samp['directions']} of {w.D} directions, {samp['runs']} runs, {samp['seconds']:.1f} s",
               "single_core": {"value": v1, "cores": 1,
                               "sample": f"1 timestep x {samp1['directions']} directions, {samp1['runs']} runs, "
                                         f"{samp1['seconds']:.1f} s"}}

    if rank == 0:
        line = {
            "metric": "vis-directions/s", "value": value, "unit": "vis-directions/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 rotation + f64 phase arguments" if prec else "f64", "data": "synthetic",
            "config": w.config,
            "e2e": e2e,
            "gpu_launches": gpu_launches,
            "roofline": roof,
            "cpu_baseline": cpu,
            "plain_fp64": plain,
            "checks": checks or None,
            "alternative_kernel": alt_kernel,
            "metadata_build_s": round(getattr(w, "metadata_s", 0.0), 3),
            "metadata_build": "leap_build_metadata (device pseudo-inverse) + host copies of A and Ad for the checks",
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="mwa", choices=["mwa", "batched", "ska_low", "differentiable"],
                    help="mwa: 128 antennas, 14 t, 384 ch, 64 directions (default); batched: 32 uneven chunks, "
                         "256 directions; ska_low: 512 stations, 16 t, 384 ch, 128 directions")
    ap.add_argument("--timesteps", type=int, default=0, help="0: the workload's own count (MWA 14, SKA-Low 16)")
    ap.add_argument("--channels", type=int, default=384)
    ap.add_argument("--directions", type=int, default=0, help="0: the workload's own count")
    ap.add_argument("--chunks", type=int, default=32)
    ap.add_argument("--e2e", type=int, default=-1, help="1/0: force the host-buffer end-to-end timing on/off")
    ap.add_argument("--tc-rotation", type=int, default=-1,
                    help="tensor-core rotate + average: 0 never, 1 autotuned (library default), 2 always")
    ap.add_argument("--gridded", type=int, default=-1,
                    help="gridded rotate + average (tcgen05 grid product): 0 off, 1 on, -1 library default")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-plain", action="store_true")
    args = ap.parse_args()
    if args.directions == 0 and args.workload == "mwa":
        args.directions = 64
    if args.e2e < 0:
        args.e2e = 1 if args.workload == "mwa" else 0
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        if not os.path.exists(os.path.join(PKG, "leap_gb300", "_lib", "libleap_gb300.so")):
            sys.path.insert(0, PKG)
            import build as _b
            _b.build()
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
