"""Benchmark of the GB300 LEAP calibration hot path.

Metric: vis-directions/s — one visibility sample (pol, row, channel) phase-
rotated and averaged for one calibration direction, through the whole path
(rotate + average, phase angles, both pseudoinverse contractions).

Headline workload (default): the batched uneven workload — 128 antennas (8256
baselines with autocorrelations), 32 integration chunks with timesteps uniform
in 1..64 and channels from {48, 96, 384} (seed 4), 4 pols, complex<float>
(52.3 GB resident), 256 directions dealt round-robin to the chunks, one
leap_calibrate_batched call per step (graph replay).  Synthetic, seeded, the
visibilities generated on the device.  Inputs are larger than L2 (129 MB), so
no L2 flush is needed between steps.

The JSON line:
  value        inputs resident in HBM, mixed-precision form, the library's CUDA
               events on its stream around each call (exactly --steps calls)
  e2e          the same call through the C ABI from host buffers: every step
               uploads each chunk from page-locked host memory
               (leap_set_integration) and reads the cal phases back
  roofline     the bulk rotate + average kernel: the bytes it must move (each
               sample read once, UVWs, one avgData write) over its event-timed
               duration, against the measured HBM copy rate; the per-direction
               convention (every direction re-reading the cube) beside it
  plain_fp64   the all-FP64 form on the same workload
  checks       both forms against the oracle over every chunk and direction
               (branch choices at arg() cuts proved, oracle/branch_cuts.py)
  cpu_baseline the oracle (C restatement of CpuLeapCalibrator, OpenMP over
               (chunk, direction) pairs) on a bounded sample: the first timestep
               of every chunk with all its directions
  sub_results  the 128-antenna 14-timestep workload (64 directions), the
               512-station SKA-Low-like workload (128 directions), the
               reference's own direction spread, and the C++ drop-in call
               (LeapCalibratorFactory::Create(gb300)->Calibrate) — each with its
               own roofline, FP64 comparison and oracle checks

``--impl reference`` times the reference CPU algorithm (the oracle port of
CpuLeapCalibrator; the reference itself cannot be built here) on all host cores
on the same sample, with the same config; it maps no product library.
Multi-GPU (torchrun): the direction set grows with the rank count; each rank
calibrates its shard_range of it and rank 0 gathers the cal vectors
(leap_gb300.sharding.calibrate_sharded) — weak scaling, host-side gather only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "icrar-leap-accelerate_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG)

MIXED_TOL = 1e-5      # cal-phase bar of the mixed form against the FP64 oracle (rad)
FP64_TOL = 1e-10      # bar of the all-FP64 form
BRANCH_MARGIN = 1e-4  # angles this close to +-pi may take either branch in the mixed form


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


def _oracle():
    if ORACLE_DIR not in sys.path:
        sys.path.insert(0, ORACLE_DIR)
    import oracle
    return oracle


def mapped_libraries():
    """Shared objects of this repository mapped into the process."""
    try:
        maps = open("/proc/self/maps").read().split("\n")
    except OSError:
        return None
    real = os.path.realpath(ROOT)
    libs = sorted({ln.split()[-1] for ln in maps if ln.strip().endswith(".so") and real in ln})
    return [os.path.relpath(p, real) for p in libs]


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


# ---------------------------------------------------------------------------
# Workload definitions shared by both arms
# ---------------------------------------------------------------------------

def batched_shapes(args):
    from leap_gb300 import synth
    return synth.uneven_chunks(args.chunks, seed=4)


def workload_config(name: str, args) -> dict:
    """The `config` of a workload; both arms print the same one."""
    if name == "batched":
        shapes = batched_shapes(args)
        nd = args.directions or 256
        gb = sum(s.timesteps * s.channels for s in shapes) * 8256 * 4 * 8 / 1e9
        return {"workload": f"batched_uneven 128ant/8256bl, {len(shapes)} chunks (T 1-64, C in 48/96/384, seed 4; "
                            f"{sum(s.timesteps for s in shapes)} timesteps), {nd} directions round-robin, 4pol "
                            f"complex<float> ({gb:.1f} GB)",
                "chunks": [[s.timesteps, s.channels] for s in shapes], "precision": args.precision,
                "l2": f"inputs ({gb:.1f} GB) larger than L2; no flush"}
    if name == "mwa":
        t = args.timesteps or 14
        nd = args.directions or 64
        gb = t * 8256 * args.channels * 4 * 8 / 1e9
        return {"workload": f"mwa_precision 128ant/8256bl/{t}t/{args.channels}ch/4pol/{nd}dir complex<float>",
                "precision": args.precision, "l2": f"inputs ({gb:.2f} GB) larger than L2; no flush"}
    if name == "ska_low":
        t = args.timesteps or 16
        nd = args.directions or 128
        return {"workload": f"ska_low 512st/131328bl/{t}t/384ch/4pol/{nd}dir complex<float>", "precision": args.precision,
                "l2": f"inputs ({t * 131328 * 384 * 32 / 1e9:.1f} GB) larger than L2; no flush"}
    if name == "differentiable":
        return {"workload": "differentiable 128ant/8256bl/8t/96ch/4pol/16dir complex<float>: forward + FP64 adjoint "
                            "(d/d(l,m) and d/dV)", "precision": args.precision,
                "l2": "inputs (203 MB) larger than L2; no flush"}
    raise ValueError(name)


class CpuSample:
    """A bounded sample of a workload for the oracle, on host memory: chunks of
    (vis (channels, rows, pols), uvw (rows, 3), dds (D, 3, 3)), one metadata."""

    def __init__(self, chunks, mdo, description):
        self.chunks = chunks
        self.mdo = mdo
        self.description = description
        self.units = float(sum(v.shape[0] * v.shape[1] * v.shape[2] * d.shape[0] for v, _, d in chunks))

    def run(self, threads: int):
        _oracle().calibrate_items(self.chunks, self.mdo, nthreads=threads)


def cpu_sample(name: str, args) -> CpuSample:
    """The oracle's sample of workload `name`: the same in the reference arm and in the
    gb300 arm's cpu_baseline."""
    from leap_gb300 import synth
    oracle = _oracle()
    if name == "batched":
        obs_list, dirs, items, _ = synth.batched_uneven(chunks=args.chunks, directions=args.directions or 256,
                                                        sample_timesteps=1)
        mdo = oracle.metadata(obs_list[0])
        dds = np.stack([oracle.dd_matrix(*obs_list[0].phase_centre, r, d) for r, d in dirs])
        chunks = [(obs_list[sl].vis, obs_list[sl].uvw, dds[d0:d0 + n]) for sl, d0, n in items]
        return CpuSample(chunks, mdo, f"the first timestep of each of the {len(items)} chunks with all its "
                                      f"directions ({len(dirs)} directions in all)")
    if name in ("mwa", "differentiable"):
        if name == "mwa":
            obs, dirs = synth.mwa_precision(timesteps=1, channels=args.channels, directions=args.directions or 64)
        else:
            obs, _ = synth.mwa_precision(timesteps=1, channels=96, directions=16)
            _, lm = synth.random_directions(16, seed=31)
            dirs = synth.lm_to_radec(lm[:, 0], lm[:, 1])
        mdo = oracle.metadata(obs)
        dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs])
        return CpuSample([(obs.vis, obs.uvw, dds)], mdo, f"1 timestep x all {len(dirs)} directions")
    if name == "ska_low":
        obs, dirs = synth.ska_low(timesteps=1, directions=args.directions or 128)
        mdo = oracle.metadata(obs)
        dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs[:16]])
        return CpuSample([(obs.vis, obs.uvw, dds)], mdo, "1 timestep x 16 directions")
    raise ValueError(name)


def time_cpu_sample(sample: CpuSample, threads: int, budget_s: float):
    sample.run(threads)  # warm-up
    runs, total = 0, 0.0
    while total < budget_s or runs == 0:
        t0 = time.perf_counter()
        sample.run(threads)
        total += time.perf_counter() - t0
        runs += 1
    return sample.units * runs / total, runs, total


def run_reference(args, name: str, rank: int, world: int):
    """The reference's CPU algorithm (the oracle port) on the host cores; rank 0 only."""
    if rank != 0:
        return
    oracle = _oracle()
    threads = oracle.max_threads()
    sample = cpu_sample(name, args)
    for _ in range(args.warmup):
        sample.run(threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sample.run(threads)
    dt = (time.perf_counter() - t0) / args.steps
    value = sample.units / dt
    line = {
        "impl": "reference", "metric": "vis-directions/s", "value": value, "unit": "vis-directions/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(name, args),
        "cpu_baseline": {"value": value, "unit": "vis-directions/s", "cores": threads, "kind": "port",
                         "sample": f"each step: {sample.description} ({sample.units:.3g} vis-directions)"},
        "e2e": {"value": value, "unit": "vis-directions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "libraries_mapped": mapped_libraries(),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Parity against the oracle (after the timed regions)
# ---------------------------------------------------------------------------

def compare_with_oracle(cal: np.ndarray, cal_o: np.ndarray, avg_o: np.ndarray, mdo, tol: float, margin: float):
    """Per-direction max |cal - cal_oracle|; directions over `tol` must be a branch choice at
    an arg() within `margin` of +-pi (proved by re-solving the oracle's avgData)."""
    import branch_cuts
    err = np.abs(cal - cal_o).max(axis=1)
    flips, unexplained, rest = 0, [], []
    proved = np.zeros(err.shape, dtype=bool)
    for d in np.flatnonzero(err > tol):
        ok, _, r = branch_cuts.explain(cal[d], avg_o[d][:, 0], mdo, tol, margin)
        if ok:
            flips += 1
            rest.append(r)
            proved[d] = True
        else:
            unexplained.append(int(d))
    # Every direction counts except those proved to be a branch choice.
    plain = err[~proved] if (~proved).any() else err
    return {"directions": int(len(err)), "max_rad": float(plain.max()), "median_rad": float(np.median(plain)),
            "p99_rad": float(np.percentile(plain, 99)), "max_incl_branch_choices_rad": float(err.max()),
            "branch_choices": flips, "max_after_branch_choice_rad": float(max(rest)) if rest else None,
            "unexplained_directions": unexplained, "tolerance_rad": tol, "pass": not unexplained}


def metadata_check(md, mdo) -> dict:
    """The library's pseudo-inverses (built on the device) against the oracle's."""
    return {"Ad_max_abs_diff": float(np.abs(md.Ad - mdo.Ad).max()),
            "Ad1_max_abs_diff": float(np.abs(md.Ad1 - mdo.Ad1).max()),
            "Ad_max_abs": float(np.abs(mdo.Ad).max()), "A_equal": bool(np.array_equal(md.A, mdo.A)),
            "I_equal": bool(np.array_equal(md.I, mdo.I)), "I1_equal": bool(np.array_equal(md.I1, mdo.I1))}


def oracle_checks(chunks, cal_mixed, cal_fp64, mdo, threads: int, what: str):
    """chunks: [(vis, uvw, dds, row slice of the cal arrays)]."""
    oracle = _oracle()
    t0 = time.perf_counter()
    cals, avgs = oracle.calibrate_items([(v, u, d) for v, u, d, _ in chunks], mdo, nthreads=threads, return_avg=True)
    t_o = time.perf_counter() - t0
    cal_o = np.concatenate(cals)
    avg_o = np.concatenate(avgs)
    rows = np.concatenate([np.arange(s.start, s.stop) for *_, s in chunks])
    out = {"sample": what, "oracle_s": round(t_o, 1)}
    if cal_mixed is not None:
        out["mixed"] = compare_with_oracle(cal_mixed[rows], cal_o, avg_o, mdo, MIXED_TOL, BRANCH_MARGIN)
    if cal_fp64 is not None:
        out["fp64"] = compare_with_oracle(cal_fp64[rows], cal_o, avg_o, mdo, FP64_TOL, 1e-8)
    return out


# ---------------------------------------------------------------------------
# Device workloads
# ---------------------------------------------------------------------------

class Workload:
    """One workload resident on the device.  step(precision) launches one pass of the hot path."""
    name = ""
    units = 0.0            # vis-directions per step
    kernel_bytes = 0.0     # bytes the bulk kernel must move per launch (each sample once)
    per_direction_bytes = 0.0  # the per-direction convention: every direction reads the cube
    traffic = None         # ncu-measured DRAM bytes per launch of the bulk kernel, if known
    kernel_name = ""
    grid = None            # (tensor-core FLOPs per call, mean and max grid passes) of the gridded kernel
    timing = "events"      # "events": torch events on the bench stream; "library": the library's own events
    e2e_step = None
    h2d = d2h = 0
    extra_launches = 0

    def close(self):
        pass


def read_once_bytes(samples: float, rows: float, nbl: int, ndir: int) -> float:
    """Each complex<float> sample once, the split UVWs (24 B per row), one FP64 avgData write."""
    return samples * 8 + rows * 24 + ndir * nbl * 4 * 16


def per_direction_bytes(samples: float, rows: float, nbl: int, ndir: int) -> float:
    """The reference's per-direction loop: every direction reads the cube and 24 B of UVW per row."""
    return ndir * (samples * 8 + rows * 24) + ndir * nbl * 4 * 16


def grid_windows_host(obs, dds: np.ndarray, taps: int = 10, jw_max: int = 64, stride: int = 48, load: int = 11):
    """The gridded kernel's grid windows of one call, computed as its grid_windows kernel does
    (one window per quad of baselines over all directions): (tensor-core FLOPs per call, mean
    passes per tile, max passes)."""
    C, nbl, T = obs.channels, obs.nbaselines, obs.timesteps
    n, lbase = 2 * C, ((C + taps + 8 + 7) // 8) * 8
    nchunk = (C + 15) // 16
    kb = -(dds[:, 2, :] - np.array([0.0, 0.0, 1.0])) * obs.freq_inc_hz / 299792458.0  # (D, 3) turns per metre
    uvw = obs.uvw.reshape(T, nbl, 3)
    nquad = (nbl + 3) // 4
    flops, passes, tiles, pmax = 0.0, 0.0, 0.0, 0
    for d0 in range(0, 1):
        B = np.einsum("tbj,dj->tbd", uvw, kb)
        B = B - np.rint(B)
        s = np.floor(B * n).astype(np.int64) - taps // 2 + 1  # stencil start
        pad = nquad * 4 - nbl
        smin = np.pad(s.min(axis=(0, 2)), (0, pad), constant_values=1 << 40).reshape(nquad, 4).min(axis=1)
        smax = np.pad(s.max(axis=(0, 2)), (0, pad), constant_values=-(1 << 40)).reshape(nquad, 4).max(axis=1)
        r0 = ((smin + lbase) >> 3) * 8
        need = smax + load + lbase - r0
        single = need <= jw_max
        jw = np.where(single, np.maximum(8, (need + 7) & ~7), jw_max)
        npass = np.where(single, 1, (smax + lbase - r0) // stride + 1)
        ntb = (T + 3) // 4
        flops += float((ntb * npass * nchunk * 3 * 2 * 128 * 2 * jw * 16).sum())  # 3 FP16 MMAs, K = 16, per chunk
        passes += float((ntb * npass).sum())
        tiles += float(ntb * nquad)
        pmax = max(pmax, int(npass.max()))
    return flops, passes / tiles, pmax


def setup_batched(run, dir_ids=None) -> Workload:
    """32 uneven integration chunks, their directions dealt round-robin; one
    leap_calibrate_batched call per step."""
    from leap_gb300 import synth
    args, ctx, lg, torch = run.args, run.ctx, run.lg, run.torch
    nd = args.directions or 256
    obs_list, dirs, items, _ = synth.batched_uneven(chunks=args.chunks, directions=nd, direction_ids=dir_ids)
    w = Workload()
    w.name = "batched"
    t0 = time.perf_counter()
    md = ctx.build_metadata(obs_list[0])
    w.metadata_s = time.perf_counter() - t0
    keep_host = bool(args.e2e) or (run.rank == 0 and not args.skip_checks)
    hosts = []
    for i, obs in enumerate(obs_list):
        vis = synth.device_visibilities(obs, run.dev, seed=2000 + i)
        ctx.set_integration(i, vis, torch.from_numpy(obs.uvw).to(run.dev))
        if keep_host:
            vh = torch.empty(vis.shape, dtype=vis.dtype, pin_memory=True)
            vh.copy_(vis)
            hosts.append((vh, torch.from_numpy(obs.uvw).pin_memory()))
        del vis
    torch.cuda.empty_cache()
    dds = np.stack([lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs])
    D, S = len(dirs), md.A.shape[1]
    holder = {}

    def step(p):
        holder["cal"] = ctx.calibrate_batched(items, dds, p)

    w.step = step
    w.result = lambda: holder["cal"].copy()
    w.timing = "library"
    w.obs_list, w.items, w.dds, w.md, w.D, w.S = obs_list, items, dds, md, D, S
    w.units = sum(4.0 * obs_list[sl].rows * obs_list[sl].channels * n for sl, _, n in items)
    samples = {sl: 4.0 * obs_list[sl].rows * obs_list[sl].channels for sl, _, _ in items}
    w.kernel_bytes = sum(read_once_bytes(samples[sl], obs_list[sl].rows, 8256, n) for sl, _, n in items)
    w.per_direction_bytes = sum(per_direction_bytes(samples[sl], obs_list[sl].rows, 8256, n) for sl, _, n in items)
    w.vis_bytes = sum(samples.values()) * 8
    w.kernel_name = ("rotate_average_mixed_pipe<8,4,4> (persistent, TMA-pipelined, 4 tiles x 8 directions per block; "
                     "FP32 CUDA cores with compensated sums) + the rotate stage's small kernels")
    # DRAM traffic of the bulk kernel, from an ncu capture (dram__bytes_read.sum +
    # dram__bytes_write.sum) of the same kernel on 4 timesteps of the 128-antenna array with 8
    # directions: 408.99 MB read for 405.80 MB of visibilities (the rest is the split UVWs), a few
    # MB of partial-sum writes.  Reads scale with the visibilities; writes taken as one avgData.
    w.traffic = w.vis_bytes * (408.99 / 405.80) + sum(n * 8256 * 4 * 16 for _, _, n in items)
    w.hosts = hosts
    w.min_ndir = min(n for _, _, n in items)
    if args.e2e and hosts:
        prec = lg.LEAP_PRECISION_MIXED if args.precision == "mixed" else lg.LEAP_PRECISION_FP64
        from leap_gb300 import _abi

        def e2e_step():
            for i, (vh, uh) in enumerate(hosts):
                C, rows, P = vh.shape
                ctx._check(_abi.lib.leap_set_integration(ctx.handle, i, _abi.LEAP_VIS_C64, vh.data_ptr(),
                                                         uh.data_ptr(), rows, C, P, _abi.LEAP_MEMORY_HOST))
            ctx.calibrate_batched(items, dds, prec)

        w.e2e_step = e2e_step
        w.e2e_mode = ("serial: every step uploads all 32 chunks from page-locked host memory (leap_set_integration), "
                      "then one leap_calibrate_batched call returns the cal phases to host memory")
        w.h2d = sum(vh.numel() * 8 + uh.numel() * 8 for vh, uh in hosts) + dds.nbytes
        w.d2h = D * S * 8

    def checks(cal_mixed, cal_fp64, threads):
        mdo = _oracle().metadata(obs_list[0])
        chunks = [(hosts[sl][0].numpy(), obs_list[sl].uvw, dds[d0:d0 + n], slice(d0, d0 + n)) for sl, d0, n in items]
        out = oracle_checks(chunks, cal_mixed, cal_fp64, mdo, threads,
                            f"every chunk (all {sum(o.timesteps for o in obs_list)} timesteps) x all {D} directions")
        out["metadata"] = metadata_check(md, mdo)
        return out

    w.checks = checks if hosts else None
    return w


def setup_single(run, kind: str, dir_ids=None) -> Workload:
    """One integration, all directions in one leap_calibrate_async call."""
    from leap_gb300 import synth
    args, ctx, lg, torch = run.args, run.ctx, run.lg, run.torch
    w = Workload()
    w.name = kind
    if kind == "mwa":
        obs, dirs = synth.mwa_precision(timesteps=args.timesteps or 14, channels=args.channels,
                                        directions=args.directions or 64)
        vis_np = obs.vis
        vis_dev = torch.from_numpy(vis_np).to(run.dev)
    else:
        obs, dirs = synth.ska_low(with_vis=False, timesteps=args.timesteps or 16, directions=args.directions or 128)
        vis_dev = synth.device_visibilities(obs, run.dev, seed=2)
        vis_np = vis_dev.cpu().numpy() if (run.rank == 0 and not args.skip_checks) else None
    if dir_ids is not None:
        dirs = dirs[dir_ids]
    t0 = time.perf_counter()
    md = ctx.build_metadata(obs)
    w.metadata_s = time.perf_counter() - t0
    uvw_host = torch.from_numpy(obs.uvw).pin_memory()
    ctx.set_integration(0, vis_dev, uvw_host.to(run.dev))
    del vis_dev
    torch.cuda.empty_cache()
    dds = np.stack([lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs])
    D, S = len(dirs), md.A.shape[1]
    dd_dev = torch.from_numpy(dds.reshape(-1)).to(run.dev)
    cal_dev = torch.empty((D, S), dtype=torch.float64, device=run.dev)
    stream = torch.cuda.current_stream().cuda_stream

    def step(p):
        ctx.calibrate_async(0, dd_dev.data_ptr(), D, p, cal_dev.data_ptr(), stream)

    w.step = step
    w.result = lambda: cal_dev.cpu().numpy().copy()
    w.obs, w.dirs, w.dds, w.md, w.D, w.S = obs, dirs, dds, md, D, S
    w.min_ndir = D
    samples = 4.0 * obs.rows * obs.channels
    w.units = samples * D
    w.kernel_bytes = read_once_bytes(samples, obs.rows, obs.nbaselines, D)
    w.per_direction_bytes = per_direction_bytes(samples, obs.rows, obs.nbaselines, D)
    w.vis_bytes = samples * 8
    w.grid = grid_windows_host(obs, dds)
    # DRAM traffic of one launch of the gridded kernel, from an ncu capture
    # (dram__bytes_read.sum + dram__bytes_write.sum) of the 4-timestep case of this
    # workload: 101.8 MB read per timestep (the visibilities, once) + 26.9 MB of sum
    # writes, scaled to the timesteps of this run.
    if kind == "mwa" and obs.nbaselines == 8256 and obs.channels == 384 and D == 64:
        w.grid_traffic = 101.80e6 * obs.timesteps + 26.94e6
        w.pipe_traffic = 101.74e6 * obs.timesteps + 44.74e6

    def checks(cal_mixed, cal_fp64, threads):
        if vis_np is None:
            return None
        mdo = _oracle().metadata(obs)
        if kind == "mwa":
            sel, what = slice(0, D), f"all {D} directions x all {obs.timesteps} timesteps"
        else:
            sel, what = slice(0, min(D, 16)), f"the first {min(D, 16)} directions x all {obs.timesteps} timesteps"
        out = oracle_checks([(vis_np, obs.uvw, dds[sel], sel)], cal_mixed, cal_fp64, mdo, threads, what)
        out["metadata"] = metadata_check(md, mdo)
        return out

    w.checks = checks
    if kind == "mwa" and args.e2e:
        # The host holds the visibilities in MeasurementSet order, [row][channel][pol]
        # (page-locked); each step ingests them through leap_set_integration_ms, which
        # transposes on the device, then calibrates with host dd / cal buffers.
        vis_host = torch.from_numpy(vis_np)
        ms_host = torch.empty((vis_host.shape[1], vis_host.shape[0], vis_host.shape[2]), dtype=vis_host.dtype,
                              pin_memory=True)
        ms_host.copy_(vis_host.permute(1, 0, 2))
        uvw_np = uvw_host.numpy()
        cal_host = np.zeros((D, S), dtype=np.float64)
        C, rows, P = vis_np.shape
        prec = lg.LEAP_PRECISION_MIXED if args.precision == "mixed" else lg.LEAP_PRECISION_FP64
        from leap_gb300 import _abi
        lib = _abi.lib

        def e2e_step():
            ctx._check(lib.leap_set_integration_ms(ctx.handle, 0, _abi.LEAP_VIS_C64, ms_host.data_ptr(), C, 0,
                                                   uvw_np.ctypes.data, rows, C, P, _abi.LEAP_MEMORY_HOST))
            ctx._check(lib.leap_calibrate(ctx.handle, 0, dds.ctypes.data, D, prec, cal_host.ctypes.data))

        def e2e_pipelined(n):
            # Double-buffered: the upload of step k+1's visibilities (asynchronous, copy stream) overlaps
            # the calibration of step k; every step still moves its full input and output.
            ctx._check(lib.leap_set_integration_ms_async(ctx.handle, 0, _abi.LEAP_VIS_C64, ms_host.data_ptr(), C, 0,
                                                         uvw_host.data_ptr(), rows, C, P, _abi.LEAP_MEMORY_HOST))
            for k in range(n):
                if k + 1 < n:
                    ctx._check(lib.leap_set_integration_ms_async(ctx.handle, (k + 1) % 2, _abi.LEAP_VIS_C64,
                                                                 ms_host.data_ptr(), C, 0, uvw_host.data_ptr(), rows,
                                                                 C, P, _abi.LEAP_MEMORY_HOST))
                ctx._check(lib.leap_calibrate(ctx.handle, k % 2, dds.ctypes.data, D, prec, cal_host.ctypes.data))

        w.e2e_step = e2e_step
        w.e2e_pipelined = e2e_pipelined
        w.e2e_mode = "serial: upload (MeasurementSet order, transposed on the device), then calibrate, each step"
        w.h2d = vis_np.nbytes + obs.uvw.nbytes + dds.nbytes
        w.d2h = cal_host.nbytes
    return w


def setup_differentiable(run) -> Workload:
    """Forward + backward of the differentiable form: 128 antennas, 8 timesteps, 96 channels,
    16 directions, complex<float>; loss = sum of squared wrapped residuals to the gain phases,
    gradients with respect to every direction's (l, m) and the visibilities."""
    from leap_gb300 import synth
    from leap_gb300.autograd import calibrate_lm
    args, ctx, lg, torch = run.args, run.ctx, run.lg, run.torch
    w = Workload()
    w.name = "differentiable"
    nd = args.directions or 16
    obs, _ = synth.mwa_precision(timesteps=8, channels=96, directions=nd)
    _, lm = synth.random_directions(nd, seed=31 + 1000 * run.rank)
    md = lg.build_metadata(obs)
    ctx.set_metadata(md)
    vis = torch.from_numpy(obs.vis).to(run.dev).requires_grad_()
    uvw = torch.from_numpy(obs.uvw).to(run.dev)
    gain = torch.from_numpy(np.angle(obs.gains)).to(run.dev)
    lm_t = torch.from_numpy(lm).to(run.dev).requires_grad_()
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
    w.timing = "events"
    w.whole_step_is_kernel = True
    w.extra_launches = 8  # leap_backward: 2 transposed contractions, cal1, 2 avgData, (l, m, n) + reduce, vis
    w.md, w.D, w.S, w.min_ndir = md, nd, md.A.shape[1], nd
    samples = 4.0 * obs.rows * obs.channels
    w.units = samples * nd
    w.kernel_bytes = read_once_bytes(samples, obs.rows, obs.nbaselines, nd)
    w.per_direction_bytes = per_direction_bytes(samples, obs.rows, obs.nbaselines, nd)
    w.vis_bytes = samples * 8
    w.kernel_name = "whole forward + backward step"
    w.checks = None
    return w


class Run:
    """Device, context and stream of one workload run."""

    def __init__(self, args, torch, lg, local, rank, world, dist):
        self.args, self.torch, self.lg = args, torch, lg
        self.local, self.rank, self.world, self.dist = local, rank, world, dist
        self.dev = f"cuda:{local}"
        self.ctx = lg.Context(local)
        from leap_gb300 import _abi
        if args.tc_rotation >= 0:
            self.ctx.set_option(_abi.LEAP_OPTION_TENSOR_CORE_ROTATION, args.tc_rotation)
        if args.gridded >= 0:
            self.ctx.set_option(_abi.LEAP_OPTION_GRIDDED_ROTATION, args.gridded)
        if args.grid_shared >= 0:
            self.ctx.set_option(_abi.LEAP_OPTION_GRID_SHARED_GROUPS, args.grid_shared)

    def timed(self, w: Workload, p: int, steps: int, warmup: int):
        """W untimed steps, then exactly `steps` steps between barriers and synchronisations;
        CUDA events on the launching stream (or the library's own events on its stream for
        blocking batched calls); max over ranks."""
        torch, dist = self.torch, self.dist
        from leap_gb300 import _abi
        lib = _abi.lib
        for _ in range(warmup):
            w.step(p)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        lib.leap_timing_reset(self.ctx.handle)
        e0.record()
        for _ in range(steps):
            w.step(p)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        t = _abi.LeapTimings()
        self.ctx._check(lib.leap_get_timings(self.ctx.handle, t))
        if w.timing == "library":
            ms = t.total_ms / max(1, t.calls)  # blocking calls on the library's stream: its own events
        if dist:
            tt = torch.tensor([ms], device=self.dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            dist.barrier()
            ms = float(tt.item())
        return ms, t

    def close(self):
        self.ctx.close()
        self.torch.cuda.synchronize()
        self.torch.cuda.empty_cache()


def kernel_time(run: Run, w: Workload, p: int, ms: float, tim) -> float:
    """Event-timed duration of the rotate + average stage (the bulk kernel and the small kernels
    launched with it on the same stream) per call."""
    from leap_gb300 import _abi
    if getattr(w, "whole_step_is_kernel", False):
        return ms
    if w.timing == "library":
        # Graph replays record no event between the stages: time eager calls of the same launches.
        run.ctx.set_option(_abi.LEAP_OPTION_GRAPH_REPLAY, 0)
        try:
            _, t = run.timed(w, p, 5, 1)
        finally:
            run.ctx.set_option(_abi.LEAP_OPTION_GRAPH_REPLAY, 1)
        return t.rotate_ms / max(1, t.calls)
    return tim.rotate_ms / max(1, tim.calls)


def roofline(w: Workload, k_ms: float, gridded: bool, peaks) -> dict:
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = w.kernel_bytes / (k_ms / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": w.traffic, "kernel": w.kernel_name, "kernel_ms": k_ms,
            "algorithmic_bytes_per_launch": w.kernel_bytes,
            "algorithmic_bytes": "each complex<float> sample read once (8 B), the split UVWs (24 B per row), one "
                                 "FP64 avgData write per (baseline, pol, direction)",
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6.8 TB/s (of fallback)",
            "per_direction_convention": {
                "bytes": w.per_direction_bytes, "frac": w.per_direction_bytes / (k_ms / 1e3) / 1e9 / peak,
                "note": "the reference's per-direction loop reads the cube once per direction; this kernel reads it "
                        "once for all directions, so this figure is not a roofline fraction"}}
    if gridded and w.grid is not None:
        flops, mean_pass, max_pass = w.grid
        f16_peak = (peaks["bf16_tflops"] if peaks and "bf16_tflops" in peaks else 1900.0) * 1e12
        roof["tensor"] = {"f16_flops_per_s": flops / (k_ms / 1e3), "peak_flops_per_s": f16_peak,
                          "frac": flops / (k_ms / 1e3) / f16_peak, "mma_flops_per_call": flops,
                          "grid_passes_per_tile_mean": mean_pass, "grid_passes_max": max_pass,
                          "peak_source": "MEASURED_PEAKS.json bf16_tflops (the dense FP16 rate, of measured)" if peaks
                          else "the 1.9 PFLOP/s bf16 fallback (of fallback)"}
    if roof["traffic"]:
        roof["dram_traffic_frac"] = roof["traffic"] / (k_ms / 1e3) / 1e9 / peak
    return roof


def uses_gridded(args, w, p, lg) -> bool:
    return p == lg.LEAP_PRECISION_MIXED and (args.gridded == 1 or (
        args.gridded in (-1, 2) and args.tc_rotation != 2 and w.min_ndir >= 32))


def time_e2e(run: Run, w: Workload, steps: int):
    torch, dist = run.torch, run.dist
    for _ in range(2):
        w.e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        w.e2e_step()
    e2e_s = (time.perf_counter() - t0) / steps
    if dist:
        tt = torch.tensor([e2e_s], device=run.dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())
    e2e = {"value": w.units * run.world / e2e_s, "unit": "vis-directions/s", "h2d_bytes_per_step": int(w.h2d),
           "d2h_bytes_per_step": int(w.d2h), "ms_per_step": e2e_s * 1e3, "steps": steps, "mode": w.e2e_mode}
    pipe = getattr(w, "e2e_pipelined", None)
    if pipe is not None:
        pipe(2)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        pipe(steps)
        pl_s = (time.perf_counter() - t0) / steps
        e2e["serial"] = {"value": e2e["value"], "ms_per_step": e2e["ms_per_step"]}
        e2e.update({"value": w.units * run.world / pl_s, "ms_per_step": pl_s * 1e3,
                    "mode": "double-buffered: step k+1's upload overlaps step k's calibration; every step moves "
                            "its full input (host -> device) and result (device -> host)"})
    return e2e


def run_workload(name, args, torch, lg, local, rank, world, dist, steps, warmup, headline=False):
    """Time one workload and measure everything reported about it."""
    from leap_gb300.sharding import shard_range
    run = Run(args, torch, lg, local, rank, world, dist)
    bstream = torch.cuda.Stream(device=run.dev)  # calls and timing events on one non-null stream
    torch.cuda.set_stream(bstream)
    dir_ids = None
    if world > 1:
        # Weak scaling: the direction set grows with the ranks; each rank takes its shard.
        per = args.directions or {"batched": 256, "mwa": 64, "ska_low": 128}.get(name, 16)
        dir_ids = np.asarray(shard_range(per * world, world, rank))
    if name == "batched":
        w = setup_batched(run, dir_ids)
    elif name == "differentiable":
        w = setup_differentiable(run)
    else:
        w = setup_single(run, name, dir_ids)
    prec = lg.LEAP_PRECISION_MIXED if args.precision == "mixed" else lg.LEAP_PRECISION_FP64
    with ClockSampler(local) as clk:
        ms, tim = run.timed(w, prec, steps, warmup)
    out = {"ms_per_step": ms, "value": w.units * world / (ms / 1e3), "clocks": clk.summary(),
           "gpu_launches": (int(tim.kernels) + w.extra_launches) * steps, "config": workload_config(name, args)}
    cal_main = w.result()
    gridded = uses_gridded(args, w, prec, lg)
    if gridded and name in ("mwa", "ska_low"):
        w.kernel_name = ("rotate_average_gridded<10> (3xFP16 tcgen05 grid product + 10-point interpolation per "
                         "direction) + grid_windows + the compensated reference-antenna pass")
        w.traffic = getattr(w, "grid_traffic", None)
    elif name in ("mwa", "ska_low"):
        w.kernel_name = "rotate_average_mixed_pipe (persistent, TMA-pipelined, FP32 CUDA cores, compensated sums)"
        w.traffic = getattr(w, "pipe_traffic", None)
    if not gridded:
        w.grid = None
    k_ms = kernel_time(run, w, prec, ms, tim)
    out["roofline"] = roofline(w, k_ms, gridded, _peaks())
    if gridded and args.gridded != 1 and name in ("mwa", "ska_low"):
        # The same call through the FP32 CUDA-core pipelined kernel, for comparison.
        from leap_gb300 import _abi
        run.ctx.set_option(_abi.LEAP_OPTION_GRIDDED_ROTATION, 0)
        ms_alt, t_alt = run.timed(w, prec, max(1, min(steps, 5)), 2)
        cal_alt = w.result()
        run.ctx.set_option(_abi.LEAP_OPTION_GRIDDED_ROTATION, 2)
        out["alternative_kernel"] = {
            "kernel": "rotate_average_mixed_pipe (FP32 CUDA cores, compensated sums)", "ms_per_step": ms_alt,
            "kernel_ms": t_alt.rotate_ms / max(1, t_alt.calls), "value": w.units * world / (ms_alt / 1e3),
            "max_cal_diff_vs_gridded_rad": float(np.abs(cal_main - cal_alt).max())}
    if gridded and name == "ska_low" and args.grid_shared < 0 and w.D > 64:
        # The other arrangement of the direction groups (one grid product per tile for all groups).
        from leap_gb300 import _abi
        run.ctx.set_option(_abi.LEAP_OPTION_GRID_SHARED_GROUPS, 1)
        ms_sh, t_sh = run.timed(w, prec, max(1, min(steps, 5)), 2)
        run.ctx.set_option(_abi.LEAP_OPTION_GRID_SHARED_GROUPS, 0)
        out["alternative_grouping"] = {
            "grouping": "one grid product per tile for both groups of 64 directions (one-tile units)",
            "ms_per_step": ms_sh, "kernel_ms": t_sh.rotate_ms / max(1, t_sh.calls),
            "max_cal_diff_rad": float(np.abs(w.result() - cal_main).max())}
    cal64 = None
    if not args.skip_plain and prec == lg.LEAP_PRECISION_MIXED:
        n64 = 1 if name == "ska_low" else max(1, min(steps, 3))
        ms64, _ = run.timed(w, lg.LEAP_PRECISION_FP64, n64, 1)
        cal64 = w.result()
        per_dir = np.abs(cal_main - cal64).max(axis=1)
        out["plain_fp64"] = {"value": w.units * world / (ms64 / 1e3), "ms_per_step": ms64, "dtype": "f64",
                             "speedup_mixed_over_fp64": ms64 / ms,
                             "mixed_vs_fp64_cal_rad": {"max": float(per_dir.max()),
                                                       "median": float(np.median(per_dir)),
                                                       "p99": float(np.percentile(per_dir, 99))}}
    if rank == 0 and not args.skip_checks and w.checks is not None:
        out["checks"] = w.checks(cal_main, cal64, _oracle().max_threads())
    if w.e2e_step is not None:
        out["e2e"] = time_e2e(run, w, max(1, min(steps, 3)) if name == "batched" else steps)
    if world > 1:
        from leap_gb300.sharding import calibrate_sharded
        holder = {}

        def cal_fn(part):
            t0 = time.perf_counter()
            w.step(prec)
            r = w.result()
            holder["cal_s"] = time.perf_counter() - t0
            return r

        t0 = time.perf_counter()
        gathered = calibrate_sharded(cal_fn, np.zeros((per * world, 3, 3)), w.S)
        total = time.perf_counter() - t0
        out["sharding"] = {"directions_total": per * world, "directions_per_rank": len(dir_ids),
                           "gather_s": total - holder.get("cal_s", 0.0),
                           "gathered_rows": None if gathered is None else int(gathered.shape[0])}
    out["metadata_build_s"] = round(getattr(w, "metadata_s", 0.0), 3)
    w.close()
    del w
    run.close()
    return out


def run_reference_directions(args, torch, lg, local):
    """The reference's own direction spread (E2EPerformanceTests.cc:65-76: nine directions up
    to ~1 rad from the phase centre of its MWA test set) on the 128-antenna array, 14 timesteps,
    384 channels: the gridded kernel (forced on) and the pipelined kernel against the oracle."""
    from leap_gb300 import synth, _abi
    kats = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_kats.json")))
    pc = tuple(kats["dd"]["phase_centre"])
    dirs = np.asarray(kats["e2e_directions"]["radec"], dtype=np.float64)
    obs = synth.mwa_at_phase_centre(pc, timesteps=args.timesteps or 14, channels=args.channels)
    ctx = lg.Context(local)
    md = ctx.build_metadata(obs)
    ctx.set_integration(0, obs.vis, obs.uvw)
    dds = np.stack([lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs])
    out = {"source": kats["e2e_directions"]["source"], "phase_centre": list(pc), "directions": int(len(dirs)),
           "workload": f"128ant/8256bl/{obs.timesteps}t/{obs.channels}ch/4pol complex<float>"}
    flops, mean_pass, max_pass = grid_windows_host(obs, dds)
    cals = {}
    for label, opt in (("gridded", 1), ("pipelined", 0)):
        ctx.set_option(_abi.LEAP_OPTION_GRIDDED_ROTATION, opt)
        ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED)
        ctx.timing_reset()
        for _ in range(5):
            cals[label] = ctx.calibrate(0, dds, lg.LEAP_PRECISION_MIXED)
        t = ctx.timings()
        out[label] = {"ms_per_call": t["total_ms"] / t["calls"], "kernel_ms": t["rotate_ms"] / t["calls"]}
    out["gridded"].update({"grid_passes_per_tile_mean": mean_pass, "grid_passes_max": max_pass,
                           "mma_flops_per_call": flops})
    cal64 = ctx.calibrate(0, dds, lg.LEAP_PRECISION_FP64)
    ctx.close()
    oracle = _oracle()
    mdo = oracle.metadata(obs)
    (cal_o,), (avg_o,) = oracle.calibrate_items([(obs.vis, obs.uvw, dds)], mdo, return_avg=True)
    for label in ("gridded", "pipelined"):
        out[label]["vs_oracle"] = compare_with_oracle(cals[label], cal_o, avg_o, mdo, MIXED_TOL, BRANCH_MARGIN)
    out["fp64_vs_oracle"] = compare_with_oracle(cal64, cal_o, avg_o, mdo, FP64_TOL, 1e-8)
    return out


def run_dropin(args):
    """The C++ drop-in call, LeapCalibratorFactory::Create(gb300)->Calibrate, on the 128-antenna
    14-timestep workload written as a .leapms file: Slice(1) (one solution per timestep) and
    Slice(-1) (one solution for all), mixed form, 64 directions."""
    from leap_gb300 import synth
    import leap_gb300 as lg
    exe = os.path.join(os.path.dirname(lg.LIB_PATH), "leap_dropin_bench")
    obs, dirs = synth.mwa_precision(timesteps=args.timesteps or 14, channels=args.channels,
                                    directions=args.directions or 64)
    out = {"call": "LeapCalibratorFactory::Create(ComputeImplementation::gb300)->Calibrate(ms, directions, slice, "
                   "0.0, nullopt, false), mixed form",
           "workload": f"128ant/8256bl/{obs.timesteps}t/{obs.channels}ch/4pol/{len(dirs)}dir complex<float>, "
                       "MeasurementSet stand-in in host memory"}
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "mwa.leapms")
        synth.write_leapms(obs, path)
        units = 4.0 * obs.rows * obs.channels * len(dirs)
        for label, s in (("slice_1", "1"), ("slice_all", "-1")):
            r = subprocess.run([exe, "-f", path, "-d", json.dumps(dirs.tolist()), "-s", s, "-p", "mixed",
                                "--warmup", "2", "--repeat", "5"], capture_output=True, text=True, timeout=900)
            if r.returncode != 0:
                raise RuntimeError(f"leap_dropin_bench failed: {r.stderr}")
            res = json.loads(r.stdout.strip().splitlines()[-1])
            ms = statistics.median(res["ms_per_call"])
            out[label] = {"ms_per_call_median": ms, "ms_per_call": res["ms_per_call"], "solutions": res["solutions"],
                          "value": units / (ms / 1e3), "unit": "vis-directions/s",
                          "h2d_bytes_per_call": res["visibility_bytes"]}
    return out


def run_gpu(args, rank: int, world: int):
    import torch
    import leap_gb300 as lg

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    headline = "batched" if args.workload == "all" else args.workload
    head = run_workload(headline, args, torch, lg, local, rank, world, dist, args.steps, args.warmup, headline=True)
    subs = {}
    if args.workload == "all" and world == 1 and not args.skip_sub:
        saved = (args.directions, args.timesteps)
        args.directions, args.timesteps = 0, 0
        for name in ("mwa", "ska_low"):
            subs[name] = run_workload(name, args, torch, lg, local, rank, world, dist, max(3, min(args.steps, 10)), 3)
        subs["reference_directions"] = run_reference_directions(args, torch, lg, local)
        subs["dropin"] = run_dropin(args)
        args.directions, args.timesteps = saved
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        oracle = _oracle()
        thr = oracle.max_threads()
        sample = cpu_sample(headline, args)
        v, runs, secs = time_cpu_sample(sample, thr, args.cpu_budget)
        v1, runs1, secs1 = time_cpu_sample(sample, 1, args.cpu_budget / 5) if headline != "batched" else (None, 0, 0)
        cpu = {"value": v, "unit": "vis-directions/s", "cores": thr, "kind": "port",
               "sample": f"{sample.description} ({sample.units:.3g} vis-directions), {runs} runs, {secs:.1f} s"}
        if v1:
            cpu["single_core"] = {"value": v1, "cores": 1, "sample": f"same, {runs1} runs, {secs1:.1f} s"}
    if rank == 0:
        prec_mixed = args.precision == "mixed"
        line = {
            "metric": "vis-directions/s", "value": head["value"], "unit": "vis-directions/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 rotation + f64 phase arguments" if prec_mixed else "f64", "data": "synthetic",
            "config": head["config"],
            "e2e": head.get("e2e"),
            "gpu_launches": head["gpu_launches"],
            "roofline": head["roofline"],
            "cpu_baseline": cpu,
            "plain_fp64": head.get("plain_fp64"),
            "checks": head.get("checks"),
            "sharding": head.get("sharding"),
            "alternative_kernel": head.get("alternative_kernel"),
            "alternative_grouping": head.get("alternative_grouping"),
            "metadata_build_s": head["metadata_build_s"],
            "sub_results": subs or None,
            "clocks": head["clocks"],
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="all", choices=["all", "batched", "mwa", "ska_low", "differentiable"],
                    help="all (default): the batched workload as the headline, with the 128-antenna, SKA-Low, "
                         "reference-direction and drop-in results beside it; otherwise that workload alone")
    ap.add_argument("--timesteps", type=int, default=0, help="0: the workload's own count (MWA 14, SKA-Low 16)")
    ap.add_argument("--channels", type=int, default=384)
    ap.add_argument("--directions", type=int, default=0, help="0: the workload's own count")
    ap.add_argument("--chunks", type=int, default=32)
    ap.add_argument("--e2e", type=int, default=-1, help="1/0: force the host-buffer end-to-end timing on/off")
    ap.add_argument("--tc-rotation", type=int, default=-1,
                    help="tensor-core rotate + average: 0 never, 1 autotuned (library default), 2 always")
    ap.add_argument("--gridded", type=int, default=-1,
                    help="gridded rotate + average (tcgen05 grid product): 0 off, 1 on, -1 library default")
    ap.add_argument("--grid-shared", type=int, default=-1,
                    help="gridded kernel, > 64 directions: 1 one grid product per tile for all direction groups, "
                         "0 one per group, -1 library default")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-checks", action="store_true", help="no oracle comparison")
    ap.add_argument("--skip-sub", action="store_true", help="headline only")
    args = ap.parse_args()
    if args.e2e < 0:
        args.e2e = 1 if args.workload in ("all", "batched", "mwa") else 0
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    headline = "batched" if args.workload == "all" else args.workload
    if args.impl == "reference":
        run_reference(args, headline, rank, world)
        return
    if not os.path.exists(os.path.join(PKG, "leap_gb300", "_lib", "libleap_gb300.so")):
        import build as _b
        _b.build()
    run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
