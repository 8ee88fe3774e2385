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
  e2e        the public C ABI with host buffers: per step the pinned host->device
             upload of the step's visibilities + UVWs (leap_set_integration), the
             calibration (leap_calibrate) and the device->host read of the cal phases
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
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

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
    obs, dirs = synth.mwa_precision(timesteps=args.timesteps, channels=args.channels, directions=args.directions)
    if rank:
        # Each rank calibrates its own directions (same array and integration).
        _, lm = synth.random_directions(args.directions, seed=3 + 1000 * rank)
        dirs = synth.lm_to_radec(lm[:, 0], lm[:, 1])
    return obs, dirs


def vis_dirs(obs, ndir: int) -> float:
    return float(obs.pols) * obs.rows * obs.channels * ndir


def bench_cpu(obs, dirs, md_host, threads: int, budget_s: float):
    """Oracle port on a bounded sample: the first timesteps and directions of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    mdo = oracle.metadata(obs)
    nbl = obs.nbaselines
    t_s = 1
    d_s = max(1, min(len(dirs), threads))
    vis = np.ascontiguousarray(obs.vis[:, : t_s * nbl, :])
    uvw = obs.uvw[: t_s * nbl]
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
    units = float(obs.pols) * vis.shape[1] * obs.channels * d_s
    return units / dt, {"timesteps": t_s, "directions": d_s, "seconds": dt}


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

    obs, dirs = make_workload(args, rank)
    md = lg.build_metadata(obs)
    ctx = lg.Context(local)
    ctx.set_metadata(md)
    dds = np.stack([lg.dd_matrix(md.phase_centre_ra_rad, md.phase_centre_dec_rad, r, d) for r, d in dirs])
    D, S = len(dirs), md.A.shape[1]

    vis_host = torch.from_numpy(obs.vis).pin_memory()
    uvw_host = torch.from_numpy(obs.uvw).pin_memory()
    vis_dev = vis_host.to(f"cuda:{local}")
    uvw_dev = uvw_host.to(f"cuda:{local}")
    ctx.set_integration(0, vis_dev, uvw_dev)
    dd_dev = torch.from_numpy(dds.reshape(-1)).to(f"cuda:{local}")
    cal_dev = torch.empty((D, S), dtype=torch.float64, device=f"cuda:{local}")
    # A dedicated stream: the calls and the timing events go on the same (non-null) stream.
    bstream = torch.cuda.Stream(device=f"cuda:{local}")
    torch.cuda.set_stream(bstream)
    stream = bstream.cuda_stream
    prec = lg.LEAP_PRECISION_MIXED if args.precision == "mixed" else lg.LEAP_PRECISION_FP64

    def step(p):
        ctx.calibrate_async(0, dd_dev.data_ptr(), D, p, cal_dev.data_ptr(), stream)

    def timed(p, steps, warmup):
        for _ in range(warmup):
            step(p)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        lib = _abi.lib
        lib.leap_timing_reset(ctx.handle)
        e0.record()
        for _ in range(steps):
            step(p)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        t = _abi.LeapTimings()
        lib.leap_get_timings(ctx.handle, t)
        if dist:
            tt = torch.tensor([ms], device=f"cuda:{local}")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            dist.barrier()
            ms = float(tt.item())
        return ms, t

    with ClockSampler(local) as clk:
        ms, tim = timed(prec, args.steps, args.warmup)
    clocks = clk.summary()
    units = vis_dirs(obs, D)
    value = units * world / (ms / 1e3)
    cal_mixed = cal_dev.cpu().numpy().copy()

    # plain FP64 on the same workload
    plain = None
    if not args.skip_plain and prec == lg.LEAP_PRECISION_MIXED:
        ms64, _ = timed(lg.LEAP_PRECISION_FP64, max(1, min(args.steps, 3)), 1)
        cal64 = cal_dev.cpu().numpy().copy()
        err = float(np.abs(np.angle(np.exp(1j * (cal_mixed - cal64)))).max())
        plain = {"value": units * world / (ms64 / 1e3), "ms_per_step": ms64, "dtype": "f64",
                 "mixed_vs_fp64_max_cal_err_rad": err}

    # e2e through the C ABI with host buffers
    cal_host = np.zeros((D, S), dtype=np.float64)
    vis_np = vis_host.numpy()
    uvw_np = uvw_host.numpy()
    C, rows, P = obs.vis.shape

    def e2e_step():
        ctx._check(_abi.lib.leap_set_integration(ctx.handle, 0, _abi.LEAP_VIS_C64, vis_np.ctypes.data, uvw_np.ctypes.data,
                                                 rows, C, P, _abi.LEAP_MEMORY_HOST))
        ctx._check(_abi.lib.leap_calibrate(ctx.handle, 0, dds.ctypes.data, D, prec, cal_host.ctypes.data))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / args.steps
    if dist:
        tt = torch.tensor([e2e_s], device=f"cuda:{local}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())
    h2d = obs.vis.nbytes + obs.uvw.nbytes + dds.nbytes
    d2h = cal_host.nbytes

    # roofline of the rotate+average kernel (SURVEY convention: s_vis bytes per vis-direction
    # + 24 B of UVW per row and direction + the FP64 avgData write)
    peaks = _peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    rot_ms = tim.rotate_ms / max(1, tim.calls)
    vis_bytes = obs.vis.itemsize
    b_alg = D * (units / D * vis_bytes + obs.rows * 24) + D * obs.nbaselines * P * 16
    achieved = b_alg / (rot_ms / 1e3) / 1e9
    fp32_ops = D * obs.rows * obs.channels * (P * 4 + 5)  # FMA-pipe issue slots per (row, channel, direction)
    # DRAM traffic of one launch of the bulk kernel, from an ncu capture
    # (dram__bytes_read.sum + dram__bytes_write.sum) of the 2-timestep case of this
    # workload: 101.7 MB read per timestep (the visibilities, once) + 44.7 MB of
    # partial-sum writes, scaled to the timesteps of this run.
    traffic = (101.74e6 * obs.timesteps + 44.74e6) if (obs.nbaselines == 8256 and obs.channels == 384 and D == 64) else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "kernel": "rotate_average", "kernel_ms": rot_ms,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6.8 TB/s",
            "note": "B_alg counts the vis once per direction; the kernel reads it once for all directions",
            "compute": {"fp32_issue_per_s": fp32_ops / (rot_ms / 1e3), "fp32_peak_fma_per_s": 3.6e13,
                        "frac": fp32_ops / (rot_ms / 1e3) / 3.6e13}}

    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        thr = oracle.max_threads()
        v, samp = bench_cpu(obs, dirs, md, thr, args.cpu_budget)
        cpu = {"value": v, "unit": "vis-directions/s", "cores": thr, "kind": "port",
               "sample": f"{samp['timesteps']} of {obs.timesteps} timesteps x {samp['directions']} of {D} directions, "
                         f"{samp['seconds']:.1f} s"}

    if rank == 0:
        line = {
            "metric": "vis-directions/s", "value": value, "unit": "vis-directions/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 rotation + f64 phase arguments" if prec else "f64",
            "data": "synthetic",
            "config": {"workload": f"mwa_precision {obs.num_stations}ant/{obs.nbaselines}bl/{obs.timesteps}t/"
                                   f"{obs.channels}ch/{P}pol/{D}dir c64",
                       "precision": args.precision, "l2": "inputs (1.42 GB) larger than L2; no flush"},
            "e2e": {"value": units * world / e2e_s, "unit": "vis-directions/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3},
            "gpu_launches": int(tim.kernels) * args.steps,
            "roofline": roof,
            "cpu_baseline": cpu,
            "plain_fp64": plain,
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
    ap.add_argument("--timesteps", type=int, default=14)
    ap.add_argument("--channels", type=int, default=384)
    ap.add_argument("--directions", type=int, default=64)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-plain", action="store_true")
    args = ap.parse_args()
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
