"""Direction sharding with the GPU calibrator: two gloo ranks (separate processes, both
on cuda:0, whose kernels are independent of each other) each calibrate their
shard_range of the directions through GpuLeapCalibrator, and rank 0 gathers the cal
vectors with calibrate_sharded (the in-process form of the reference's
ProduceConfig -> CallLeap -> LeapGather scale-out, R/leap_drops/ProduceConfig.py:71-93,
CallLeap.py:70-84, LeapGather.py:47-54).

The gathered result must equal, bit for bit, what one process computes for the same
shards, and match one single-process call over all directions and the oracle within
the form's tolerance."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import oracle
import leap_gb300 as lg
from leap_gb300 import synth
from leap_gb300.sharding import shard_range
from test_gpu_parity import assert_cal_close

pytestmark = pytest.mark.gpu

CASE = dict(stations=48, timesteps=3, channels=40, directions=11, vis_dtype=np.complex64, seed_shift=17)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _calibrate(cal, obs, dirs, precision):
    """cal vectors (D, S) of one GpuLeapCalibrator call over `dirs` (all timesteps)."""
    out = cal.calibrate(obs, dirs, (0, -1, -1))
    return np.array([b["beamCalibration"] for b in out[0]["calibration"]]).reshape(len(dirs), -1)


def _worker(rank, world, port, precision, out_path):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "icrar-leap-accelerate_gb300"), os.path.join(root, "oracle")]
    import numpy as np
    import torch.distributed as dist
    import leap_gb300 as lg
    from leap_gb300 import synth
    from leap_gb300.sharding import calibrate_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    obs, dirs = synth.small_case(**CASE)
    cal = lg.GpuLeapCalibrator(0, precision)

    def calibrate_rows(part):
        # calibrate_sharded hands this rank its rows of the direction matrices; the
        # calibrator takes (ra, dec), so calibrate the same rows of `dirs`.
        rows = shard_range(len(dirs), world, rank)
        assert part.shape[0] == len(rows)
        return _calibrate(cal, obs, dirs[rows.start:rows.stop], precision)

    dds = np.zeros((len(dirs), 3, 3))
    got = calibrate_sharded(calibrate_rows, dds, obs.num_stations)
    if rank == 0:
        np.save(out_path, got)
    else:
        assert got is None
    cal.ctx.close()
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("precision,tol", [(lg.LEAP_PRECISION_FP64, 1e-10), (lg.LEAP_PRECISION_MIXED, 1e-5)],
                         ids=["fp64", "mixed"])
def test_sharded_gpu_calibration_gathers_exactly(tmp_path, precision, tol):
    out = str(tmp_path / "cal.npy")
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), precision, out), nprocs=world, join=True,
                       start_method="spawn")
    gathered = np.load(out)
    obs, dirs = synth.small_case(**CASE)
    cal = lg.GpuLeapCalibrator(0, precision)
    per_shard = np.concatenate([_calibrate(cal, obs, dirs[r.start:r.stop], precision)
                                for r in (shard_range(len(dirs), world, k) for k in range(world))])
    whole = _calibrate(cal, obs, dirs, precision)
    cal.ctx.close()
    assert gathered.shape == (len(dirs), obs.num_stations)
    np.testing.assert_array_equal(gathered, per_shard)
    assert np.abs(gathered - whole).max() <= tol
    mdo = oracle.metadata(obs)
    dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs])
    cal_o, avg_o = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo, return_avg=True)
    assert_cal_close(gathered, cal_o, avg_o, mdo, tol)
