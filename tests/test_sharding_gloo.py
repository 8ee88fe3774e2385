"""Direction sharding over processes (world size 2, gloo, CPU): each rank
calibrates its contiguous direction range (the oracle stands in for the
per-rank GPU calibration here) and rank 0 gathers the cal vectors; the result
equals the single-process calibration of all directions exactly."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from leap_gb300.sharding import shard_range


def test_shard_range_covers_each_direction_once():
    for count in (0, 1, 5, 64, 257):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in shard_range(count, world, r)]
            assert got == list(range(count))
            sizes = [len(shard_range(count, world, r)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, ndir, out_path):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "icrar-leap-accelerate_gb300"), os.path.join(root, "oracle")]
    import torch.distributed as dist
    import oracle
    from leap_gb300 import synth
    from leap_gb300.sharding import calibrate_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    obs, dirs = synth.small_case(stations=9, timesteps=2, channels=5, directions=ndir, seed_shift=3)
    mdo = oracle.metadata(obs)
    dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs])
    cal = calibrate_sharded(lambda part: oracle.calibrate_interval(obs.vis, obs.uvw, part, mdo, nthreads=1), dds,
                            mdo.Ad.shape[0])
    if rank == 0:
        np.save(out_path, cal)
    else:
        assert cal is None
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("ndir", [5, 1])
def test_gather_equals_single_process(tmp_path, ndir):
    import oracle
    from leap_gb300 import synth
    out = str(tmp_path / "cal.npy")
    mp.start_processes(_worker, args=(2, _free_port(), ndir, out), nprocs=2, join=True, start_method="spawn")
    obs, dirs = synth.small_case(stations=9, timesteps=2, channels=5, directions=ndir, seed_shift=3)
    mdo = oracle.metadata(obs)
    dds = np.stack([oracle.dd_matrix(*obs.phase_centre, r, d) for r, d in dirs])
    exp = oracle.calibrate_interval(obs.vis, obs.uvw, dds, mdo, nthreads=1)
    np.testing.assert_array_equal(np.load(out), exp)
