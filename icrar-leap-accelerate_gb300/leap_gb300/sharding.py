"""Direction sharding across processes (one GPU per process).

Directions are independent given the visibilities
(LA/algorithm/cpu/CpuLeapCalibrator.cc:132-139), so a calibration over many
directions splits into contiguous direction ranges, one per rank, with no
device collective: every rank holds its own copy of the metadata and of the
integration, calibrates its range, and the per-direction cal vectors
(D x S doubles) are gathered on the host.  This is the in-process form of the
reference's own process-level scale-out (R/leap_drops/ProduceConfig.py:71-93 ->
CallLeap.py:70-84 -> LeapGather.py:47-54).
"""
from __future__ import annotations

from typing import Callable, List, Optional, Sequence

import numpy as np


def shard_range(count: int, world: int, rank: int) -> range:
    """Contiguous, balanced range of `count` items for `rank` of `world` (the first
    count % world ranks take one extra; a rank may get none)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(count, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def gather_rows(local: np.ndarray, count: int, group=None, dst: int = 0) -> Optional[np.ndarray]:
    """Gather each rank's rows (its shard_range of `count`) on rank `dst`, in rank order.
    Host-side only (torch.distributed object gather: gloo or nccl process groups)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    parts = [None] * world if rank == dst else None
    dist.gather_object(np.ascontiguousarray(local), parts, dst=dst, group=group)
    if rank != dst:
        return None
    width = next((p.shape[1] for p in parts if p.ndim == 2 and p.shape[0]), local.shape[1] if local.ndim == 2 else 0)
    out = np.concatenate([p.reshape(-1, width) for p in parts], axis=0)
    if out.shape[0] != count:
        raise RuntimeError(f"gathered {out.shape[0]} rows, expected {count}")
    return out


def calibrate_sharded(calibrate: Callable[[np.ndarray], np.ndarray], dds: np.ndarray, stations: int,
                      group=None) -> Optional[np.ndarray]:
    """Run `calibrate(dds_shard) -> (n, stations)` on this rank's directions and gather
    all cal vectors on rank 0 (None on the other ranks)."""
    import torch.distributed as dist
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    mine = shard_range(len(dds), world, rank)
    local = calibrate(dds[mine.start:mine.stop]) if len(mine) else np.zeros((0, stations))
    return gather_rows(np.asarray(local, dtype=np.float64).reshape(-1, stations), len(dds), group)
