"""Several GPUs of one node, one process per GPU.

The all-pairs path shards by targets: every target's result depends on all
sources and on nothing else, so ranks hold all sources (replicated once) and
compute disjoint, contiguous target ranges; the results are concatenated by
one all-gather. No data-path collective is needed otherwise. The reference
has no multi-device path (its OpenCL code uses the first enabled device,
src/ocl_P3D.cpp:46).

* target_range: the balanced contiguous split used by every rank.
* sharded_p3d_vel_dvort: velocity and stretching of a particle set with the
  targets split across the ranks of the default process group; each rank
  calls the C ABI on its shard (GPU or host path, whichever the library has
  enabled) and all ranks receive the full result.
* max_over_ranks: the slowest rank's time (whole-job time of a replicated or
  sharded step).
"""
from __future__ import annotations

import os

import numpy as np


def dist_env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def target_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous range [lo, hi) of rank `rank`: sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _all_gather_rows(local: np.ndarray, n_total: int, world: int) -> np.ndarray:
    import torch
    import torch.distributed as dist
    width = local.shape[1]
    chunk = -(-n_total // world)
    pad = np.zeros((chunk, width), local.dtype)
    pad[: len(local)] = local
    parts = [torch.empty((chunk, width), dtype=torch.float32) for _ in range(world)]
    dist.all_gather(parts, torch.from_numpy(pad))
    rows = []
    for r, t in enumerate(parts):
        lo, hi = target_range(n_total, r, world)
        rows.append(t.numpy()[: hi - lo])
    return np.concatenate(rows, axis=0)


def sharded_p3d_vel_dvort(cv, particles: np.ndarray, reg: str, sigma: float):
    """(vel, dvort) of every particle of `particles` on itself, targets split
    across the ranks of the default process group (CPU tensors for the
    gather: gloo, or NCCL with the results moved to the host)."""
    import torch.distributed as dist
    rank, world = dist.get_rank(), dist.get_world_size()
    lo, hi = target_range(len(particles), rank, world)
    shard = np.ascontiguousarray(particles[lo:hi])
    vel = cv.p3d_vel(particles, shard["coord"], reg, sigma)
    dv = cv.p3d_dvort(particles, shard, reg, sigma)
    return (_all_gather_rows(vel, len(particles), world),
            _all_gather_rows(dv, len(particles), world))


def max_over_ranks(value: float, device: str = "cpu") -> float:
    """Maximum of `value` over the ranks of the default group (identity
    without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
