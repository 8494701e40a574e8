"""Several GPUs on one survey: shots are independent (wem.c:141-176 and the per-shot
workers of ShotProfileWEM.jl:104-106), so each rank migrates a contiguous block of
shots on its own GPU and the partial images are added once at the end -- the stacking
of ShotProfileWEM.jl:140-199 as one all-reduce of an nx*ny*nz FP32 image. Modelling
(demigration) needs no exchange at all: each rank models its own shots.

The per-rank operator is any callable shots -> image (normally Context.migrate on the
rank's device); the sum goes through torch.distributed (NCCL between GPUs, gloo on the
host).
"""
from __future__ import annotations

import numpy as np

from .api import Shots


def shard_bounds(nshot: int, rank: int, world: int) -> tuple[int, int]:
    """[first, last) shots of `rank`: contiguous blocks whose sizes differ by at most one
    (every shot costs the same nfreq * nz units)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    q, r = divmod(nshot, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def shard_shots(shots: Shots, rank: int, world: int) -> Shots:
    """The rank's block of shots with its traces, offsets rebased to 0."""
    lo, hi = shard_bounds(shots.nshot, rank, world)
    t0, t1 = int(shots.trace_offset[lo]), int(shots.trace_offset[hi])
    return Shots(np.asarray(shots.sx[lo:hi]), np.asarray(shots.sy[lo:hi]),
                 np.asarray(shots.trace_offset[lo:hi + 1], np.int64) - t0,
                 np.asarray(shots.trace_cell[t0:t1]), np.asarray(shots.data[t0:t1]))


def migrate_sharded(migrate, shots: Shots, rank: int, world: int, group=None, device=None) -> np.ndarray:
    """Migrate this rank's block of `shots` with `migrate` and add the partial images of
    all ranks (in float64 on the host path, so the sum does not depend on the order the
    collective adds in beyond FP64 rounding). Returns the full image on every rank."""
    import torch
    import torch.distributed as dist
    part = shard_shots(shots, rank, world)
    img = migrate(part) if part.nshot > 0 else None
    if img is None:
        raise ValueError("every rank needs at least one shot (world > nshot)")
    if world == 1:
        return img
    backend = dist.get_backend(group)
    if backend == "nccl":
        t = torch.from_numpy(np.ascontiguousarray(img)).to(device or torch.device("cuda", torch.cuda.current_device()))
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        return t.cpu().numpy()
    t = torch.from_numpy(np.ascontiguousarray(img, dtype=np.float64))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy().astype(np.float32)
