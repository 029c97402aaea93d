"""Work partitioning across ranks: one process per GPU, no collective on the data path.

Pixels are independent within a pass (AbstractImageKernel.java:273-283), so a frame splits into row
bands and a batch of scenes into whole-scene shards. The only exchanges are the gather of finished
film bands at read-out and the sum of gradient vectors of the adjoint; both go through
torch.distributed (NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

import numpy as np


def row_band(height: int, world: int, rank: int) -> tuple[int, int]:
    """Rows [r0, r1) of rank `rank`: contiguous bands whose sizes differ by at most one row."""
    if not (0 <= rank < world) or height < 0:
        raise ValueError(f"bad partition: height={height} world={world} rank={rank}")
    base, extra = divmod(height, world)
    r0 = rank * base + min(rank, extra)
    return r0, r0 + base + (1 if rank < extra else 0)


def scene_shard(costs, world: int, rank: int) -> list[int]:
    """Whole scenes for `rank`: longest-processing-time-first over the given per-scene costs."""
    load = [0.0] * world
    owner = {}
    for i in sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i)):
        r = min(range(world), key=lambda r: (load[r], r))
        owner[i] = r
        load[r] += float(costs[i])
    return sorted(i for i, r in owner.items() if r == rank)


def gather_film(band: np.ndarray, height: int, width: int, channels: int = 3):
    """Gathers each rank's row band (band rows x width x channels, float32) into the full film on
    rank 0 (other ranks get None)."""
    import torch
    import torch.distributed as dist

    world, rank = dist.get_world_size(), dist.get_rank()
    full_rows = max(row_band(height, world, r)[1] - row_band(height, world, r)[0] for r in range(world))
    padded = torch.zeros(full_rows, width, channels, dtype=torch.float32)
    r0, r1 = row_band(height, world, rank)
    padded[: r1 - r0] = torch.from_numpy(np.ascontiguousarray(band, dtype=np.float32))
    if dist.get_backend() == "nccl":
        padded = padded.cuda()
    parts = [torch.zeros_like(padded) for _ in range(world)] if rank == 0 else None
    dist.gather(padded, parts, dst=0)
    if rank != 0:
        return None
    out = np.zeros((height, width, channels), np.float32)
    for r in range(world):
        a, b = row_band(height, world, r)
        out[a:b] = parts[r][: b - a].cpu().numpy()
    return out


def allreduce_sum(values: np.ndarray) -> np.ndarray:
    """Sum of a float64 vector over all ranks (the gradient reduction of the adjoint)."""
    import torch
    import torch.distributed as dist

    t = torch.from_numpy(np.ascontiguousarray(values, dtype=np.float64))
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()
