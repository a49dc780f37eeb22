"""Several GPUs, one process per GPU (torch.distributed): the host side of the replica plan.

Frames of a batch and views of the differentiable renderer are independent units, so they are
dealt round-robin over the ranks and every rank renders its own share on its own GPU with no
exchange on the data path.  Results meet only on the host: timings as the maximum over ranks,
per-rank sums (the differentiable renderer's parameter gradients over views) as a host-staged
all-reduce.  Nothing here touches a GPU; the same calls run over `gloo` (CPU) and `nccl`.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np


def my_units(count: int, rank: int, world: int) -> List[int]:
    """The units (frames, views) of `count` that `rank` of `world` renders: rank, rank + world, ..."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return list(range(rank, count, world))


def _reduce(values: np.ndarray, op, dist, device) -> np.ndarray:
    import torch
    t = torch.from_numpy(np.ascontiguousarray(values)).to(device)
    dist.all_reduce(t, op=op)
    return t.cpu().numpy()


def _device(dist):
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def max_over_ranks(seconds: float, dist=None) -> float:
    """The largest of every rank's `seconds` (the job's time is its slowest rank's)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(seconds)
    return float(_reduce(np.array([seconds], np.float64), dist.ReduceOp.MAX, dist, _device(dist))[0])


def sum_over_ranks(arrays: Sequence[np.ndarray], dist=None) -> List[np.ndarray]:
    """Every rank's arrays added up element by element, returned on every rank (host-staged:
    one flat float64 buffer per call, so one collective however many arrays)."""
    arrays = [np.asarray(a, np.float64) for a in arrays]
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [a.copy() for a in arrays]
    flat = np.concatenate([a.reshape(-1) for a in arrays]) if arrays else np.zeros(0)
    total = _reduce(flat, dist.ReduceOp.SUM, dist, _device(dist))
    out, at = [], 0
    for a in arrays:
        out.append(total[at:at + a.size].reshape(a.shape))
        at += a.size
    return out


def gather_on_root(obj, dist=None, root: int = 0) -> Optional[list]:
    """Every rank's `obj` as a list on `root` (None elsewhere); [obj] without a process group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return [obj]
    rank = dist.get_rank()
    out = [None] * dist.get_world_size() if rank == root else None
    dist.gather_object(obj, out, dst=root)
    return out
