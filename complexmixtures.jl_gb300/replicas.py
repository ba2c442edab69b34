"""Replicas across GPUs: frames are sharded by contiguous ranges, each rank
runs its own engine, and the exact int64 counts are summed once at the end.

This is the reference's chunk model (src/mddf.jl:287-338 with sum!,
src/results.jl:629-649) spread over processes: integer sums are
order-independent, so any sharding gives the single-process counts.  There is
no exchange on the data path; the only collective is the final sum.
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np


def frame_range(nframes: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous [start, stop) of frames for one rank (sizes differ by <= 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(nframes, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def allreduce_counts(counts: Dict[str, np.ndarray], group=None) -> Dict[str, np.ndarray]:
    """Sum int64 (or FP64) count arrays over the ranks of a torch.distributed
    process group (any backend that reduces CPU tensors, e.g. gloo)."""
    import torch
    import torch.distributed as dist

    out = {}
    for k in sorted(counts):
        v = counts[k]
        if not isinstance(v, np.ndarray):
            t = torch.tensor([v], dtype=torch.float64)
            dist.all_reduce(t, group=group)
            out[k] = type(v)(t.item())
            continue
        t = torch.from_numpy(np.ascontiguousarray(v)).clone()
        dist.all_reduce(t, group=group)
        out[k] = t.numpy()
    return out
