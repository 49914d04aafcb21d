"""Column sharding across ranks (one process per GPU).

Columns are independent, so a multi-GPU run gives each rank a contiguous
column range, replicates the tree and model, and needs no data-path
collective; results are concatenated along the column axis (the last axis of
every output).  ``gather_columns`` does that concatenation with one
all_gather when the caller wants the full result on every rank.
"""
from __future__ import annotations

import numpy as np


def column_range(C: int, rank: int, world: int):
    """Contiguous [start, stop) of rank's columns; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    base, extra = divmod(C, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def local_alignment(alignment, rank: int, world: int):
    start, stop = column_range(alignment.shape[1], rank, world)
    return alignment[:, start:stop]


def gather_columns(local, C: int, group=None):
    """Concatenate every rank's (..., C_local) array along the last axis.

    Uses torch.distributed.all_gather_object on the host arrays (gloo or
    NCCL process groups both work); this is the only collective and it sits
    outside the compute path.
    """
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, np.asarray(local), group=group)
    out = np.concatenate(parts, axis=-1)
    assert out.shape[-1] == C
    return out


def max_over_ranks(value: float, group=None, device=None) -> float:
    """Max of a scalar (e.g. a step time) over ranks."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
