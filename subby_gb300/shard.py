"""Column sharding across ranks (one process per GPU).

Columns are independent, so a multi-GPU run gives each rank a contiguous
column range, replicates the tree and model, and needs no data-path
collective; results are concatenated along the column axis (the last axis of
every output).  ``gather_columns`` does that concatenation with one
all_gather when the caller wants the full result on every rank.

The gradient of sum_c g_c logL_c is the one exception: it is a sum over
columns (subby/jax/vjp.py:116-117 contracts the per-column terms), so each
rank computes its shard's gradient vector and one all-reduce-sum of the
packed (R + A(A-1)/2) vector (``allreduce_sum``, ``sharded_loglike_grad``)
gives every rank the whole-alignment gradient.
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


def allreduce_sum(*arrays, group=None, device=None):
    """Sum each array over ranks with ONE all-reduce of their packed FP64
    concatenation; returns the summed arrays in the input shapes.

    ``device`` is where the packed buffer lives for the collective (a CUDA
    device for NCCL process groups, None = CPU for gloo).
    """
    import torch
    import torch.distributed as dist
    flat = [np.asarray(a, dtype=np.float64).ravel() for a in arrays]
    sizes = [f.size for f in flat]
    buf = torch.from_numpy(np.concatenate(flat) if flat else np.zeros(0))
    if device is not None:
        buf = buf.to(device)
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    out = buf.cpu().numpy()
    res, at = [], 0
    for a, n in zip(arrays, sizes):
        res.append(out[at:at + n].reshape(np.shape(a)))
        at += n
    return res


def sharded_loglike_grad(plan, alignment, rank: int, world: int, g=None, log_exch=None, pi=None,
                         group=None, device=None):
    """Whole-alignment gradient of sum_c g_c logL_c from column shards.

    Rank ``rank`` runs the adjoint on its column range of ``alignment``
    (``Plan.grad``; ``g`` is the full (C,) cotangent or None for ones) and
    the ranks sum their gradient vectors with one all-reduce: the branch-
    length gradient (R,) and either the log-exchangeability gradient
    (A(A-1)/2,) when ``log_exch`` and ``pi`` are given, or d/dS~ (A, A).
    Returns (local logLike, dldt, dle_or_dS).
    """
    start, stop = column_range(alignment.shape[1], rank, world)
    loc = alignment[:, start:stop]
    gl = None if g is None else np.asarray(g, dtype=np.float32)[start:stop]
    ll, dldt, G = plan.grad(loc, g=gl)
    if log_exch is not None:
        from .autograd import exchangeability_grad
        second = exchangeability_grad(G, log_exch, pi)
    else:
        second = G
    dldt, second = allreduce_sum(dldt, second, group=group, device=device)
    return ll, dldt, second
