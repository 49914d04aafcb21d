"""World-size-2 gloo run of the column-sharding host logic on CPU.

Each rank takes its column range, computes LogLike / Counts / RootProb for it
(with the FP64 oracle standing in for the GPU, which this CPU test cannot
use), the ranks gather along the column axis, and rank 0 checks the result
equals the unsharded computation; the MAX reduction used for step timing is
checked too.  The gradient test sums two column shards' gradient vectors
(branch lengths and log-exchangeabilities, FP64 oracle standing in for the
adjoint kernel) with the single all-reduce of ``shard.allreduce_sum`` and
compares them with the unsharded gradient.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        from subby_gb300 import synth, shard
        w = synth.plain_small(seed=1, C=203)
        aln, tree, m = w['alignment'], w['tree'], w['model']
        t = oracle.Tree(tree.parentIndex, tree.distanceToParent)
        md = m._asdict()
        loc = shard.local_alignment(aln, rank, world)
        ll = shard.gather_columns(oracle.LogLike(loc, t, md), aln.shape[1])
        ct = shard.gather_columns(oracle.Counts(loc, t, md), aln.shape[1])
        rp = shard.gather_columns(oracle.RootProb(loc, t, md), aln.shape[1])
        mx = shard.max_over_ranks(1.0 + rank)
        if rank == 0:
            ok = (np.allclose(ll, oracle.LogLike(aln, t, md), rtol=0, atol=1e-12)
                  and np.allclose(ct, oracle.Counts(aln, t, md), rtol=0, atol=1e-12)
                  and np.allclose(rp, oracle.RootProb(aln, t, md), rtol=0, atol=1e-12)
                  and mx == float(world))
            q.put(ok)
    finally:
        dist.destroy_process_group()


def _grad_worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        from subby_gb300 import synth, shard, models
        rng = np.random.default_rng(12)
        model, log_exch, pi = models.random_reversible(4, rng, 0.5, 2.0)
        tree = synth.random_tree(6, 0.1, rng)
        aln = synth.simulated_alignment(tree, model, 61, 0.1, rng)
        t = oracle.Tree(tree.parentIndex, tree.distanceToParent)
        g = rng.uniform(0.5, 1.5, aln.shape[1])
        a, b = shard.column_range(aln.shape[1], rank, world)
        loc = aln[:, a:b]
        dt_loc = oracle.loglike_distance_grad(loc, t, model._asdict(), g=g[a:b])
        # FD of sum over the local columns only (unit cotangent)
        ds_loc = oracle.loglike_fd_grad(loc, t, log_exch, pi, h=1e-5, wrt="exchangeabilities")
        dt, ds = shard.allreduce_sum(dt_loc, ds_loc)
        if rank == 0:
            dt_ref = oracle.loglike_distance_grad(aln, t, model._asdict(), g=g)
            ds_ref = oracle.loglike_fd_grad(aln, t, log_exch, pi, h=1e-5, wrt="exchangeabilities")
            ok = (dt.shape == dt_ref.shape and ds.shape == ds_ref.shape
                  and np.allclose(dt, dt_ref, rtol=1e-10, atol=1e-10)
                  and np.allclose(ds, ds_ref, rtol=1e-6, atol=1e-7))
            q.put(bool(ok))
    finally:
        dist.destroy_process_group()


def test_column_ranges_partition():
    from subby_gb300 import shard
    for C in (0, 1, 7, 1024, 1025):
        for world in (1, 2, 3, 8):
            spans = [shard.column_range(C, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == C
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(b - a for a, b in spans) - min(b - a for a, b in spans) <= 1


def test_sharded_results_equal_unsharded_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, q), nprocs=2, join=True, start_method="spawn")
    assert q.get(timeout=60) is True


def test_sharded_gradient_allreduce_equals_unsharded_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    mp.start_processes(_grad_worker, args=(2, port, q), nprocs=2, join=True, start_method="spawn")
    assert q.get(timeout=60) is True
