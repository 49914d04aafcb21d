"""Continuous-batching loop: jobs of uneven R, C and A run concurrently on
several streams; each job's result equals the same job run alone (and the
oracle on a column subsample), within the parity tolerances."""
import numpy as np
import pytest

import oracle
from tests._tol import assert_cols, assert_loglike, COUNTS_RTOL

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import synth, serve  # noqa: E402


def _jobs(n=24, seed=8):
    desc = synth.serving_jobs(n_jobs=n, rate=1000.0, seed=seed, max_columns=3000, min_columns=40,
                              min_leaves=4, max_leaves=48)
    jobs = []
    for d in desc:
        aln, tree, model = synth.materialize_job(d)
        jobs.append(serve.Job(id=d['id'], alignment=aln, tree=tree, model=model, f81=(d['kind'] == 'f81'),
                              want=("logLike", "counts"), arrival=d['arrival']))
    return jobs


def test_results_identical_alone_and_in_the_mix():
    jobs = _jobs()
    srv = serve.Server(max_inflight=6, device_budget=1 << 30)
    done = srv.run(jobs, realtime=False)
    assert len(done) == len(jobs)
    assert len({j.id for j in done}) == len(jobs)
    for j in done:
        assert not j.error, f"job {j.id}: {j.error}"
        plan = sg.Plan(j.tree, j.model)
        alone = plan.run(j.alignment, loglike=True, counts=True, f81=j.f81)
        plan.close()
        assert_cols(j.result['counts'], alone['counts'], COUNTS_RTOL, f"job {j.id} counts")
        assert_loglike(j.result['logLike'], alone['logLike'])
    # oracle spot check on the first columns of three jobs
    for j in done[:3]:
        sub = j.alignment[:, :16]
        t = oracle.Tree(j.tree.parentIndex, j.tree.distanceToParent)
        md = sg.models.ensure_diag(j.model)._asdict()
        assert_cols(j.result['counts'][:, :, :16], oracle.Counts(sub, t, md, f81_fast=j.f81),
                    COUNTS_RTOL, "oracle")
    stats = serve.latency_stats(done)
    assert stats['p99_ms'] >= stats['p50_ms'] > 0
    srv.close()


def test_admission_respects_budget_and_slots():
    jobs = _jobs(n=10, seed=9)
    srv = serve.Server(max_inflight=3, device_budget=1)   # budget below any job: one at a time
    peak = []
    srv.run(jobs, realtime=False, on_admit=lambda j: peak.append(len(srv.inflight)))
    assert max(peak) == 1
    srv.close()


def test_sliced_long_jobs_and_priority_streams_give_identical_results():
    """With a tiny slice budget and 128-column slice granularity every job is
    cut into 128-column slices (and
    short-job threshold 0 sends all to normal-priority streams, a large one
    to high-priority streams); the results equal the unsliced run bit for
    bit, because every column is computed independently."""
    jobs = _jobs(n=8, seed=10)
    ref = {}
    for j in jobs:
        plan = sg.Plan(j.tree, j.model)
        ref[j.id] = plan.run(j.alignment, loglike=True, counts=True, f81=j.f81)
        plan.close()
    for short_ms, slice_ms in ((0.0, 1e-6), (1e9, 1e-6)):
        srv = serve.Server(max_inflight=4, device_budget=1 << 30, short_ms=short_ms, slice_ms=slice_ms,
                           wave_cols=128)
        done = srv.run(_jobs(n=8, seed=10), realtime=False)
        assert len(done) == len(jobs)
        for j in done:
            np.testing.assert_array_equal(j.result['counts'], ref[j.id]['counts'])
            np.testing.assert_array_equal(j.result['logLike'], ref[j.id]['logLike'])
        srv.close()


def test_plan_trim_releases_workspace_and_keeps_results():
    rng = np.random.default_rng(3)
    m = sg.models.random_reversible(20, rng, 0.5, 2.0)[0]
    tree = synth.random_tree(12, 0.1, rng)
    aln = synth.simulated_alignment(tree, m, 300, 0.1, rng)
    plan = sg.Plan(tree, m)
    a = plan.run(aln, loglike=True, counts=True)
    held = plan.device_bytes()
    plan.trim()
    assert plan.device_bytes() < held
    b = plan.run(aln, loglike=True, counts=True)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    plan.close()


def test_irreversible_jobs_in_the_mix():
    """Irreversible-model jobs share the loop with reversible ones; each result
    equals its job run alone."""
    rng = np.random.default_rng(21)
    jobs = []
    for i in range(6):
        A = 4 if i % 2 else 20
        m = sg.models.random_irreversible(A, rng) if i < 4 else sg.models.random_reversible(A, rng)[0]
        tree = synth.random_tree(int(rng.integers(4, 20)), 0.1, rng)
        aln = rng.integers(0, A + 2, size=(len(tree.parentIndex), int(rng.integers(50, 900)))).astype(np.int32)
        jobs.append(serve.Job(id=i, alignment=aln, tree=tree, model=m, f81=False, want=("logLike", "counts"),
                              arrival=0.0))
    srv = serve.Server(max_inflight=3, device_budget=1 << 30)
    done = srv.run(jobs, realtime=False)
    assert len(done) == 6
    for j in done:
        assert not j.error, j.error
        plan = sg.Plan(j.tree, j.model)
        alone = plan.run(j.alignment, loglike=True, counts=True)
        plan.close()
        np.testing.assert_array_equal(j.result['counts'], alone['counts'])
        np.testing.assert_array_equal(j.result['logLike'], alone['logLike'])
    srv.close()
