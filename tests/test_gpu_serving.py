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


# ---------------------------------------------------------------------------
# the library's serving engine (subby_server_*, serve.NativeServer)
# ---------------------------------------------------------------------------

def _pinned(aln):
    t = torch.empty(aln.shape, dtype=torch.int32, pin_memory=True)
    t.numpy()[:] = aln
    return t


def _native_jobs(n=24, seed=8, want=("logLike", "counts", "rootProb")):
    out = []
    for j in _jobs(n=n, seed=seed):
        j.want = want
        j.host = j.alignment
        j.alignment = _pinned(j.host)
        out.append(j)
    return out


def _alone(j, bm="auto"):
    plan = sg.Plan(j.tree, j.model)
    r = plan.run(j.host, loglike=True, counts=True, rootprob=True, f81=j.f81, branch_mask=bm)
    plan.close()
    return r


@pytest.mark.parametrize("pack", [1, 0], ids=["packed", "one_launch_per_job"])
def test_native_engine_results_identical_alone_and_in_the_mix(pack):
    jobs = _native_jobs()
    srv = serve.NativeServer(max_inflight=6, device_budget=1 << 30, pack=pack)
    done = srv.run(jobs, realtime=False)
    assert len(done) == len(jobs) and len({j.id for j in done}) == len(jobs)
    for j in done:
        assert not j.error, f"job {j.id}: {j.error}"
        ref = _alone(j)
        for k in ("logLike", "counts", "rootProb"):
            np.testing.assert_array_equal(j.result[k], ref[k])
        assert j.finish >= j.start >= j.arrival - 1e-6
        j.release()
    assert (srv.stats()["packed_jobs"] > 0) == bool(pack)
    # oracle on the first columns of three jobs
    for j in jobs[:3]:
        sub = j.host[:, :16]
        t = oracle.Tree(j.tree.parentIndex, j.tree.distanceToParent)
        md = sg.models.ensure_diag(j.model)._asdict()
        assert_cols(_alone(j)['counts'][:, :, :16], oracle.Counts(sub, t, md, f81_fast=j.f81), COUNTS_RTOL, "oracle")
    srv.close()


def test_native_engine_slices_and_priorities_give_identical_results():
    """Every job cut into 128-column slices, on low- and on high-priority
    streams: bit-identical to the single call, because every column is
    computed independently."""
    jobs = _native_jobs(n=8, seed=10)
    ref = {j.id: _alone(j) for j in jobs}
    for short_ms in (0.0, 1e9):
        srv = serve.NativeServer(max_inflight=4, device_budget=1 << 30, short_ms=short_ms, slice_ms=1e-6,
                                 wave_cols=128, pack=0)
        done = srv.run(_native_jobs(n=8, seed=10), realtime=False)
        assert len(done) == len(jobs)
        for j in done:
            assert not j.error
            for k in ("logLike", "counts", "rootProb"):
                np.testing.assert_array_equal(j.result[k], ref[j.id][k])
            j.release()
        srv.close()


def test_native_engine_host_row_windows_and_unmasked_counts():
    """Alignments given as row-mapped windows of a pinned host buffer (how
    the serving benchmark feeds jobs), counts unmasked, A = 4 and 16."""
    rng = np.random.default_rng(4)
    pool = _pinned(rng.integers(0, 6, size=(40, 5000)).astype(np.int32))
    pool.numpy()[39] = 4
    srv = serve.NativeServer(max_inflight=3, device_budget=1 << 30)
    jobs = []
    for i in range(6):
        tree = synth.random_tree(int(rng.integers(3, 15)), 0.1, rng)
        model = sg.models.hky85_diag(2.0, rng.dirichlet(np.ones(4)))
        R = len(tree.parentIndex)
        C = int(rng.integers(10, 3000))
        off = int(rng.integers(0, 5000 - C + 1))
        rowmap = rng.choice(39, size=R, replace=False).astype(np.int32)
        rowmap[~synth.leaf_mask(tree)] = 39
        j = serve.Job(id=i, alignment=serve.HostRows(base=pool, col0=off, rowmap=rowmap, R=R, C=C), tree=tree,
                      model=model, want=("counts", "logLike", "rootProb"), branch_mask=None)
        j.host = np.ascontiguousarray(pool.numpy()[rowmap, off:off + C])
        jobs.append(j)
    done = srv.run(jobs, realtime=False)
    assert len(done) == len(jobs)
    for j in done:
        assert not j.error
        ref = _alone(j, bm=None)
        for k in ("logLike", "counts", "rootProb"):
            np.testing.assert_array_equal(j.result[k], ref[k])
        j.release()
    srv.close()


def test_native_engine_packs_short_a4_jobs_into_few_launches():
    """Short A = 4 jobs submitted together run as batches of the persistent
    packed kernel over their (job, column-tile) queue; each job's results
    equal its single call bit for bit, F81 and eigen jobs in their own
    batches."""
    rng = np.random.default_rng(12)
    jobs = []
    for i in range(20):
        tree = synth.random_tree(int(rng.integers(3, 60)), 0.1, rng)
        model = sg.models.hky85_diag(2.0, rng.dirichlet(np.ones(4)))
        aln = synth.simulated_alignment(tree, model, int(rng.integers(1, 3000)), 0.1, rng)
        j = serve.Job(id=i, alignment=_pinned(aln), tree=tree, model=model, f81=(i % 3 == 0),
                      want=("logLike", "counts", "rootProb"))
        j.host = aln
        jobs.append(j)
    srv = serve.NativeServer(max_inflight=2, device_budget=1 << 30)
    done = srv.run(jobs, realtime=False)
    st = srv.stats()
    assert st["packed_jobs"] == 20 and st["packed_launches"] < 20
    for j in done:
        assert not j.error
        ref = _alone(j)
        for k in ("logLike", "counts", "rootProb"):
            np.testing.assert_array_equal(j.result[k], ref[k])
        j.release()
    srv.close()


def test_native_engine_reports_a_wait_that_gave_up():
    """A=64 job run with the bounded-wait test hook: the job completes with
    SUBBY_ERR_TIMEOUT read from the plan's status word; the next job, with
    the hook off, is correct."""
    from subby_gb300 import _lib
    rng = np.random.default_rng(5)
    model = sg.models.random_reversible(64, rng, 0.5, 2.0)[0]
    tree = synth.random_tree(6, 0.1, rng)
    aln = synth.simulated_alignment(tree, model, 200, 0.1, rng)
    lib = _lib.load()
    srv = serve.NativeServer(max_inflight=2, device_budget=1 << 30)
    j1 = serve.Job(id=1, alignment=_pinned(aln), tree=tree, model=model, want=("counts",))
    try:
        lib.subby_debug_fail_waits(8)
        d1 = srv.run([j1], realtime=False)
    finally:
        lib.subby_debug_fail_waits(0)
    assert d1[0].error and "timed out" in d1[0].error
    d1[0].release()
    j2 = serve.Job(id=2, alignment=_pinned(aln), tree=tree, model=model, want=("counts",))
    j2.host = aln
    d2 = srv.run([j2], realtime=False)
    assert not d2[0].error
    np.testing.assert_array_equal(d2[0].result['counts'], _alone(j2)['counts'])
    srv.close()


def test_native_engine_rejects_what_it_does_not_serve():
    rng = np.random.default_rng(6)
    srv = serve.NativeServer(max_inflight=2, device_budget=1 << 30)
    tree = synth.random_tree(5, 0.1, rng)
    aln = _pinned(rng.integers(0, 4, size=(len(tree.parentIndex), 10)).astype(np.int32))
    irr = sg.models.random_irreversible(4, rng)
    with pytest.raises(ValueError):
        srv.submit(serve.Job(id=0, alignment=aln, tree=tree, model=irr))
    rev = sg.models.hky85_diag(2.0, [0.25] * 4)
    with pytest.raises(ValueError):
        srv.submit(serve.Job(id=1, alignment=aln, tree=tree, model=rev, branch_mask=np.ones((5, 10), bool)))
    with pytest.raises(ValueError):
        srv.submit(serve.Job(id=2, alignment=aln.numpy(), tree=tree, model=rev))
    srv.close()


def test_packed_kernel_queue_wait_gives_up_and_reports_timeout():
    """An open queue with nothing published: each CTA's claim waits a bounded
    number of polls, gives up and records it; the host reads TIMEOUT and the
    device stays usable."""
    import ctypes
    from subby_gb300 import _lib
    lib = _lib.load()
    n = ctypes.c_int(0)
    rc = lib.subby_debug_packed_queue_wait(64, 4, ctypes.byref(n))
    assert rc == _lib.ERR_TIMEOUT and n.value == 4
    j = _native_jobs(n=1, seed=3)[0]
    srv = serve.NativeServer(max_inflight=2, device_budget=1 << 30)
    d = srv.run([j], realtime=False)
    assert not d[0].error
    np.testing.assert_array_equal(d[0].result['counts'], _alone(j)['counts'])
    srv.close()


def test_packed_work_item_shapes_give_identical_results():
    """Items spanning 1 or 3 tiles of 256 columns (the autotuned shape): each
    job's results equal its single call bit for bit."""
    rng = np.random.default_rng(13)
    jobs = []
    for i in range(12):
        # trees whose tables fit the A = 4 kernel's shared memory (larger
        # ones take the one-job path)
        tree = synth.random_tree(int(rng.integers(3, 70)), 0.1, rng)
        model = sg.models.hky85_diag(2.0, rng.dirichlet(np.ones(4)))
        aln = synth.simulated_alignment(tree, model, int(rng.integers(1, 5000)), 0.1, rng)
        jobs.append((tree, model, aln))
    for tiles in (1, 3):
        srv = serve.NativeServer(max_inflight=2, device_budget=1 << 30, pack_tiles_r64=tiles,
                                 pack_tiles_r256=tiles, pack_tiles_big=tiles)
        batch = []
        for i, (tree, model, aln) in enumerate(jobs):
            j = serve.Job(id=i, alignment=_pinned(aln), tree=tree, model=model, want=("logLike", "counts"))
            j.host = aln
            batch.append(j)
        done = srv.run(batch, realtime=False)
        assert srv.stats()["packed_jobs"] == len(jobs)
        for j in done:
            assert not j.error
            ref = _alone(j)
            for k in ("logLike", "counts"):
                np.testing.assert_array_equal(j.result[k], ref[k])
            j.release()
        srv.close()


def test_autotune_packed_writes_and_applies_its_choice(tmp_path):
    cache = str(tmp_path / "autotune.json")
    got = serve.autotune_packed(cache=cache, candidates=(1, 4), n_jobs=6, trials=1)
    assert set(got) == {k for k, _ in serve.PACK_TILE_KEYS} and set(got.values()) <= {1, 4}
    assert serve.load_autotune(cache) == got
    j = _native_jobs(n=1, seed=3)[0]
    srv = serve.NativeServer(max_inflight=2, device_budget=1 << 30, autotune_cache=cache)
    d = srv.run([j], realtime=False)
    assert not d[0].error
    np.testing.assert_array_equal(d[0].result['counts'], _alone(j)['counts'])
    srv.close()
