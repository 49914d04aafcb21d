"""Host-side pieces of the serving loop (subby_gb300/serve.py) that need no
GPU: plan keys, the device-time and footprint estimates that order and
admit jobs, job bookkeeping and the latency summary."""
import numpy as np

from subby_gb300 import models, serve, synth
from subby_gb300.types import Tree


def test_plan_key_separates_trees_and_models():
    rng = np.random.default_rng(0)
    t = synth.random_tree(8, 0.1, rng)
    m = models.hky85_diag(2.0, [0.3, 0.2, 0.25, 0.25])
    k = serve._plan_key(t, m)
    assert k == serve._plan_key(Tree(t.parentIndex.copy(), t.distanceToParent.copy()), m)
    assert k != serve._plan_key(Tree(t.parentIndex, t.distanceToParent * 1.5), m)
    assert k != serve._plan_key(t, models.hky85_diag(2.5, [0.3, 0.2, 0.25, 0.25]))
    ir = models.random_irreversible(4, rng)
    ir2 = ir._replace(eigenvectors_inv=ir.eigenvectors_inv * (1 + 1e-9))
    assert serve._plan_key(t, ir) != serve._plan_key(t, ir2)      # complex fields are part of the key


def test_cost_and_footprint_estimates():
    for A in (4, 16, 64):
        for f81 in (False, True):
            a = serve.job_cost_ms(255, 1000, A, f81)
            assert a > 0 and serve.job_cost_ms(255, 2000, A, f81) == 2 * a
            assert serve.job_cost_ms(511, 1000, A, f81) > a
    assert serve.job_cost_ms(127, 65536, 64) > serve.job_cost_ms(127, 65536, 64, f81=True)
    small = serve.job_device_bytes(15, 100, 4)
    assert 0 < small < serve.job_device_bytes(255, 1 << 20, 4)
    # tokens and outputs alone are a floor; the large-A staging is capped per plan
    R, C, A = 127, 1 << 22, 64
    b = serve.job_device_bytes(R, C, A)
    assert b >= 4 * R * C + 4 * C * (A * A + A + 1)
    assert b - serve.job_device_bytes(R, C // 2, A) <= 4 * R * C + 4 * C * (A * A + A + 1)


def test_job_bookkeeping_and_latency_stats():
    jobs = []
    for i in range(100):
        j = serve.Job(id=i, alignment=np.zeros((5, 10 + i), np.int32), tree=None, model=None, arrival=0.01 * i)
        j.start, j.finish = j.arrival + 0.002, j.arrival + 0.002 + 0.001 * (1 + i % 10)
        jobs.append(j)
    assert jobs[3].RC == (5, 13)
    assert serve.Job(id=0, alignment=None, tree=None, model=None, shape=(7, 9)).RC == (7, 9)
    given = []
    jobs[0].result = {"counts": 1}
    jobs[0]._pinned, jobs[0]._give_back = ["block"], given.append
    jobs[0].release()
    assert jobs[0].result == {} and given == [["block"]]
    s = serve.latency_stats(jobs)
    lat = np.array([j.latency for j in jobs]) * 1e3
    assert s["jobs"] == 100 and s["columns"] == sum(10 + i for i in range(100))
    assert abs(s["p50_ms"] - np.percentile(lat, 50)) < 1e-9 and abs(s["p99_ms"] - np.percentile(lat, 99)) < 1e-9
    assert abs(s["queue_p50_ms"] - 2.0) < 1e-9 and s["max_ms"] == lat.max()
    assert abs(s["span_s"] - (jobs[-1].finish - 0.0)) < 1e-12
