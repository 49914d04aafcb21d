"""Adjoint kernel (subby_plan_grad) and the torch.autograd wrappers vs FP64
finite differences of the oracle and the oracle's own Fisher-identity
distance gradient (subby/jax/vjp.py:92-124 restated in oracle/)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import synth, models, autograd  # noqa: E402

GRAD_RTOL = 2e-4   # relative to the largest gradient component


def _close(got, ref, what, rtol=GRAD_RTOL):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    scale = max(np.max(np.abs(ref)), 1e-12)
    err = np.max(np.abs(got - ref)) / scale
    assert err <= rtol, f"{what}: max |d| / max |ref| = {err:.2e} > {rtol:.0e}"


def _case(A, leaves, C, seed, gap=0.15):
    rng = np.random.default_rng(seed)
    model, log_exch, pi = models.random_reversible(A, rng, 0.5, 2.0)
    tree = synth.random_tree(leaves, 0.08, rng)
    aln = synth.simulated_alignment(tree, model, C, gap, rng)
    return aln, tree, model, log_exch, pi


@pytest.mark.parametrize("A,leaves,C", [(4, 12, 300), (20, 10, 128)])
def test_distance_gradient_matches_oracle(A, leaves, C):
    aln, tree, model, _, _ = _case(A, leaves, C, 40 + A)
    md = model._asdict()
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    g = np.random.default_rng(1).uniform(0.5, 1.5, C)
    plan = sg.Plan(tree, model)
    ll, dldt, _ = plan.grad(aln, g=g.astype(np.float32))
    ref = oracle.loglike_distance_grad(aln, ot, md, g=g.astype(np.float32).astype(np.float64))
    _close(dldt, ref, "d(sum g logL)/dt")
    assert dldt[0] == 0.0
    np.testing.assert_allclose(ll, oracle.LogLike(aln, ot, md), rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("A,leaves,C", [(4, 8, 200), (20, 7, 64)])
def test_autograd_vs_central_differences(A, leaves, C):
    """c4-style check: d(sum logL)/d(branch lengths, log-exchangeabilities)
    from the adjoint kernel vs central differences with h = 1e-4 in FP64."""
    aln, tree, model, log_exch, pi = _case(A, leaves, C, 60 + A)
    d = torch.tensor(np.asarray(tree.distanceToParent), dtype=torch.float64, requires_grad=True)
    le = torch.tensor(log_exch, dtype=torch.float64, requires_grad=True)
    ll = autograd.loglike_reversible(aln, tree.parentIndex, d, le, pi)
    ll.sum().backward()
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    fd_t = oracle.loglike_fd_grad(aln, ot, log_exch, pi, h=1e-4, wrt="distances")
    fd_s = oracle.loglike_fd_grad(aln, ot, log_exch, pi, h=1e-4, wrt="exchangeabilities")
    _close(d.grad.numpy(), fd_t, "d/dt vs FD", rtol=1e-3)
    _close(le.grad.numpy(), fd_s, "d/dlog s vs FD", rtol=1e-3)


def test_loglike_custom_grad_api():
    aln, tree, model, _, _ = _case(4, 10, 128, 77)
    d = torch.tensor(np.asarray(tree.distanceToParent), dtype=torch.float64, requires_grad=True)
    ll = sg.LogLikeCustomGrad(aln, sg.Tree(tree.parentIndex, d), model)
    ll.sum().backward()
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    ref = oracle.loglike_distance_grad(aln, ot, model._asdict())
    _close(d.grad.numpy(), ref, "LogLikeCustomGrad d/dt")


@pytest.mark.parametrize("A,leaves,C", [(16, 9, 300), (20, 12, 500), (64, 6, 200)])
def test_walk_gradient_matches_warp_adjoint(A, leaves, C):
    """Large alphabets: the walk + per-branch X_n path (default) and the
    warp-per-column adjoint (kernel selector 1) give the same logL, distance
    gradient and exchangeability gradient; the distance gradient also
    matches the oracle."""
    from subby_gb300 import _lib
    aln, tree, model, _, _ = _case(A, leaves, C, 50 + A)
    g = np.random.default_rng(A).uniform(0.5, 1.5, C).astype(np.float32)
    plan = sg.Plan(tree, model)
    ll0, dt0, dS0 = plan.grad(aln, g=g)
    try:
        _lib.load().subby_debug_set_kernel(1)
        ll1, dt1, dS1 = plan.grad(aln, g=g)
    finally:
        _lib.load().subby_debug_set_kernel(0)
    plan.close()
    np.testing.assert_allclose(ll0, ll1, rtol=1e-5, atol=1e-4)
    _close(dt0, dt1, "distance gradient, walk vs warp")
    _close(dS0, dS1, "exchangeability gradient, walk vs warp")
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    _close(dt0, oracle.loglike_distance_grad(aln, ot, model._asdict(), g=g.astype(np.float64)), "vs oracle")
