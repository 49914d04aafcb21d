"""CPU checks of the gradient algebra the adjoint kernel relies on (no GPU):

* the oracle's Fisher-identity distance gradient equals FP64 central
  differences, and
* G = sum_c V C_c V^T (unmasked eigenbasis counts) is d(sum logL)/dS~, so the
  host chain rule of subby_gb300.autograd.exchangeability_grad turns it into
  the log-exchangeability gradient that matches central differences.
"""
import numpy as np
import pytest

import oracle
from subby_gb300 import synth, models

torch = pytest.importorskip("torch")
from subby_gb300.autograd import exchangeability_grad  # noqa: E402


def _case(A, leaves, C, seed):
    rng = np.random.default_rng(seed)
    model, log_exch, pi = models.random_reversible(A, rng, 0.5, 2.0)
    tree = synth.random_tree(leaves, 0.08, rng)
    aln = synth.simulated_alignment(tree, model, C, 0.15, rng)
    return aln, oracle.Tree(tree.parentIndex, tree.distanceToParent), model, log_exch, pi


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-12)


@pytest.mark.parametrize("A", [4, 6])
def test_distance_gradient_identity(A):
    aln, t, model, le, pi = _case(A, 7, 40, 3 + A)
    g = oracle.loglike_distance_grad(aln, t, model._asdict())
    fd = oracle.loglike_fd_grad(aln, t, le, pi, h=1e-5, wrt="distances")
    assert _rel(g, fd) < 1e-6


@pytest.mark.parametrize("A", [4, 5])
def test_exchangeability_gradient_from_eigen_counts(A):
    aln, t, model, le, pi = _case(A, 6, 30, 11 + A)
    md = model._asdict()
    M = oracle.compute_sub_matrices(md, t.distanceToParent)
    U, lnU, lnL = oracle.upward_pass(aln, t, M, md['pi'])
    D, lnD = oracle.downward_pass(U, lnU, t, M, md['pi'], aln)
    J = oracle.compute_J(md['eigenvalues'], t.distanceToParent)
    Ut, Dt = oracle.eigenbasis_project(U, D, md)
    Ce = oracle.accumulate_C(Dt, Ut, J, lnU, lnD, lnL, t.parentIndex)
    V = md['eigenvectors']
    G = V @ Ce.sum(axis=-1) @ V.T
    dle = exchangeability_grad(G, le, pi)
    fd = oracle.loglike_fd_grad(aln, t, le, pi, h=1e-5, wrt="exchangeabilities")
    assert _rel(dle, fd) < 1e-5


@pytest.mark.parametrize("A", [4, 20])
def test_per_branch_gram_identities(A):
    """The large-alphabet gradient path (k_xgram + host FP64) in numpy: with
    X_n = sum_c g_c D~_nc (x) U~_nc (D~ carrying exp(lnD + lnU - lnL)),
    d/dt_n = sum_k mu_k e^{mu_k t_n} X_n[k][k] equals the oracle's distance
    gradient, and V (sum_n J_n o X_n) V^T equals sum_c g_c V C_c V^T."""
    aln, t, model, le, pi = _case(A, 6, 25, 40 + A)
    md = model._asdict()
    C = aln.shape[1]
    g = np.random.default_rng(A).uniform(0.5, 1.5, C)
    M = oracle.compute_sub_matrices(md, t.distanceToParent)
    U, lnU, lnL = oracle.upward_pass(aln, t, M, md['pi'])
    D, lnD = oracle.downward_pass(U, lnU, t, M, md['pi'], aln)
    J = oracle.compute_J(md['eigenvalues'], t.distanceToParent)
    Ut, Dt = oracle.eigenbasis_project(U, D, md)
    mu, tt = np.asarray(md['eigenvalues']), t.distanceToParent
    R = len(tt)
    grad = np.zeros(R)
    Cg = np.zeros((A, A))
    for n in range(1, R):
        s = np.exp(lnD[n] + lnU[n] - lnL)
        X = np.einsum('c,ck,cl->kl', g * s, Dt[n], Ut[n])
        grad[n] = np.sum(mu * np.exp(mu * tt[n]) * np.diag(X))
        Cg += J[n] * X
    assert _rel(grad, oracle.loglike_distance_grad(aln, t, md, g=g)) < 1e-12
    V = md['eigenvectors']
    Ce = oracle.accumulate_C(Dt, Ut, J, lnU, lnD, lnL, t.parentIndex)
    assert _rel(V @ Cg @ V.T, V @ np.einsum('klc,c->kl', Ce, g) @ V.T) < 1e-12


def test_irreversible_gradient_identity():
    """D^T (dM/dt) U with dM/dt = Re V diag(mu e^{mu t}) V^-1 (the tables of
    the complex-system gradient kernel) equals the reference's irreversible
    vjp projection (Re sum_k (D V)_k mu_k e^{mu_k t} (V^-1 U)_k), and the
    oracle's gradient matches central differences."""
    rng = np.random.default_rng(8)
    m = models.random_irreversible(4, rng)._asdict()
    tree = synth.random_tree(6, 0.2, rng)
    t = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    aln = synth.simulated_alignment(tree, models.random_irreversible(4, np.random.default_rng(9)), 30, 0.1, rng)
    M = oracle.compute_sub_matrices_irrev(m, t.distanceToParent)
    U, lnU, lnL = oracle.upward_pass(aln, t, M, m['pi'])
    D, lnD = oracle.downward_pass(U, lnU, t, M, m['pi'], aln)
    V, Vi, mu = m['eigenvectors'], m['eigenvectors_inv'], m['eigenvalues']
    grad = np.zeros(len(t.distanceToParent))
    for n in range(1, len(grad)):
        dM = (V * (mu * np.exp(mu * t.distanceToParent[n]))) @ Vi
        s = np.exp(lnD[n] + lnU[n] - lnL)
        grad[n] = np.sum(s * np.einsum('ca,ab,cb->c', D[n], dM.real, U[n]))
    ref = oracle.loglike_distance_grad(aln, t, m)
    assert _rel(grad, ref) < 1e-10
    h = 1e-6
    fd = np.zeros_like(ref)
    for n in range(1, len(ref)):
        dp, dm = t.distanceToParent.copy(), t.distanceToParent.copy()
        dp[n] += h
        dm[n] -= h
        fd[n] = (oracle.LogLike(aln, oracle.Tree(t.parentIndex, dp), m).sum()
                 - oracle.LogLike(aln, oracle.Tree(t.parentIndex, dm), m).sum()) / (2 * h)
    assert _rel(ref, fd) < 1e-5
