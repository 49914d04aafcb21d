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
