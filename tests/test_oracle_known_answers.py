"""Known answers of the FP64 oracle, from mathematics rather than from the
reference's fixtures — the facts the reference's own tests check
(tests/test_eigensub.py:51-119, tests/test_outside.py:39-72,
tests/test_f81_fast.py:24-81, tests/test_oracle.py:503-582), here with
tighter tolerances where the fact is exact:

* J(t) closed forms, its symmetry and the 1e-8 degeneracy switch;
* expected counts on a small tree by brute force: the states of every node
  without an observed token enumerated, each branch's endpoint-conditioned
  integrals I[a, b, i, j] = int_0^t M(s)_ai M(t - s)_jb ds by Gauss-Legendre
  quadrature over scipy's expm;
* sum_a D_n,a (M_n U_n)_a = P(x) for every branch (outside-pass consistency);
* F81 / JC closed form = the general eigenbasis path; total dwell time =
  total branch length when every branch is in the Steiner tree;
* branch mask semantics (no gaps: masked = unmasked; one ungapped leaf: no
  counts; gaps: they differ); root posteriors sum to 1; counts >= 0.
CPU only."""
import itertools

import numpy as np
import pytest
from scipy.linalg import expm

import oracle

TREE7 = oracle.Tree(np.array([-1, 0, 0, 1, 1, 2, 2], np.int32), np.array([0.0, 0.1, 0.2, 0.15, 0.25, 0.12, 0.18]))


def _rate_matrix(md):
    """Q = diag(pi)^-1/2 V diag(mu) V^T diag(pi)^1/2 of a reversible model."""
    V, mu, pi = (np.asarray(md[k], np.float64) for k in ("eigenvectors", "eigenvalues", "pi"))
    sp = np.sqrt(pi)
    return (V * mu) @ V.T / sp[:, None] * sp[None, :]


def _endpoint_integrals(Q, t, n=40):
    x, w = np.polynomial.legendre.leggauss(n)
    s, w = 0.5 * t * (x + 1.0), 0.5 * t * w
    return sum(wk * np.einsum("ai,jb->abij", expm(Q * sk), expm(Q * (t - sk))) for sk, wk in zip(s, w))


def _brute_force_counts(aln, tree, md):
    """(A, A, C) expected dwell times / substitution counts by enumeration."""
    Q = _rate_matrix(md)
    pi = np.asarray(md["pi"], np.float64)
    A = len(pi)
    R, C = aln.shape
    par, dist = tree.parentIndex, tree.distanceToParent
    M = [None] + [expm(Q * dist[n]) for n in range(1, R)]
    E = [None]
    for n in range(1, R):                       # E_n[a, b] (A, A) per endpoint pair
        I = _endpoint_integrals(Q, dist[n])
        w = np.where(np.eye(A, dtype=bool), 1.0, Q)
        E.append(I * w[None, None] / M[n][:, :, None, None])
    out = np.zeros((A, A, C))
    for c in range(C):
        free = [n for n in range(R) if not 0 <= aln[n, c] < A]
        px = 0.0
        acc = np.zeros((A, A))
        for states in itertools.product(range(A), repeat=len(free)):
            x = aln[:, c].copy()
            x[free] = states
            p = pi[x[0]] * np.prod([M[n][x[par[n]], x[n]] for n in range(1, R)])
            px += p
            acc += p * sum(E[n][x[par[n]], x[n]] for n in range(1, R))
        out[:, :, c] = acc / px
    return out


def test_J_closed_forms_and_threshold():
    t = 0.5
    mu = np.array([0.0, -1.0, -1.0, -2.0])
    J = oracle.compute_J(mu, np.array([t]))[0]
    np.testing.assert_allclose(np.diag(J), t * np.exp(mu * t), rtol=1e-15)
    assert J[1, 2] == pytest.approx(t * np.exp(-t), rel=1e-15)
    J = oracle.compute_J(np.array([0.0, -1.0, -2.0, -3.0]), np.array([t]))[0]
    assert J[0, 1] == pytest.approx(1.0 - np.exp(-t), rel=1e-14)
    assert J[1, 3] == pytest.approx((np.exp(-t) - np.exp(-3 * t)) / 2.0, rel=1e-14)
    np.testing.assert_allclose(J, J.T, rtol=1e-15)
    for gap in (5e-9, 2e-8):                    # either side of the 1e-8 switch
        J = oracle.compute_J(np.array([-1.0, -1.0 - gap]), np.array([t]))[0]
        exact = np.exp(-t) * -np.expm1(-gap * t) / gap
        assert J[0, 1] == pytest.approx(exact, rel=1e-6)
        if gap < 1e-8:
            assert J[0, 1] == t * np.exp(-t)


@pytest.mark.parametrize("kind", ["hky", "random"])
def test_counts_match_brute_force_enumeration(kind):
    rng = np.random.default_rng(3)
    if kind == "hky":
        md = oracle.hky85_diag(2.5, np.array([0.3, 0.2, 0.15, 0.35]))
    else:
        pi = rng.dirichlet(np.ones(4))
        md = oracle.diagonalize_rate_matrix(oracle.reversible_rate_matrix(rng.normal(size=6), pi), pi)
    aln = rng.integers(0, 4, size=(7, 9)).astype(np.int32)
    aln[:3] = 4                                  # internal nodes unobserved
    aln[3, 2] = 5                                # a gapped leaf
    aln[5, 4] = -1                               # a legacy gap
    aln[1, 6] = 2                                # an observed internal node
    got = oracle.Counts(aln, TREE7, md, branch_mask=None)
    np.testing.assert_allclose(got, _brute_force_counts(aln, TREE7, md), rtol=1e-9, atol=1e-12)


def test_outside_pass_consistency():
    rng = np.random.default_rng(123)
    md = oracle.hky85_diag(2.0, np.array([0.1, 0.4, 0.3, 0.2]))
    aln = rng.integers(-1, 6, size=(7, 12)).astype(np.int32)
    M = oracle.compute_sub_matrices(md, TREE7.distanceToParent)
    U, lnU, lnL = oracle.upward_pass(aln, TREE7, M, md["pi"])
    D, lnD = oracle.downward_pass(U, lnU, TREE7, M, md["pi"], aln)
    for n in range(1, 7):
        joint = np.einsum("ca,ab,cb->c", D[n], M[n], U[n])
        np.testing.assert_allclose(np.log(joint) + lnD[n] + lnU[n], lnL, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("A", [4, 20])
def test_f81_closed_form_equals_general_path(A):
    rng = np.random.default_rng(A)
    aln = rng.integers(-1, A + 2, size=(7, 10)).astype(np.int32)
    for md in (oracle.jukes_cantor_model(A), oracle.f81_model(rng.dirichlet(np.ones(A)))):
        for mask in ("auto", None):
            np.testing.assert_allclose(oracle.Counts(aln, TREE7, md, f81_fast=True, branch_mask=mask),
                                       oracle.Counts(aln, TREE7, md, branch_mask=mask), rtol=1e-9, atol=1e-12)


def test_total_dwell_is_total_branch_length():
    rng = np.random.default_rng(5)
    aln = rng.integers(0, 4, size=(7, 6)).astype(np.int32)
    for md in (oracle.jukes_cantor_model(4), oracle.hky85_diag(3.0, np.array([0.4, 0.1, 0.2, 0.3]))):
        for f81 in (False, True) if md["pi"][0] == 0.25 else (False,):
            c = oracle.Counts(aln, TREE7, md, f81_fast=f81)
            np.testing.assert_allclose(np.einsum("iic->c", c), TREE7.distanceToParent.sum(), rtol=1e-12)


def test_branch_mask_semantics_and_posterior_normalisation():
    rng = np.random.default_rng(114)
    md = oracle.jukes_cantor_model(4)
    full = rng.integers(0, 4, size=(7, 6)).astype(np.int32)
    np.testing.assert_allclose(oracle.Counts(full, TREE7, md), oracle.Counts(full, TREE7, md, branch_mask=None),
                               rtol=1e-12, atol=1e-15)
    gappy = full.copy()
    gappy[3, :4] = 5
    gappy[4, 2:6] = 5
    assert not np.allclose(oracle.Counts(gappy, TREE7, md), oracle.Counts(gappy, TREE7, md, branch_mask=None))
    assert oracle.Counts(gappy, TREE7, md).min() >= -1e-12
    cherry = oracle.Tree(np.array([-1, 0, 0], np.int32), np.array([0.0, 0.1, 0.2]))
    one = np.array([[0, 0, 0], [1, 2, 3], [5, 5, 5]], np.int32)
    np.testing.assert_array_equal(oracle.Counts(one, cherry, md), 0.0)
    np.testing.assert_allclose(oracle.RootProb(gappy, TREE7, md).sum(axis=0), 1.0, rtol=1e-13)
