"""Irreversible counts against quadrature (CPU, no GPU).

E[N_ij] on a branch of length t = (1/P) sum_ab D_a U_b int_0^t [e^{Qs}]_ai
Q_ij [e^{Q(t-s)}]_jb ds (dwell time on the diagonal, without Q_ii).  The
midpoint rule with scipy's expm checks:

* the reversible eigen path of the oracle (pinned to the reference) —
  validates the quadrature;
* the oracle's ``irrev_exact`` variant (D~ = D V, U~ = Vinv U, back-transform
  Vinv^T C V^T) for a model with complex eigenvalues;
* that the reference's irreversible formula (subby/oracle/oracle.py:537-693,
  restated as the oracle's default) gives instead the counts of the
  transposed process, and disagrees with the reversible path on a reversible
  model written in irreversible form, while ``irrev_exact`` agrees with it.
"""
import numpy as np
import pytest

import oracle

scipy_linalg = pytest.importorskip("scipy.linalg")


def _quadrature(Q, pi, t1, t2, o1, o2, N=600):
    A = Q.shape[0]
    mult = np.where(np.eye(A, dtype=bool), 1.0, Q)

    def branch(t, a_w, b):
        out = np.zeros((A, A))
        for x in (np.arange(N) + 0.5) / N * t:
            w1 = a_w @ scipy_linalg.expm(Q * x)
            w2 = scipy_linalg.expm(Q * (t - x))[:, b]
            out += np.outer(w1, w2) * mult * (t / N)
        return out
    M1 = scipy_linalg.expm(Q * t1)[:, o1]
    M2 = scipy_linalg.expm(Q * t2)[:, o2]
    P = float(np.sum(pi * M1 * M2))
    return (branch(t1, pi * M2, o1) + branch(t2, pi * M1, o2)) / P


def _cherry(A, o1, o2, t1=0.7, t2=0.4):
    aln = np.array([[A], [o1], [o2]], dtype=np.int32)       # root unobserved
    return aln, oracle.Tree([-1, 0, 0], [0.0, t1, t2])


def _irrev_rate(rng, A=4):
    Q = rng.uniform(0.05, 1.0, (A, A))
    for a in range(A):
        Q[a, (a + 1) % A] += 2.0
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(1))
    return Q


def test_quadrature_matches_reversible_oracle():
    m = oracle.hky85_diag(2.0, [0.1, 0.4, 0.3, 0.2])
    V, mu, pi = m['eigenvectors'], m['eigenvalues'], m['pi']
    sp = np.sqrt(pi)
    Q = (V * mu) @ V.T / sp[:, None] * sp[None, :]
    aln, tree = _cherry(4, 1, 3)
    q = _quadrature(Q, pi, 0.7, 0.4, 1, 3)
    np.testing.assert_allclose(oracle.Counts(aln, tree, m, branch_mask=None)[:, :, 0], q, atol=2e-6)


def test_irrev_exact_matches_quadrature_and_reference_formula_is_the_transpose():
    rng = np.random.default_rng(3)
    Q = _irrev_rate(rng)
    pi = np.full(4, 0.25)
    m = oracle.irrev_model_from_rate_matrix(Q, pi)
    assert np.any(np.abs(m['eigenvalues'].imag) > 1e-3)
    aln, tree = _cherry(4, 1, 3)
    q = _quadrature(Q, pi, 0.7, 0.4, 1, 3)
    exact = oracle.Counts(aln, tree, m, branch_mask=None, irrev_exact=True)[:, :, 0]
    np.testing.assert_allclose(exact, q, atol=2e-6)
    ref = oracle.Counts(aln, tree, m, branch_mask=None)[:, :, 0]
    assert np.abs(ref - q).max() > 1e-2
    # the reference's formula is Q_ij int (e^{Qs} D)_i (U^T e^{Q(t-s)})_j ds: the
    # integral of the transposed process, with Q_ij kept
    A = 4
    mult = np.where(np.eye(A, dtype=bool), 1.0, Q)
    M1 = scipy_linalg.expm(Q * 0.7)[:, 1]
    M2 = scipy_linalg.expm(Q * 0.4)[:, 3]
    P = float(np.sum(pi * M1 * M2))
    N = 600

    def tb(t, a_w, b):
        out = np.zeros((A, A))
        for x in (np.arange(N) + 0.5) / N * t:
            w1 = scipy_linalg.expm(Q * x) @ a_w
            w2 = scipy_linalg.expm(Q * (t - x))[b, :]
            out += np.outer(w1, w2) * mult * (t / N)
        return out
    transposed = (tb(0.7, pi * M2, 1) + tb(0.4, pi * M1, 3)) / P
    np.testing.assert_allclose(ref, transposed, atol=2e-6)


def test_reversible_model_in_irreversible_form():
    m = oracle.hky85_diag(3.0, [0.2, 0.3, 0.1, 0.4])
    W, mu, pi = m['eigenvectors'], m['eigenvalues'], m['pi']
    sp = np.sqrt(pi)
    mi = {'eigenvalues': mu.astype(complex), 'eigenvectors': (W / sp[:, None]).astype(complex),
          'eigenvectors_inv': (W.T * sp[None, :]).astype(complex), 'pi': pi, 'reversible': False}
    rng = np.random.default_rng(4)
    aln = rng.integers(0, 6, size=(7, 20)).astype(np.int32)
    tree = oracle.Tree([-1, 0, 0, 1, 1, 2, 2], [0, 0.1, 0.2, 0.3, 0.1, 0.2, 0.05])
    rev = oracle.Counts(aln, tree, m, branch_mask=None)
    np.testing.assert_allclose(oracle.Counts(aln, tree, mi, branch_mask=None, irrev_exact=True), rev, atol=1e-10)
    assert np.abs(oracle.Counts(aln, tree, mi, branch_mask=None) - rev).max() > 1e-3
    np.testing.assert_allclose(oracle.LogLike(aln, tree, mi), oracle.LogLike(aln, tree, m), atol=1e-12)
