"""The product's host model constructors (subby_gb300/models.py) against the
reference's (subby/oracle/oracle.py:103-205, 265-386; fixtures made by
tests/golden/make_models_golden.py).  Eigenvectors are unique only up to
sign (and rotation inside a degenerate eigenspace), so the comparison is on
what the kernels consume: eigenvalues, the symmetrised rate matrix
S = V diag(mu) V^T (reversible) or Q = V diag(mu) V^-1 (irreversible), and
M(t) at several branch lengths — FP64, 1e-12 (1e-10 for eig).  CPU only."""
import numpy as np
import pytest

from subby_gb300 import models
from subby_gb300.types import DiagModel, IrrevDiagModel

Z = np.load(__file__.replace("test_models_golden.py", "golden/models/constructors.npz"))
T = (0.05, 0.3, 2.0)


def _ref(name):
    return {k.split("/", 1)[1]: Z[k] for k in Z.files if k.startswith(name + "/")}


def _check_reversible(m, ref):
    np.testing.assert_allclose(m.pi, ref["pi"], rtol=1e-15)
    np.testing.assert_allclose(np.sort(m.eigenvalues), np.sort(ref["eigenvalues"]), rtol=1e-12, atol=1e-12)
    sym = lambda V, mu: (V * mu) @ V.T  # noqa: E731
    np.testing.assert_allclose(sym(m.eigenvectors, m.eigenvalues), sym(ref["eigenvectors"], ref["eigenvalues"]),
                               atol=1e-12)
    sp = np.sqrt(ref["pi"])
    for t in T:
        M = lambda V, mu: (V * np.exp(mu * t)) @ V.T / sp[:, None] * sp[None, :]  # noqa: E731
        np.testing.assert_allclose(M(m.eigenvectors, m.eigenvalues), M(ref["eigenvectors"], ref["eigenvalues"]),
                                   atol=1e-12)


def _check_irreversible(m, ref):
    assert isinstance(m, IrrevDiagModel)
    np.testing.assert_allclose(m.pi, ref["pi"], rtol=1e-15)
    key = lambda w: np.lexsort((np.round(w.imag, 8), np.round(w.real, 8)))  # noqa: E731
    np.testing.assert_allclose(m.eigenvalues[key(m.eigenvalues)], ref["eigenvalues"][key(ref["eigenvalues"])],
                               atol=1e-10)
    for t in (0.0,) + T:
        M = lambda V, mu, Vi: ((V * np.exp(mu * t)) @ Vi).real  # noqa: E731
        np.testing.assert_allclose(M(m.eigenvectors, m.eigenvalues, m.eigenvectors_inv),
                                   M(ref["eigenvectors"], ref["eigenvalues"], ref["eigenvectors_inv"]), atol=1e-10)
    Q = ((m.eigenvectors * m.eigenvalues) @ m.eigenvectors_inv).real
    np.testing.assert_allclose(Q, ref["in_Q"], atol=1e-10)


@pytest.mark.parametrize("name", ["hky0", "hky1", "hky2"])
def test_hky85(name):
    r = _ref(name)
    _check_reversible(models.hky85_diag(float(r["in_kappa"]), r["in_pi"]), r)


@pytest.mark.parametrize("A", [2, 4, 20, 64])
def test_jukes_cantor(A):
    _check_reversible(models.jukes_cantor_model(A), _ref(f"jc{A}"))


@pytest.mark.parametrize("A", [4, 20])
def test_f81_and_rate_matrices(A):
    r = _ref(f"f81_{A}")
    _check_reversible(models.f81_model(r["in_pi"]), r)
    r = _ref(f"rev{A}")
    _check_reversible(models.diagonalize_rate_matrix(r["in_Q"], r["in_pi"]), r)
    r = _ref(f"auto_rev{A}")
    m = models.model_from_rate_matrix(r["in_Q"], r["in_pi"])
    assert isinstance(m, DiagModel)
    _check_reversible(m, r)
    r = _ref(f"irrev{A}")
    _check_irreversible(models.diagonalize_irreversible(r["in_Q"], r["in_pi"]), r)
    r = _ref(f"auto_irrev{A}")
    _check_irreversible(models.model_from_rate_matrix(r["in_Q"], r["in_pi"]), r)
    for kind in ("rev", "irrev"):
        q = _ref(f"{kind}{A}")
        assert models.check_detailed_balance(q["in_Q"], q["in_pi"]) == bool(Z[f"balance/{kind}{A}"])


@pytest.mark.parametrize("i", [0, 1])
def test_gy94(i):
    r = _ref(f"gy94_{i}")
    pi = r["in_pi"]
    m = models.gy94_model(float(r["in_omega"]), float(r["in_kappa"]), None if i == 0 else pi)
    _check_reversible(m, r)
    Q = models.gy94_rate_matrix(float(r["in_omega"]), float(r["in_kappa"]), pi)
    np.testing.assert_allclose(pi[:, None] * Q, (pi[:, None] * Q).T, atol=1e-15)   # detailed balance
    assert np.count_nonzero(Q[0]) == 1 + 8            # AAA: 9 one-nucleotide neighbours, TAA a stop


def test_model_preparation_helpers_match_the_oracle():
    """compute_J / compute_sub_matrices (host FP64, subby.jax's names) vs the
    oracle's restatement of the reference (pinned by the golden fixtures),
    single and *H-batched, reversible and irreversible."""
    import oracle
    rng = np.random.default_rng(9)
    m = models.random_reversible(6, rng)[0]
    t = rng.uniform(0.0, 1.0, 7)
    t[0] = 0.0
    np.testing.assert_allclose(models.compute_J(m.eigenvalues, t), oracle.compute_J(m.eigenvalues, t), rtol=1e-13)
    np.testing.assert_allclose(models.compute_sub_matrices(m, t), oracle.compute_sub_matrices(m._asdict(), t),
                               rtol=1e-12, atol=1e-15)
    mi = models.random_irreversible(5, rng)
    np.testing.assert_allclose(models.compute_J_complex(mi.eigenvalues, t),
                               oracle.compute_J_complex(mi.eigenvalues, t), rtol=1e-13)
    np.testing.assert_allclose(models.compute_sub_matrices(mi, t),
                               oracle.compute_sub_matrices_irrev(mi._asdict(), t), rtol=1e-12, atol=1e-14)
    b = models.scale_model(m, np.array([0.5, 2.0]))
    Jb, Mb = models.compute_J(b.eigenvalues, t), models.compute_sub_matrices(b, t)
    assert Jb.shape == (2, 7, 6, 6) and Mb.shape == (2, 7, 6, 6)
    for k, r in enumerate((0.5, 2.0)):
        mk = models.scale_model(m, r)
        np.testing.assert_allclose(Jb[k], models.compute_J(mk.eigenvalues, t), rtol=1e-14)
        np.testing.assert_allclose(Mb[k], models.compute_sub_matrices(mk, t), rtol=1e-13, atol=1e-16)
    rows = np.stack([m.eigenvalues, 2 * m.eigenvalues, m.eigenvalues])
    Jr = models.compute_J_per_row(rows, t[:3])
    for n in range(3):
        np.testing.assert_allclose(Jr[n], models.compute_J(rows[n], t[n:n + 1])[0], rtol=1e-15)
    assert models.diagonalize_rate_matrix_auto(models.reversible_rate_matrix(rng.normal(size=15), m.pi), m.pi) \
        ._fields == ("eigenvalues", "eigenvectors", "pi")
