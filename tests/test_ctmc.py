"""ExpectedCounts (subby_gb300/ctmc.py) against the reference oracle's
outputs (tests/golden/models/expected_counts.npz: HKY85, JC with its
degenerate eigenvalues, a 6-state reversible model, 4- and 5-state
irreversible models) and, at larger A, against exact identities: the dwell
times of a branch sum to t, and averaging over stationary endpoints gives
the unconditional rates (E N_ij = pi_i Q_ij t, E T_i = pi_i t).  CPU only."""
import numpy as np
import pytest
from scipy.linalg import expm

import subby_gb300 as sg
from subby_gb300 import ctmc, models
from subby_gb300.types import DiagModel, IrrevDiagModel, RateModel

Z = np.load(__file__.replace("test_ctmc.py", "golden/models/expected_counts.npz"))


@pytest.mark.parametrize("name", ["hky", "jc", "rev6", "irrev4", "irrev5"])
def test_matches_reference(name):
    g = {k.split("/", 1)[1]: Z[k] for k in Z.files if k.startswith(name + "/")}
    if "eigenvectors_inv" in g:
        m = IrrevDiagModel(g["eigenvalues"], g["eigenvectors"], g["eigenvectors_inv"], g["pi"])
    else:
        m = DiagModel(g["eigenvalues"], g["eigenvectors"], g["pi"])
    np.testing.assert_allclose(ctmc.ExpectedCounts(m, float(g["t"])), g["expected"], rtol=1e-10, atol=1e-13)


def _identities(m, Q, pi, t):
    E = ctmc.ExpectedCounts(m, t)
    A = len(pi)
    M = expm(Q * t)
    dwell = np.einsum("abii->ab", E)
    np.testing.assert_allclose(dwell, t, rtol=1e-9)
    avg = np.einsum("a,ab,abij->ij", pi, M, E)
    want = np.where(np.eye(A, dtype=bool), np.diag(pi) * t, pi[:, None] * Q * t)
    np.testing.assert_allclose(avg, want, rtol=1e-8, atol=1e-12)
    return E


@pytest.mark.parametrize("A", [20, 32])
def test_identities_reversible(A):
    rng = np.random.default_rng(A)
    m, log_exch, pi = models.random_reversible(A, rng, dirichlet_alpha=3.0)
    Q = models.reversible_rate_matrix(log_exch, pi)
    E = _identities(m, Q, pi, 0.4)
    np.testing.assert_allclose(sg.ExpectedCounts(RateModel(Q, pi), 0.4), E, rtol=1e-8, atol=1e-12)


def test_identities_irreversible_and_batches():
    rng = np.random.default_rng(8)
    m = models.random_irreversible(8, rng)
    Q = ((m.eigenvectors * m.eigenvalues) @ m.eigenvectors_inv).real
    _identities(m, Q, np.asarray(m.pi, np.float64), 0.6)
    base = models.hky85_diag(2.0, [0.25] * 4)
    batch = models.scale_model(base, np.array([0.5, 2.0]))
    E = ctmc.ExpectedCounts(batch, 0.3)
    assert E.shape == (2, 4, 4, 4, 4)
    for k, r in enumerate((0.5, 2.0)):
        np.testing.assert_allclose(E[k], ctmc.ExpectedCounts(models.scale_model(base, r), 0.3), rtol=1e-12)


def test_eigensystem_entry_points():
    rng = np.random.default_rng(2)
    m = models.random_reversible(5, rng)[0]
    np.testing.assert_array_equal(sg.expected_counts_eigen(m.eigenvalues, m.eigenvectors, m.pi, 0.3),
                                  sg.ExpectedCounts(m, 0.3))
    mi = models.random_irreversible(4, rng)
    np.testing.assert_array_equal(
        sg.expected_counts_eigen_irrev(mi.eigenvalues, mi.eigenvectors, mi.eigenvectors_inv, mi.pi, 0.3),
        sg.ExpectedCounts(mi, 0.3))
