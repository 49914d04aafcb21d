"""Single-branch CTMC integrals: ``ExpectedCounts(model, t)``
(subby/jax/ctmc.py:21-189; oracle subby/oracle/oracle.py:1909-2105).

result[..., a, b, i, j] = E[N_i->j(t) | X(0) = a, X(t) = b]   (i != j)
result[..., a, b, i, i] = E[T_i(t)   | X(0) = a, X(t) = b]    (dwell time)

for one branch of length t — no alignment and no tree, a model-level
quantity like the eigendecomposition, and computed the same way: on the host
in FP64.  The O(A^6) sum over (a, b, i, j, k, l) is two matrix products,
W = P J P^T with P[(a, i), k] = V_ak V_ik (reversible, symmetrised basis,
divided by S_t = V e^{mu t} V^T) or L J R^T with L[(a, i), k] = V_ak V^-1_ki,
R[(b, j), l] = V_jl V^-1_lb (irreversible, divided by M = Re V e^{mu t}
V^-1, the rate factor taken as Re(Q_ij W)); entries whose denominator is
below 1e-300 are 0, as in the reference.  Batched models (*H) and RateModels
are accepted.
"""
from __future__ import annotations

import numpy as np

from .models import batch_shape, ensure_diag, unbatch
from .types import IrrevDiagModel

_DEGENERATE = 1e-8


def _J(mu, t):
    """J_kl(t) = (e^{mu_k t} - e^{mu_l t}) / (mu_k - mu_l), t e^{mu_k t} when
    |mu_k - mu_l| < 1e-8."""
    e = np.exp(mu * t)
    diff = mu[:, None] - mu[None, :]
    deg = np.abs(diff) < _DEGENERATE
    return np.where(deg, t * e[:, None] * np.ones_like(diff), (e[:, None] - e[None, :]) / np.where(deg, 1.0, diff))


def _reversible(mu, V, t):
    A = len(mu)
    S_t = (V * np.exp(mu * t)) @ V.T
    S = (V * mu) @ V.T
    P = (V[:, None, :] * V[None, :, :]).reshape(A * A, A)           # [(a, i), k]
    W = (P @ _J(mu, t) @ P.T).reshape(A, A, A, A).transpose(0, 2, 1, 3)   # [a, b, i, j]
    rate = np.where(np.eye(A, dtype=bool), 1.0, S)
    ok = np.abs(S_t) >= 1e-300
    return np.where(ok[:, :, None, None], rate[None, None] * W / np.where(ok, S_t, 1.0)[:, :, None, None], 0.0)


def _irreversible(mu, V, Vi, t):
    A = len(mu)
    M = ((V * np.exp(mu * t)) @ Vi).real
    Q = (V * mu) @ Vi
    L = (V[:, None, :] * Vi.T[None, :, :]).reshape(A * A, A)        # [(a, i), k] = V_ak Vi_ki
    Rr = (V[None, :, :] * Vi.T[:, None, :]).reshape(A * A, A)       # [(b, j), l] = V_jl Vi_lb
    W = (L @ _J(mu, t) @ Rr.T).reshape(A, A, A, A).transpose(0, 2, 1, 3)  # [a, b, i, j]
    rate = np.where(np.eye(A, dtype=bool), 1.0 + 0.0j, Q)
    ok = np.abs(M) >= 1e-300
    return np.where(ok[:, :, None, None], (rate[None, None] * W).real / np.where(ok, M, 1.0)[:, :, None, None], 0.0)


def _one(m, t):
    if isinstance(m, IrrevDiagModel):
        return _irreversible(np.asarray(m.eigenvalues, np.complex128), np.asarray(m.eigenvectors, np.complex128),
                             np.asarray(m.eigenvectors_inv, np.complex128), t)
    return _reversible(np.asarray(m.eigenvalues, np.float64), np.asarray(m.eigenvectors, np.float64), t)


def ExpectedCounts(model, t: float) -> np.ndarray:
    """(*H, A, A, A, A) FP64 endpoint-conditioned dwell times (i == j) and
    substitution counts (i != j) of one branch of length t."""
    m = ensure_diag(model)
    t = float(t)
    H = batch_shape(m)
    if not H:
        return _one(m, t)
    _, ms = unbatch(m)
    return np.stack([_one(x, t) for x in ms]).reshape(tuple(H) + (len(np.asarray(ms[0].pi)),) * 4)


def expected_counts_eigen(eigenvalues, eigenvectors, pi, t) -> np.ndarray:
    """ExpectedCounts of a reversible eigensystem (subby/jax/ctmc.py:21-91)."""
    del pi
    return _reversible(np.asarray(eigenvalues, np.float64), np.asarray(eigenvectors, np.float64), float(t))


def expected_counts_eigen_irrev(eigenvalues, eigenvectors, eigenvectors_inv, pi, t) -> np.ndarray:
    """ExpectedCounts of an irreversible eigensystem (subby/jax/ctmc.py:94-158)."""
    del pi
    return _irreversible(np.asarray(eigenvalues, np.complex128), np.asarray(eigenvectors, np.complex128),
                         np.asarray(eigenvectors_inv, np.complex128), float(t))
