"""Host-side FP64 model constructors (inputs of the hot path).

The eigendecomposition stays in FP64 on the host, as in the reference
(subby/jax/models.py, subby/jax/diagonalize.py).  These build the same
``DiagModel`` values as subby's constructors:

* ``hky85_diag``             — subby/jax/models.py:7-73 (closed form)
* ``jukes_cantor_model``     — subby/jax/models.py:76-99 (QR of [1/sqrt(A) | I])
* ``f81_model``              — subby/jax/models.py:102-123 (QR of [sqrt(pi) | I])
* ``diagonalize_rate_matrix`` — subby/jax/diagonalize.py:6-26 (symmetrise + eigh)

``reversible_rate_matrix`` / ``random_reversible`` build the synthetic
general-reversible models used for the A=16/20/64 workloads.
"""
from __future__ import annotations

import numpy as np

from .types import DiagModel, RateModel


def hky85_diag(kappa: float, pi) -> DiagModel:
    pi = np.asarray(pi, dtype=np.float64)
    pA, pC, pG, pT = (float(x) for x in pi)
    pR, pY = pA + pG, pC + pT
    beta = 1.0 / (2.0 * pR * pY + 2.0 * kappa * (pA * pG + pC * pT))
    evals = np.array([0.0, -beta, -beta * (pR + kappa * pY), -beta * (pY + kappa * pR)])
    sp = np.sqrt(pi)
    w0 = sp.copy()
    w1 = np.array([sp[0] * pY, -sp[1] * pR, sp[2] * pY, -sp[3] * pR]) / np.sqrt(pR * pY)
    w2 = np.array([0.0, sp[1] * pT, 0.0, -sp[3] * pC]) / np.sqrt(pC * pT * pY)
    w3 = np.array([sp[0] * pG, 0.0, -sp[2] * pA, 0.0]) / np.sqrt(pA * pG * pR)
    return DiagModel(evals, np.stack([w0, w1, w2, w3], axis=-1), pi)


def jukes_cantor_model(A: int) -> DiagModel:
    pi = np.full(A, 1.0 / A)
    evals = np.zeros(A)
    evals[1:] = -float(A) / (A - 1.0)
    q, _ = np.linalg.qr(np.column_stack([np.full(A, 1.0 / np.sqrt(A)), np.eye(A)]))
    return DiagModel(evals, q[:, :A], pi)


def f81_model(pi) -> DiagModel:
    pi = np.asarray(pi, dtype=np.float64)
    A = len(pi)
    mu = 1.0 / (1.0 - np.sum(pi ** 2))
    evals = np.zeros(A)
    evals[1:] = -mu
    q, _ = np.linalg.qr(np.column_stack([np.sqrt(pi), np.eye(A)]))
    return DiagModel(evals, q[:, :A], pi)


def diagonalize_rate_matrix(subRate, rootProb) -> DiagModel:
    subRate = np.asarray(subRate, dtype=np.float64)
    pi = np.asarray(rootProb, dtype=np.float64)
    sp = np.sqrt(pi)
    S = subRate * sp[:, None] / sp[None, :]
    S = 0.5 * (S + S.T)
    evals, evecs = np.linalg.eigh(S)
    return DiagModel(evals, evecs, pi)


def ensure_diag(model) -> DiagModel:
    """RateModel -> DiagModel (subby/jax/__init__.py:44-50); DiagModel as is."""
    if isinstance(model, RateModel):
        return diagonalize_rate_matrix(model.subRate, model.rootProb)
    if isinstance(model, dict):
        return DiagModel(np.asarray(model['eigenvalues']), np.asarray(model['eigenvectors']),
                         np.asarray(model['pi']))
    if isinstance(model, DiagModel):
        return model
    if hasattr(model, 'eigenvalues') and hasattr(model, 'eigenvectors') and hasattr(model, 'pi'):
        if hasattr(model, 'eigenvectors_inv'):
            raise NotImplementedError("irreversible (complex) models are not supported")
        return DiagModel(np.asarray(model.eigenvalues), np.asarray(model.eigenvectors),
                         np.asarray(model.pi))
    raise TypeError(f"unsupported model type {type(model).__name__}")


def exchangeability_count(A: int) -> int:
    return A * (A - 1) // 2


def reversible_rate_matrix(log_exch, pi) -> np.ndarray:
    """Q_ij = s_ij pi_j / Z (i != j), rows sum to 0, -sum_i pi_i Q_ii = 1.

    ``log_exch`` holds log s_ij for i < j in row-major upper-triangle order.
    """
    pi = np.asarray(pi, dtype=np.float64)
    A = len(pi)
    s = np.zeros((A, A))
    s[np.triu_indices(A, 1)] = np.exp(np.asarray(log_exch, dtype=np.float64))
    s = s + s.T
    Q = s * pi[None, :]
    np.fill_diagonal(Q, 0.0)
    Q /= np.sum(pi * Q.sum(axis=1))
    np.fill_diagonal(Q, -Q.sum(axis=1))
    return Q


def random_reversible(A: int, rng: np.random.Generator, exch_sigma: float = 1.0,
                      dirichlet_alpha: float = 1.0):
    """Random reversible model: s_ij ~ LogNormal(0, sigma), pi ~ Dirichlet(alpha).

    Returns (DiagModel, log_exch, pi).
    """
    log_exch = rng.normal(0.0, exch_sigma, size=exchangeability_count(A))
    pi = rng.dirichlet(np.full(A, dirichlet_alpha))
    pi = np.maximum(pi, 1e-6)
    pi = pi / pi.sum()
    Q = reversible_rate_matrix(log_exch, pi)
    return diagonalize_rate_matrix(Q, pi), log_exch, pi


def force_near_degenerate(model: DiagModel, rng: np.random.Generator,
                          target_fraction: float = 0.05, cluster: int = 5,
                          lo: float = 1e-10, hi: float = 1e-7):
    """Pull clusters of consecutive non-zero eigenvalues to within ``hi``.

    Each cluster member gets eigenvalue base + delta with delta log-uniform in
    [lo, hi] (the first member keeps delta = 0), so every pair inside a
    cluster differs by less than ``hi``: the pairs straddle the 1e-8
    degeneracy threshold of the J(t) integrals.  Eigenvectors are kept, so
    M(t) rows still sum to one.  Returns (model, number of forced pairs).
    """
    ev = np.array(model.eigenvalues, dtype=np.float64)
    A = len(ev)
    order = np.argsort(ev)
    nz = [i for i in order if abs(ev[i]) > 1e-12]
    need = int(np.ceil(target_fraction * A * (A - 1) / 2))
    per = cluster * (cluster - 1) // 2
    n_clusters = min(len(nz) // cluster, int(np.ceil(need / per)))
    starts = np.sort(rng.choice(len(nz) // cluster, size=n_clusters, replace=False)) * cluster
    pairs = 0
    for s0 in starts:
        idx = nz[s0:s0 + cluster]
        base = ev[idx[0]]
        for j, i in enumerate(idx):
            ev[i] = base if j == 0 else base + np.exp(rng.uniform(np.log(lo), np.log(hi)))
        pairs += per
    return DiagModel(ev, np.array(model.eigenvectors), np.array(model.pi)), pairs
