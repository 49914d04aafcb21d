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

Irreversible models: ``irrev_model_from_rate_matrix`` /
``diagonalize_irreversible`` (subby/jax/diagonalize.py:49-138; oracle
subby/oracle/oracle.py:265-301: numpy ``eig`` and ``inv`` in complex128) and
``random_irreversible`` (synthetic, with complex eigenvalue pairs).

Rate heterogeneity: ``gamma_rate_categories`` (Yang 1994 quantile medians,
subby/jax/models.py:126-158) and ``scale_model`` (subby/jax/models.py:
160-186; a (K,) multiplier adds a leading batch dimension).

Codons: ``gy94_model`` / ``gy94_rate_matrix`` (subby/jax/models.py:189-232).
Reversibility: ``check_detailed_balance``, ``model_from_rate_matrix`` /
``diagonalize_rate_matrix_auto``.  Model preparation under subby.jax's
names: ``compute_J`` (and the complex / per-row variants) and
``compute_sub_matrices`` (and the irreversible variant).
"""
from __future__ import annotations

import numpy as np

from .types import DiagModel, IrrevDiagModel, RateModel


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


def diagonalize_irreversible(subRate, rootProb) -> IrrevDiagModel:
    """R = V diag(mu) V^-1 in complex128 (numpy eig, inv)."""
    subRate = np.asarray(subRate, dtype=np.float64)
    mu, V = np.linalg.eig(subRate)
    return IrrevDiagModel(mu.astype(np.complex128), V.astype(np.complex128),
                          np.linalg.inv(V).astype(np.complex128), np.asarray(rootProb, dtype=np.float64))


def irrev_model_from_rate_matrix(subRate, pi) -> IrrevDiagModel:
    return diagonalize_irreversible(subRate, pi)


def stationary_distribution(subRate) -> np.ndarray:
    """pi with pi^T R = 0, sum 1 (FP64)."""
    subRate = np.asarray(subRate, dtype=np.float64)
    A = subRate.shape[0]
    M = np.vstack([subRate.T, np.ones(A)])
    b = np.zeros(A + 1)
    b[-1] = 1.0
    return np.linalg.lstsq(M, b, rcond=None)[0]


def random_irreversible(A: int, rng: np.random.Generator, cycle: float = 2.0) -> IrrevDiagModel:
    """Random irreversible rate matrix with a strong cyclic component
    (state a -> a+1 mod A), which gives complex eigenvalue pairs; pi is its
    stationary distribution; normalised to one expected substitution per
    unit time."""
    Q = rng.uniform(0.05, 1.0, size=(A, A))
    for a in range(A):
        Q[a, (a + 1) % A] += cycle
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(axis=1))
    pi = stationary_distribution(Q)
    Q /= -np.sum(pi * np.diag(Q))
    return irrev_model_from_rate_matrix(Q, pi)


def is_irrev(model) -> bool:
    return isinstance(model, IrrevDiagModel) or hasattr(model, 'eigenvectors_inv') or (
        isinstance(model, dict) and ('eigenvectors_inv' in model or model.get('reversible', True) is False))


def ensure_diag(model):
    """RateModel -> DiagModel (subby/jax/__init__.py:44-50); DiagModel and
    IrrevDiagModel as they are (dicts with 'eigenvectors_inv' become
    IrrevDiagModel)."""
    if isinstance(model, RateModel):
        return diagonalize_rate_matrix(model.subRate, model.rootProb)
    if isinstance(model, (DiagModel, IrrevDiagModel)):
        return model
    if isinstance(model, dict):
        if 'eigenvectors_inv' in model:
            return IrrevDiagModel(np.asarray(model['eigenvalues'], np.complex128),
                                  np.asarray(model['eigenvectors'], np.complex128),
                                  np.asarray(model['eigenvectors_inv'], np.complex128), np.asarray(model['pi']))
        return DiagModel(np.asarray(model['eigenvalues']), np.asarray(model['eigenvectors']),
                         np.asarray(model['pi']))
    if hasattr(model, 'eigenvalues') and hasattr(model, 'eigenvectors') and hasattr(model, 'pi'):
        if hasattr(model, 'eigenvectors_inv'):
            return IrrevDiagModel(np.asarray(model.eigenvalues, np.complex128),
                                  np.asarray(model.eigenvectors, np.complex128),
                                  np.asarray(model.eigenvectors_inv, np.complex128), np.asarray(model.pi))
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


def near_degenerate_reversible(A: int, rng: np.random.Generator, target_fraction: float = 0.05,
                               exch_sigma: float = 1.0, dirichlet_alpha: float = 1.0,
                               split_max: float = 9e-8):
    """Random reversible model with ~``target_fraction`` of its eigenvalue
    pairs within ~1e-7 of each other, and M(t) >= 0 for every t.

    s_ij ~ LogNormal(0, sigma), pi ~ Dirichlet(alpha), then a block B of d
    states is made exchangeable (common pi inside B, one common within-block
    exchangeability, and for every outside state k one common s_ik).  That
    gives an exactly (d-1)-fold eigenvalue; d is the smallest size whose
    (d-1)(d-2)/2 pairs reach the target.  The within-block exchangeabilities
    are then multiplied by (1 + c eps_ij), eps ~ U(-1, 1), which splits the
    degenerate eigenvalue into a cluster; c is chosen so that the widest pair
    sits just under ``split_max`` and the pairwise gaps spread over
    ~1e-10..1e-7 (straddling the 1e-8 degeneracy threshold of the J(t)
    integrals).  Returns (DiagModel, log_exch, pi, forced_pairs).
    """
    need = target_fraction * A * (A - 1) / 2
    d = 3
    while (d - 1) * (d - 2) / 2 < need and d < A:
        d += 1
    log_exch = rng.normal(0.0, exch_sigma, size=exchangeability_count(A))
    pi = rng.dirichlet(np.full(A, dirichlet_alpha))
    pi = np.maximum(pi, 1e-6)
    pi /= pi.sum()
    s = np.zeros((A, A))
    iu = np.triu_indices(A, 1)
    s[iu] = np.exp(log_exch)
    s = s + s.T
    B = np.sort(rng.choice(A, size=d, replace=False))
    inB = np.zeros(A, dtype=bool)
    inB[B] = True
    pi[B] = pi[B].mean()
    cin = np.exp(rng.normal(0.0, exch_sigma))
    for k in np.nonzero(~inB)[0]:
        s[B, k] = s[k, B] = s[B[0], k]
    eps = rng.uniform(-1.0, 1.0, size=(d, d))

    def build(scale):
        ss = s.copy()
        for a in range(d):
            for b in range(a + 1, d):
                ss[B[a], B[b]] = ss[B[b], B[a]] = cin * (1.0 + scale * eps[a, b])
        le = np.log(ss[iu])
        Q = reversible_rate_matrix(le, pi)
        return diagonalize_rate_matrix(Q, pi), le

    # eigenvalue splits are linear in the perturbation: scale it so that the
    # widest pair of the cluster sits just under `split_max`
    probe = 1e-4
    m0, _ = build(probe)
    ev = np.sort(m0.eigenvalues)
    # the cluster is the run of d-1 eigenvalues with the smallest total spread
    widths = np.array([ev[i + d - 2] - ev[i] for i in range(len(ev) - d + 2)])
    w = widths.min()
    model, log_exch = build(probe * split_max / max(w, 1e-300))
    return model, log_exch, pi, (d - 1) * (d - 2) // 2


def gamma_rate_categories(alpha: float, K: int):
    """(rates, weights), each (K,): quantile medians of Gamma(alpha, 1/alpha)
    at the midpoints of K equal-probability bins, by 64 bisection steps,
    normalised to mean rate 1; uniform weights."""
    from scipy.special import gammainc
    edges = np.linspace(0.0, 1.0, K + 1)
    mids = 0.5 * (edges[:-1] + edges[1:])
    lo = np.zeros(K)
    hi = np.full(K, max(50.0, 10.0 / alpha))
    for _ in range(64):
        mid = 0.5 * (lo + hi)
        below = gammainc(alpha, mid * alpha) < mids
        lo = np.where(below, mid, lo)
        hi = np.where(below, hi, mid)
    rates = 0.5 * (lo + hi)
    return rates * K / np.sum(rates), np.full(K, 1.0 / K)


def scale_model(model, rate_multiplier):
    """Eigenvalues times the rate multiplier; a (K,) multiplier gives a model
    with a leading batch dimension K (eigenvectors and pi broadcast)."""
    m = ensure_diag(model)
    r = np.asarray(rate_multiplier, dtype=np.float64)
    if r.ndim == 0:
        return m._replace(eigenvalues=np.asarray(m.eigenvalues) * r)
    K = r.shape[0]
    ev = np.asarray(m.eigenvalues)[None, ...] * r.reshape((K,) + (1,) * np.ndim(m.eigenvalues))
    fields = {f: np.broadcast_to(np.asarray(getattr(m, f))[None, ...], (K,) + np.shape(getattr(m, f)))
              for f in m._fields if f != 'eigenvalues'}
    return type(m)(eigenvalues=ev, **fields)


def batch_shape(model):
    """Leading batch dimensions *H of a (possibly batched) diagonal model."""
    m = ensure_diag(model)
    return tuple(np.shape(m.eigenvalues)[:-1])


def unbatch(model):
    """(*H, list of the single models in C order)."""
    m = ensure_diag(model)
    H = batch_shape(m)
    if not H:
        return H, [m]
    return H, [type(m)(**{f: np.asarray(getattr(m, f))[idx] for f in m._fields}) for idx in np.ndindex(*H)]


def check_detailed_balance(subRate, pi, tol: float = 1e-10) -> bool:
    """pi_i R_ij == pi_j R_ji within tol for every pair."""
    R = np.asarray(subRate, dtype=np.float64)
    p = np.asarray(pi, dtype=np.float64)
    F = p[:, None] * R
    return bool(np.all(np.abs(F - F.T) <= tol))


def model_from_rate_matrix(subRate, pi, reversible=None, tol: float = 1e-10):
    """DiagModel when reversible (detailed balance checked when None), else
    IrrevDiagModel."""
    if reversible is None:
        reversible = check_detailed_balance(subRate, pi, tol)
    return diagonalize_rate_matrix(subRate, pi) if reversible else diagonalize_irreversible(subRate, pi)


def gy94_rate_matrix(omega: float, kappa: float, pi=None) -> np.ndarray:
    """Goldman-Yang 1994 rate matrix over the 61 sense codons (ACGT
    lexicographic order, stops removed): Q_ij = pi_j kappa^[transition]
    omega^[non-synonymous] for codons one nucleotide apart, 0 otherwise;
    rows sum to 0, scaled so that -sum_i pi_i Q_ii = 1
    (subby/oracle/oracle.py:388-471, subby/jax/models.py:189-232)."""
    from .formats import genetic_code
    gc = genetic_code()
    sense = [gc["codons"][i] for i in gc["sense_indices"]]
    aa = np.array(gc["sense_amino_acids"])
    A = len(sense)
    p = np.full(A, 1.0 / A) if pi is None else np.asarray(pi, dtype=np.float64)
    nuc = np.array([[c[k] for k in range(3)] for c in sense])            # (61, 3) letters
    differs = nuc[:, None, :] != nuc[None, :, :]                        # (61, 61, 3)
    one = differs.sum(axis=2) == 1
    pos = np.argmax(differs, axis=2)
    a = np.take_along_axis(nuc[:, None, :].repeat(A, 1), pos[..., None], 2)[..., 0]
    b = np.take_along_axis(nuc[None, :, :].repeat(A, 0), pos[..., None], 2)[..., 0]
    purine = np.isin(a, ["A", "G"]) == np.isin(b, ["A", "G"])          # A<->G or C<->T
    Q = np.where(one, p[None, :], 0.0)
    Q = Q * np.where(one & purine, kappa, 1.0) * np.where(one & (aa[:, None] != aa[None, :]), omega, 1.0)
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(axis=1))
    return Q / -np.sum(p * np.diag(Q))


def gy94_model(omega: float, kappa: float, pi=None) -> DiagModel:
    """The GY94 codon model (61 states) as a DiagModel (reversible: pi_i Q_ij
    = pi_j Q_ji).  The kernels take A up to 64 in sizes 2..8, 16, 20, 32, 64:
    61 states run through ``subby_gb300.embed.EmbeddedPlan``."""
    p = np.full(61, 1.0 / 61) if pi is None else np.asarray(pi, dtype=np.float64)
    return diagonalize_rate_matrix(gy94_rate_matrix(omega, kappa, p), p)


def diagonalize_rate_matrix_auto(subRate, rootProb, reversible=None, tol: float = 1e-10):
    """subby.jax's name for ``model_from_rate_matrix``
    (subby/jax/diagonalize.py:89-111)."""
    return model_from_rate_matrix(subRate, rootProb, reversible=reversible, tol=tol)


# Host FP64 model preparation, as subby.jax exposes it (the plans compute the
# same tables internally; these are for callers that want them).

def compute_J(eigenvalues, distances) -> np.ndarray:
    """(*H, R, A, A) J_kl(t_n) = (e^{mu_k t} - e^{mu_l t}) / (mu_k - mu_l), and
    t e^{mu_k t} when |mu_k - mu_l| < 1e-8 (subby/jax/eigensub.py:7-50;
    complex eigenvalues as compute_J_complex, :234-262)."""
    mu = np.asarray(eigenvalues)
    mu = mu.astype(np.complex128 if np.iscomplexobj(mu) else np.float64)
    t = np.asarray(distances, dtype=np.float64)
    E = np.exp(mu[..., None, :] * t[:, None])                                  # (*H, R, A)
    diff = mu[..., :, None] - mu[..., None, :]                                 # (*H, A, A)
    deg = (np.abs(diff) < 1e-8)[..., None, :, :]
    dd = (E[..., :, None] - E[..., None, :]) / np.where(deg, 1.0, diff[..., None, :, :])
    return np.where(deg, t[:, None, None] * E[..., :, None], dd)


compute_J_complex = compute_J


def compute_J_per_row(eigenvalues, distances) -> np.ndarray:
    """(R, A, A) J with each branch's own eigenvalues (eigenvalues (R, A))
    (subby/jax/eigensub.py:440-506)."""
    mu = np.asarray(eigenvalues)
    t = np.asarray(distances, dtype=np.float64)
    return np.stack([compute_J(mu[n], t[n:n + 1])[0] for n in range(len(t))])


compute_J_per_row_complex = compute_J_per_row


def compute_sub_matrices(model, distances) -> np.ndarray:
    """(*H, R, A, A) M_ij(t) = sqrt(pi_j / pi_i) sum_k V_ik e^{mu_k t} V_jk
    (subby/jax/diagonalize.py:141-172); irreversible models as
    compute_sub_matrices_irrev."""
    m = ensure_diag(model)
    if isinstance(m, IrrevDiagModel):
        return compute_sub_matrices_irrev(m, distances)
    V = np.asarray(m.eigenvectors, dtype=np.float64)
    mu = np.asarray(m.eigenvalues, dtype=np.float64)
    sp = np.sqrt(np.asarray(m.pi, dtype=np.float64))
    t = np.asarray(distances, dtype=np.float64)
    E = np.exp(mu[..., None, :] * t[:, None])                                  # (*H, R, A)
    S = np.einsum('...ik,...rk,...jk->...rij', V, E, V)
    return S / sp[..., None, :, None] * sp[..., None, None, :]


def compute_sub_matrices_irrev(model, distances) -> np.ndarray:
    """(*H, R, A, A) M(t) = Re(V e^{mu t} V^-1) (subby/jax/diagonalize.py:114-138)."""
    m = ensure_diag(model)
    V = np.asarray(m.eigenvectors, dtype=np.complex128)
    Vi = np.asarray(m.eigenvectors_inv, dtype=np.complex128)
    mu = np.asarray(m.eigenvalues, dtype=np.complex128)
    t = np.asarray(distances, dtype=np.float64)
    E = np.exp(mu[..., None, :] * t[:, None])
    return np.einsum('...ik,...rk,...kj->...rij', V, E, Vi).real
