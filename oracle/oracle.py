"""FP64 CPU oracle for the eigensubstitution hot path (TEST INFRASTRUCTURE ONLY).

This module checks the product and is never part of it: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline / reference arm of
``bench.py`` may import it.  The shipped path (``subby_gb300``) never calls it
and has no CPU fallback.

It restates, in vectorised numpy over alignment columns, the algorithms of
subby's explicit-loop oracle ``subby/oracle/oracle.py`` (ihh/subby).  Every
function cites the reference lines it follows.  The arithmetic order inside a
column follows the reference (same per-child rescaling, same 1e-300 floor,
same 1e-8 degeneracy threshold), so intermediates (U, logNormU, D, logNormD,
J, U_tilde, D_tilde, C) agree with the reference to FP64 rounding.

Parity is pinned: ``tests/test_oracle_golden.py`` checks this module against
fixtures produced by running the reference oracle itself
(``tests/golden/make_golden.py``) and, when the reference tree is mounted,
against the reference's own golden JSON files (``tests/golden/*.json`` of
ihh/subby).
"""
from __future__ import annotations

import numpy as np

DEGENERATE_THRESHOLD = 1e-8   # subby/oracle/oracle.py:955
RESCALE_FLOOR = 1e-300        # subby/oracle/oracle.py:822-823


class Tree:
    """(parentIndex, distanceToParent) pair; subby/formats.py:15-17."""

    def __init__(self, parentIndex, distanceToParent):
        self.parentIndex = np.asarray(parentIndex, dtype=np.int64)
        self.distanceToParent = np.asarray(distanceToParent, dtype=np.float64)


# ---------------------------------------------------------------------------
# Tree utilities — subby/oracle/oracle.py:19-62
# ---------------------------------------------------------------------------

def children_of(parentIndex):
    """left/right child and sibling; subby/oracle/oracle.py:19-49.

    The first child seen in index order is the left child, so left = min
    child index and right = max child index (subby/jax/_utils.py:46-75).
    """
    parentIndex = np.asarray(parentIndex)
    R = len(parentIndex)
    left = np.full(R, -1, dtype=np.int64)
    right = np.full(R, -1, dtype=np.int64)
    for n in range(1, R):
        p = parentIndex[n]
        if left[p] == -1:
            left[p] = n
        else:
            right[p] = n
    sibling = np.full(R, -1, dtype=np.int64)
    for n in range(1, R):
        p = parentIndex[n]
        sibling[n] = right[p] if left[p] == n else left[p]
    return left, right, sibling


def validate_binary_tree(parentIndex):
    """Raise ValueError unless every node has 0 or 2 children; oracle.py:52-62."""
    parentIndex = np.asarray(parentIndex)
    R = len(parentIndex)
    cnt = np.zeros(R, dtype=np.int64)
    for n in range(1, R):
        cnt[parentIndex[n]] += 1
    for n in range(R):
        if cnt[n] != 0 and cnt[n] != 2:
            raise ValueError(f"Node {n} has {cnt[n]} children; expected 0 or 2.")


def token_to_likelihood(alignment, A):
    """Tokens -> (R, C, A) likelihood vectors; subby/oracle/oracle.py:69-96.

    0..A-1 one-hot; A (ungapped-unobserved), A+1 (gapped), -1 (legacy gap)
    and anything else outside 0..A-1 give all-ones.
    """
    alignment = np.asarray(alignment)
    R, C = alignment.shape
    L = np.ones((R, C, A), dtype=np.float64)
    obs = (alignment >= 0) & (alignment < A)
    L[obs] = 0.0
    rr, cc = np.nonzero(obs)
    L[rr, cc, alignment[rr, cc]] = 1.0
    return L


# ---------------------------------------------------------------------------
# Models — subby/oracle/oracle.py:103-205, 304-335
# ---------------------------------------------------------------------------

def hky85_diag(kappa, pi):
    """Closed-form HKY85 eigensystem; subby/oracle/oracle.py:103-161."""
    pi = np.asarray(pi, dtype=np.float64)
    pA, pC, pG, pT = pi
    pR, pY = pA + pG, pC + pT
    beta = 1.0 / (2.0 * pR * pY + 2.0 * kappa * (pA * pG + pC * pT))
    ev = np.array([0.0, -beta, -beta * (pR + kappa * pY), -beta * (pY + kappa * pR)])
    sp = np.sqrt(pi)
    w0 = sp.copy()
    w1 = np.array([sp[0] * pY, -sp[1] * pR, sp[2] * pY, -sp[3] * pR]) / np.sqrt(pR * pY)
    w2 = np.array([0.0, sp[1] * pT, 0.0, -sp[3] * pC]) / np.sqrt(pC * pT * pY)
    w3 = np.array([sp[0] * pG, 0.0, -sp[2] * pA, 0.0]) / np.sqrt(pA * pG * pR)
    return {'eigenvalues': ev, 'eigenvectors': np.column_stack([w0, w1, w2, w3]), 'pi': pi}


def jukes_cantor_model(A):
    """JC model via QR of [1/sqrt(A) | I]; subby/oracle/oracle.py:164-181."""
    pi = np.ones(A) / A
    ev = np.zeros(A)
    ev[1:] = -float(A) / (A - 1.0)
    Q, _ = np.linalg.qr(np.column_stack([np.ones(A) / np.sqrt(A), np.eye(A)]))
    return {'eigenvalues': ev, 'eigenvectors': Q[:, :A], 'pi': pi}


def f81_model(pi):
    """F81 model normalised to rate 1; subby/oracle/oracle.py:184-205."""
    pi = np.asarray(pi, dtype=np.float64)
    A = len(pi)
    mu = 1.0 / (1.0 - np.sum(pi ** 2))
    ev = np.zeros(A)
    ev[1:] = -mu
    Q, _ = np.linalg.qr(np.column_stack([np.sqrt(pi), np.eye(A)]))
    return {'eigenvalues': ev, 'eigenvectors': Q[:, :A], 'pi': pi}


def diagonalize_rate_matrix(subRate, rootProb):
    """Symmetrise S_ij = R_ij sqrt(pi_i/pi_j) and eigh; oracle.py:304-335."""
    subRate = np.asarray(subRate, dtype=np.float64)
    pi = np.asarray(rootProb, dtype=np.float64)
    sp = np.sqrt(pi)
    S = subRate * sp[:, None] * (1.0 / sp)[None, :]
    S = 0.5 * (S + S.T)
    ev, V = np.linalg.eigh(S)
    return {'eigenvalues': ev, 'eigenvectors': V, 'pi': pi}


def diagonalize_irreversible(subRate, rootProb):
    """Complex eigensystem R = V diag(mu) V^-1 via numpy eig; oracle.py:265-288."""
    subRate = np.asarray(subRate, dtype=np.float64)
    mu, V = np.linalg.eig(subRate)
    return {'eigenvalues': mu, 'eigenvectors': V, 'eigenvectors_inv': np.linalg.inv(V),
            'pi': np.asarray(rootProb, dtype=np.float64), 'reversible': False}


def irrev_model_from_rate_matrix(subRate, pi):
    """oracle.py:291-301."""
    return diagonalize_irreversible(subRate, pi)


def is_irrev(model):
    """A model dict is irreversible when it says reversible=False
    (oracle.py:1442-1444) or carries V^-1."""
    return (not model.get('reversible', True)) or ('eigenvectors_inv' in model)


def compute_sub_matrices_irrev(model, distances):
    """M_ij(t) = Re sum_k V_ik e^{mu_k t} Vinv_kj; oracle.py:474-501."""
    V = np.asarray(model['eigenvectors'], dtype=np.complex128)
    Vi = np.asarray(model['eigenvectors_inv'], dtype=np.complex128)
    mu = np.asarray(model['eigenvalues'], dtype=np.complex128)
    t = np.asarray(distances, dtype=np.float64)
    E = np.exp(mu[None, :] * t[:, None])                    # (R, A)
    return np.einsum('ik,rk,kj->rij', V, E, Vi).real


def compute_J_complex(eigenvalues, distances):
    """Complex J^{kl}(t), 1e-8 degeneracy test on |mu_k - mu_l|; oracle.py:508-534."""
    mu = np.asarray(eigenvalues, dtype=np.complex128)
    t = np.asarray(distances, dtype=np.float64)
    E = np.exp(mu[None, :] * t[:, None])
    diff = mu[:, None] - mu[None, :]
    deg = np.abs(diff) < DEGENERATE_THRESHOLD
    safe = np.where(deg, 1.0, diff)
    J = (E[:, :, None] - E[:, None, :]) / safe[None]
    Jdeg = t[:, None, None] * E[:, :, None] * np.ones_like(diff)[None]
    return np.where(deg[None], Jdeg, J)


def eigenbasis_project_irrev(U, D, model):
    """U~_k = sum_b U_b V_bk, D~_k = sum_a D_a Vinv_ka; oracle.py:537-570."""
    V = np.asarray(model['eigenvectors'], dtype=np.complex128)
    Vi = np.asarray(model['eigenvectors_inv'], dtype=np.complex128)
    return U @ V, D @ Vi.T


def accumulate_C_complex(D_tilde, U_tilde, J, logNormU, logNormD, logLike, parentIndex,
                         branch_mask=None):
    """Complex C_kl,c = sum_{n>0} D~_k J_kl U~_l exp(lnD+lnU-lnL); oracle.py:573-603."""
    R, C, A = U_tilde.shape
    out = np.zeros((A, A, C), dtype=np.complex128)
    for n in range(1, R):
        s = np.exp(logNormD[n] + logNormU[n] - logLike)
        if branch_mask is not None:
            s = np.where(np.asarray(branch_mask)[n], s, 0.0)
        out += np.einsum('ck,kl,cl->klc', D_tilde[n] * s[:, None], J[n], U_tilde[n])
    return out


def accumulate_C_complex_per_branch(D_tilde, U_tilde, J, logNormU, logNormD, logLike, parentIndex,
                                    branch_mask=None):
    """Per-branch complex C (R, A, A, C), branch 0 zero; oracle.py:606-639."""
    R, C, A = U_tilde.shape
    out = np.zeros((R, A, A, C), dtype=np.complex128)
    for n in range(1, R):
        s = np.exp(logNormD[n] + logNormU[n] - logLike)
        if branch_mask is not None:
            s = np.where(np.asarray(branch_mask)[n], s, 0.0)
        out[n] = np.einsum('ck,kl,cl->klc', D_tilde[n] * s[:, None], J[n], U_tilde[n])
    return out


def _rate_irrev(model):
    V = np.asarray(model['eigenvectors'], dtype=np.complex128)
    Vi = np.asarray(model['eigenvectors_inv'], dtype=np.complex128)
    mu = np.asarray(model['eigenvalues'], dtype=np.complex128)
    if model.get('_exact'):
        # rate matrix of the original model; the vectors are swapped below
        V0, Vi0 = Vi.T, V.T
        return V, Vi, (V0 * mu[None, :]) @ Vi0
    return V, Vi, (V * mu[None, :]) @ Vi


def irrev_exact_model(model):
    """The model dict whose reference-formula counts are the expected counts
    of M(t) = e^{Qt} itself: (V, Vinv) replaced by (Vinv^T, V^T), so that
    D~ = D V, U~ = Vinv U and the back-transform is Vinv^T C V^T, with the
    off-diagonal factor still Q.  (For non-reversible Q the reference's
    formula, oracle.py:537-693, gives the counts of the transposed process;
    tests/test_irrev_math.py checks both against quadrature.)"""
    m = dict(model)
    m['eigenvectors'] = np.asarray(model['eigenvectors_inv'], dtype=np.complex128).T
    m['eigenvectors_inv'] = np.asarray(model['eigenvectors'], dtype=np.complex128).T
    m['_exact'] = True
    m['reversible'] = False
    return m


def back_transform_irrev(Ceig, model):
    """Re of V C Vinv on the diagonal, of R_ij (V C Vinv)_ij off it, with
    R = V diag(mu) Vinv; oracle.py:642-693."""
    V, Vi, Rm = _rate_irrev(model)
    VCV = np.einsum('ik,klc,lj->ijc', V, Ceig, Vi)
    A = V.shape[0]
    eye = np.eye(A, dtype=bool)[:, :, None]
    return np.where(eye, VCV, Rm[:, :, None] * VCV).real


def back_transform_irrev_per_branch(Ceig, model):
    """oracle.py:696-740."""
    V, Vi, Rm = _rate_irrev(model)
    VCV = np.einsum('ik,nklc,lj->nijc', V, Ceig, Vi)
    A = V.shape[0]
    eye = np.eye(A, dtype=bool)[None, :, :, None]
    return np.where(eye, VCV, Rm[None, :, :, None] * VCV).real


# ---------------------------------------------------------------------------
# Substitution matrices, inside and outside — oracle.py:747-924
# ---------------------------------------------------------------------------

def compute_sub_matrices(model, distances):
    """M_ij(t) = sqrt(pi_j/pi_i) sum_k V_ik e^{mu_k t} V_jk; oracle.py:747-777."""
    V = np.asarray(model['eigenvectors'], dtype=np.float64)
    mu = np.asarray(model['eigenvalues'], dtype=np.float64)
    pi = np.asarray(model['pi'], dtype=np.float64)
    d = np.asarray(distances, dtype=np.float64)
    E = np.exp(mu[None, :] * d[:, None])                  # (R, A)
    S = np.einsum('ik,rk,jk->rij', V, E, V)
    sp = np.sqrt(pi)
    return S * (1.0 / sp)[None, :, None] * sp[None, None, :]


def upward_pass(alignment, tree, subMatrices, rootProb):
    """Inside pass with per-child max rescaling; oracle.py:784-838.

    Returns U (R,C,A), logNormU (R,C), logLike (C,).
    """
    parentIndex = tree.parentIndex
    alignment = np.asarray(alignment)
    R, C = alignment.shape
    A = subMatrices.shape[-1]
    U = token_to_likelihood(alignment, A)
    logNormU = np.zeros((R, C))
    for n in range(R - 1, 0, -1):                           # oracle.py:806
        p = parentIndex[n]
        contrib = U[n] @ subMatrices[n].T                   # sum_j M_bj U_j
        U[p] *= contrib
        mx = np.max(U[p], axis=-1)
        mx = np.where(mx < RESCALE_FLOOR, RESCALE_FLOOR, mx)
        U[p] /= mx[:, None]
        logNormU[p] += logNormU[n] + np.log(mx)
    with np.errstate(divide='ignore'):
        logLike = logNormU[0] + np.log(U[0] @ np.asarray(rootProb))   # oracle.py:831-836
    return U, logNormU, logLike


def downward_pass(U, logNormU, tree, subMatrices, rootProb, alignment):
    """Outside pass; oracle.py:845-924.  D[root] stays 0."""
    parentIndex = tree.parentIndex
    R, C, A = U.shape
    _, _, sibling = children_of(parentIndex)
    obs = token_to_likelihood(alignment, A)
    rootProb = np.asarray(rootProb)
    D = np.zeros((R, C, A))
    logNormD = np.zeros((R, C))
    for n in range(1, R):                                   # oracle.py:869
        p = parentIndex[n]
        sib = sibling[n]
        sib_contrib = U[sib] @ subMatrices[sib].T           # sum_j M_sib[a,j] U_sib[j]
        if p == 0:
            par = np.broadcast_to(rootProb, (C, A)).copy()
            prior = 0.0
        else:
            par = D[p] @ subMatrices[p]                     # sum_i D_p[i] M_p[i,a]
            prior = logNormD[p]
        par = par * obs[p]
        raw = sib_contrib * par
        mx = np.max(raw, axis=-1)
        mx = np.where(mx < RESCALE_FLOOR, RESCALE_FLOOR, mx)
        D[n] = raw / mx[:, None]
        logNormD[n] = logNormU[sib] + prior + np.log(mx)
    return D, logNormD


# ---------------------------------------------------------------------------
# Eigenbasis counts — oracle.py:931-1137
# ---------------------------------------------------------------------------

def compute_J(eigenvalues, distances):
    """J^{kl}(t) divided differences, 1e-8 degeneracy test; oracle.py:931-959."""
    mu = np.asarray(eigenvalues, dtype=np.float64)
    t = np.asarray(distances, dtype=np.float64)
    E = np.exp(mu[None, :] * t[:, None])                    # (R, A)
    diff = mu[:, None] - mu[None, :]
    deg = np.abs(diff) < DEGENERATE_THRESHOLD
    safe = np.where(deg, 1.0, diff)
    J = (E[:, :, None] - E[:, None, :]) / safe[None]
    Jdeg = t[:, None, None] * E[:, :, None] * np.ones_like(diff)[None]
    return np.where(deg[None], Jdeg, J)


def eigenbasis_project(U, D, model):
    """U~ = (U*sqrt(pi)) V, D~ = (D/sqrt(pi)) V; oracle.py:966-1003."""
    V = np.asarray(model['eigenvectors'], dtype=np.float64)
    sp = np.sqrt(np.asarray(model['pi'], dtype=np.float64))
    return (U * sp) @ V, (D / sp) @ V


def accumulate_C(D_tilde, U_tilde, J, logNormU, logNormD, logLike, parentIndex,
                 branch_mask=None):
    """C_kl,c = sum_{n>0} D~_k J_kl U~_l exp(lnD+lnU-lnL); oracle.py:1010-1044."""
    R, C, A = U_tilde.shape
    out = np.zeros((A, A, C))
    for n in range(1, R):
        s = np.exp(logNormD[n] + logNormU[n] - logLike)
        if branch_mask is not None:
            s = np.where(np.asarray(branch_mask)[n], s, 0.0)
        out += np.einsum('ck,kl,cl->klc', D_tilde[n] * s[:, None], J[n], U_tilde[n])
    return out


def back_transform(Ceig, model):
    """counts = V C V^T on the diagonal, S*(V C V^T) off it; oracle.py:1087-1137."""
    V = np.asarray(model['eigenvectors'], dtype=np.float64)
    mu = np.asarray(model['eigenvalues'], dtype=np.float64)
    S = (V * mu[None, :]) @ V.T
    VCV = np.einsum('ik,klc,jl->ijc', V, Ceig, V)
    A = V.shape[0]
    eye = np.eye(A, dtype=bool)[:, :, None]
    return np.where(eye, VCV, S[:, :, None] * VCV)


def f81_counts(U, D, logNormU, logNormD, logLike, distances, pi, parentIndex,
               branch_mask=None):
    """Closed-form F81/JC counts; oracle.py:1190-1256 (mu from pi, not eigenvalues)."""
    R, C, A = U.shape
    pi = np.asarray(pi, dtype=np.float64)
    mu = 1.0 / (1.0 - np.sum(pi ** 2))
    out = np.zeros((A, A, C))
    offdiag = ~np.eye(A, dtype=bool)
    for n in range(1, R):
        t = distances[n]
        e = np.exp(-mu * t)
        p = 1.0 - e
        alpha = t * e
        beta = p / mu - t * e
        gamma = t * (1.0 + e) - 2.0 * p / mu
        s = np.exp(logNormD[n] + logNormU[n] - logLike)
        if branch_mask is not None:
            s = np.where(np.asarray(branch_mask)[n], s, 0.0)
        Ds = D[n] * s[:, None]                              # (C, A)
        piU = U[n] @ pi                                     # (C,)
        Dsum = Ds.sum(-1)                                   # (C,)
        I = (alpha * np.einsum('ci,cj->ijc', Ds, U[n])
             + beta * (np.einsum('ci,c->ic', Ds, piU)[:, None, :]
                       + np.einsum('i,c,cj->ijc', pi, Dsum, U[n]))
             + gamma * np.einsum('i,c->ic', pi, Dsum * piU)[:, None, :])
        out += np.where(offdiag[:, :, None], mu * pi[None, :, None] * I, I)
    return out


def accumulate_C_per_branch(D_tilde, U_tilde, J, logNormU, logNormD, logLike, parentIndex,
                            branch_mask=None):
    """Per-branch eigenbasis counts (R, A, A, C), branch 0 zero; oracle.py:1047-1084."""
    R, C, A = U_tilde.shape
    out = np.zeros((R, A, A, C))
    for n in range(1, R):
        s = np.exp(logNormD[n] + logNormU[n] - logLike)
        if branch_mask is not None:
            s = np.where(np.asarray(branch_mask)[n], s, 0.0)
        out[n] = np.einsum('ck,kl,cl->klc', D_tilde[n] * s[:, None], J[n], U_tilde[n])
    return out


def back_transform_per_branch(Ceig, model):
    """V C_n V^T per branch: dwell on the diagonal, S * VCV off it; oracle.py:1140-1183."""
    V = np.asarray(model['eigenvectors'], dtype=np.float64)
    mu = np.asarray(model['eigenvalues'], dtype=np.float64)
    S = (V * mu[None, :]) @ V.T
    VCV = np.einsum('ik,nklc,jl->nijc', V, Ceig, V)
    A = V.shape[0]
    eye = np.eye(A, dtype=bool)[None, :, :, None]
    return np.where(eye, VCV, S[None, :, :, None] * VCV)


def f81_counts_per_branch(U, D, logNormU, logNormD, logLike, distances, pi, parentIndex,
                          branch_mask=None):
    """Closed-form F81/JC counts per branch (R, A, A, C); oracle.py:1259-1331."""
    R, C, A = U.shape
    pi = np.asarray(pi, dtype=np.float64)
    mu = 1.0 / (1.0 - np.sum(pi ** 2))
    out = np.zeros((R, A, A, C))
    offdiag = ~np.eye(A, dtype=bool)
    for n in range(1, R):
        t = distances[n]
        e = np.exp(-mu * t)
        p = 1.0 - e
        alpha = t * e
        beta = p / mu - t * e
        gamma = t * (1.0 + e) - 2.0 * p / mu
        s = np.exp(logNormD[n] + logNormU[n] - logLike)
        if branch_mask is not None:
            s = np.where(np.asarray(branch_mask)[n], s, 0.0)
        Ds = D[n] * s[:, None]
        piU = U[n] @ pi
        Dsum = Ds.sum(-1)
        I = (alpha * np.einsum('ci,cj->ijc', Ds, U[n])
             + beta * (np.einsum('ci,c->ic', Ds, piU)[:, None, :]
                       + np.einsum('i,c,cj->ijc', pi, Dsum, U[n]))
             + gamma * np.einsum('i,c->ic', pi, Dsum * piU)[:, None, :])
        out[n] = np.where(offdiag[:, :, None], mu * pi[None, :, None] * I, I)
    return out


def compute_branch_mask(alignment, parentIndex, A):
    """Steiner-tree branch mask of ungapped leaves; oracle.py:1372-1435.

    Token 0..A counts as ungapped; only leaves can be ungapped; root False.
    """
    alignment = np.asarray(alignment)
    parentIndex = np.asarray(parentIndex)
    R, C = alignment.shape
    cnt = np.zeros(R, dtype=np.int64)
    for n in range(1, R):
        cnt[parentIndex[n]] += 1
    is_leaf = cnt == 0
    ung_leaf = is_leaf[:, None] & (alignment >= 0) & (alignment <= A)
    has = ung_leaf.copy()
    for n in range(R - 1, 0, -1):
        has[parentIndex[n]] |= has[n]
    ucc = np.zeros((R, C), dtype=np.int64)
    for n in range(1, R):
        ucc[parentIndex[n]] += has[n]
    st = ung_leaf | (ucc >= 2)
    for n in range(1, R):
        st[n] |= st[parentIndex[n]] & has[n]
    mask = np.zeros((R, C), dtype=bool)
    for n in range(1, R):
        mask[n] = st[n] & st[parentIndex[n]]
    return mask


# ---------------------------------------------------------------------------
# Public API — oracle.py:1454-1595
# ---------------------------------------------------------------------------

def LogLike(alignment, tree, model):
    """Per-column log-likelihood (C,); oracle.py:1454-1467."""
    M = _sub_matrices(model, tree.distanceToParent)
    return upward_pass(alignment, tree, M, model['pi'])[2]


def Counts(alignment, tree, model, f81_fast=False, branch_mask="auto", irrev_exact=False):
    """(A, A, C) dwell (diag) + substitution (off-diag) counts; oracle.py:1470-1514."""
    A = len(model['pi'])
    if isinstance(branch_mask, str) and branch_mask == "auto":
        branch_mask = compute_branch_mask(alignment, tree.parentIndex, A)
    if is_irrev(model) and f81_fast:
        raise ValueError("the F81 fast path is reversible-only")
    M = _sub_matrices(model, tree.distanceToParent)
    U, lnU, lnL = upward_pass(alignment, tree, M, model['pi'])
    D, lnD = downward_pass(U, lnU, tree, M, model['pi'], alignment)
    if f81_fast:
        return f81_counts(U, D, lnU, lnD, lnL, tree.distanceToParent, model['pi'],
                          tree.parentIndex, branch_mask=branch_mask)
    if is_irrev(model):
        mp = irrev_exact_model(model) if irrev_exact else model
        J = compute_J_complex(model['eigenvalues'], tree.distanceToParent)
        Ut, Dt = eigenbasis_project_irrev(U, D, mp)
        return back_transform_irrev(
            accumulate_C_complex(Dt, Ut, J, lnU, lnD, lnL, tree.parentIndex, branch_mask=branch_mask), mp)
    J = compute_J(model['eigenvalues'], tree.distanceToParent)
    Ut, Dt = eigenbasis_project(U, D, model)
    Ceig = accumulate_C(Dt, Ut, J, lnU, lnD, lnL, tree.parentIndex, branch_mask=branch_mask)
    return back_transform(Ceig, model)


def BranchCounts(alignment, tree, model, f81_fast=False, branch_mask=None, irrev_exact=False):
    """(R, A, A, C) per-branch dwell/substitution counts, branch 0 zero;
    oracle.py:1517-1568.  The default mask is None, as in subby.jax.BranchCounts
    (subby/jax/__init__.py:450-540), which does not mask."""
    A = len(model['pi'])
    if isinstance(branch_mask, str) and branch_mask == "auto":
        branch_mask = compute_branch_mask(alignment, tree.parentIndex, A)
    if is_irrev(model) and f81_fast:
        raise ValueError("the F81 fast path is reversible-only")
    M = _sub_matrices(model, tree.distanceToParent)
    U, lnU, lnL = upward_pass(alignment, tree, M, model['pi'])
    D, lnD = downward_pass(U, lnU, tree, M, model['pi'], alignment)
    if f81_fast:
        return f81_counts_per_branch(U, D, lnU, lnD, lnL, tree.distanceToParent, model['pi'],
                                     tree.parentIndex, branch_mask=branch_mask)
    if is_irrev(model):
        mp = irrev_exact_model(model) if irrev_exact else model
        J = compute_J_complex(model['eigenvalues'], tree.distanceToParent)
        Ut, Dt = eigenbasis_project_irrev(U, D, mp)
        return back_transform_irrev_per_branch(
            accumulate_C_complex_per_branch(Dt, Ut, J, lnU, lnD, lnL, tree.parentIndex,
                                            branch_mask=branch_mask), mp)
    J = compute_J(model['eigenvalues'], tree.distanceToParent)
    Ut, Dt = eigenbasis_project(U, D, model)
    return back_transform_per_branch(
        accumulate_C_per_branch(Dt, Ut, J, lnU, lnD, lnL, tree.parentIndex, branch_mask=branch_mask), model)


def RootProb(alignment, tree, model):
    """(A, C) root posterior pi_a U_root,a e^{lnU_root - lnL}; oracle.py:1571-1595."""
    M = _sub_matrices(model, tree.distanceToParent)
    U, lnU, lnL = upward_pass(alignment, tree, M, model['pi'])
    scale = np.exp(lnU[0] - lnL)
    return (np.asarray(model['pi'])[None, :] * U[0] * scale[:, None]).T


def _sub_matrices(model, distances):
    """oracle.py:1447-1451: the irreversible M(t) for irreversible models."""
    if is_irrev(model):
        return compute_sub_matrices_irrev(model, distances)
    return compute_sub_matrices(model, distances)


def _inside_outside(alignment, tree, model, root_prob=None):
    """U, D, scales and M with the root's outside vector set to pi / max(pi),
    as InsideOutside.__init__ does (oracle.py:1631-1661).  ``root_prob``
    replaces the model's pi at the root (subby/jax/__init__.py:721-731: a
    per-column model list takes the first model's pi for every column)."""
    M = _sub_matrices(model, tree.distanceToParent)
    rp = model['pi'] if root_prob is None else root_prob
    U, lnU, lnL = upward_pass(alignment, tree, M, rp)
    D, lnD = downward_pass(U, lnU, tree, M, rp, alignment)
    pi = np.asarray(rp, dtype=np.float64)
    mx = max(float(np.max(pi)), RESCALE_FLOOR)
    D[0] = pi[None, :] / mx
    lnD[0] = np.log(mx)
    return M, U, lnU, lnL, D, lnD


def _normalise(x, axes):
    """Divide by the sum over `axes` where that sum is positive (oracle.py:1793-1795)."""
    tot = np.sum(x, axis=axes, keepdims=True)
    return np.where(tot > 0, x / np.where(tot > 0, tot, 1.0), x)


def NodePosterior(alignment, tree, model, node=None, root_prob=None):
    """Posterior state distribution of node(s); InsideOutside.node_posterior,
    oracle.py:1755-1831 (subby/jax/__init__.py:868-946).

    Root: pi_a U_0a; node n > 0: (sum_a D_na M_n[a, j]) U_nj; times
    exp(logNormU + logNormD - logLike), normalised over the states.
    Returns (A, C) for one node, (R, A, C) for node=None."""
    M, U, lnU, lnL, D, lnD = _inside_outside(alignment, tree, model, root_prob)
    scale = np.exp(lnU + lnD - lnL[None, :])                       # (R, C)
    Dt = np.einsum('rca,raj->rcj', D, M)
    Dt[0] = D[0]
    post = _normalise(Dt * U * scale[:, :, None], -1)              # (R, C, A)
    post = post.transpose(0, 2, 1)
    return post if node is None else post[node]


def BranchPosterior(alignment, tree, model, node=None, root_prob=None):
    """Joint posterior of (parent state i, child state j) on branch(es);
    InsideOutside.branch_posterior, oracle.py:1833-1905
    (subby/jax/__init__.py:948-1040): D_ni M_n[i, j] U_nj exp(logNormD +
    logNormU - logLike), normalised over (i, j).  Returns (A, A, C) for one
    node (> 0), (R, A, A, C) with branch 0 zero for node=None."""
    M, U, lnU, lnL, D, lnD = _inside_outside(alignment, tree, model, root_prob)
    scale = np.exp(lnU + lnD - lnL[None, :])
    joint = D[:, :, :, None] * M[:, None, :, :] * U[:, :, None, :] * scale[:, :, None, None]  # (R, C, A, A)
    joint = _normalise(joint, (-2, -1))
    joint = joint.transpose(0, 2, 3, 1)
    if node is not None:
        return joint[node]
    joint[0] = 0.0
    return joint


def pipeline(alignment, tree, model, branch_mask=None, f81_fast=False):
    """Every intermediate of one Counts call, for fixture comparison."""
    M = compute_sub_matrices(model, tree.distanceToParent)
    U, lnU, lnL = upward_pass(alignment, tree, M, model['pi'])
    D, lnD = downward_pass(U, lnU, tree, M, model['pi'], alignment)
    out = dict(sub_matrices=M, U=U, logNormU=lnU, logLike=lnL, D=D, logNormD=lnD)
    if f81_fast:
        out['counts'] = f81_counts(U, D, lnU, lnD, lnL, tree.distanceToParent,
                                   model['pi'], tree.parentIndex, branch_mask=branch_mask)
    else:
        J = compute_J(model['eigenvalues'], tree.distanceToParent)
        Ut, Dt = eigenbasis_project(U, D, model)
        Ceig = accumulate_C(Dt, Ut, J, lnU, lnD, lnL, tree.parentIndex, branch_mask=branch_mask)
        out.update(J=J, U_tilde=Ut, D_tilde=Dt, C_eigen=Ceig, counts=back_transform(Ceig, model))
    return out


# ---------------------------------------------------------------------------
# Gradients (FP64) — subby/jax/vjp.py:62-133 (distance gradient)
# ---------------------------------------------------------------------------

def loglike_distance_grad(alignment, tree, model, g=None):
    """d(sum_c g_c logL_c)/d t_n by the Fisher identity of subby/jax/vjp.py:92-124.

    dlogL_c/dt_n = sum_k D~_k mu_k e^{mu_k t_n} U~_k exp(lnD+lnU-lnL); root 0.
    Irreversible models (vjp.py:80-90): D~ = D V, U~ = V^-1 U, real part.
    """
    M = _sub_matrices(model, tree.distanceToParent)
    U, lnU, lnL = upward_pass(alignment, tree, M, model['pi'])
    D, lnD = downward_pass(U, lnU, tree, M, model['pi'], alignment)
    if is_irrev(model):
        Dt = D @ np.asarray(model['eigenvectors'], dtype=np.complex128)
        Ut = U @ np.asarray(model['eigenvectors_inv'], dtype=np.complex128).T
    else:
        Ut, Dt = eigenbasis_project(U, D, model)
    mu = np.asarray(model['eigenvalues'])
    t = tree.distanceToParent
    C = lnL.shape[0]
    g = np.ones(C) if g is None else np.asarray(g, dtype=np.float64)
    R = len(t)
    grad = np.zeros(R)
    for n in range(1, R):
        me = mu * np.exp(mu * t[n])
        s = np.exp(lnD[n] + lnU[n] - lnL)
        grad[n] = np.sum(g * s * np.einsum('ck,k,ck->c', Dt[n], me, Ut[n]).real)
    return grad


def reversible_rate_matrix(log_exch, pi):
    """Q from log-exchangeabilities (upper triangle, row-major i<j) and pi,
    normalised to one expected substitution per unit time."""
    pi = np.asarray(pi, dtype=np.float64)
    A = len(pi)
    s = np.zeros((A, A))
    iu = np.triu_indices(A, 1)
    s[iu] = np.exp(np.asarray(log_exch, dtype=np.float64))
    s = s + s.T
    Q = s * pi[None, :]
    np.fill_diagonal(Q, 0.0)
    rate = np.sum(pi * Q.sum(1))
    Q = Q / rate
    np.fill_diagonal(Q, -Q.sum(1))
    return Q


def _fd_total(args):
    """sum_c logL_c of the reversible model (log_exch, pi) on (parent, dist)."""
    alignment, parent, dist, le, pi = args
    model = diagonalize_rate_matrix(reversible_rate_matrix(le, pi), pi)
    return float(np.sum(LogLike(alignment, Tree(parent, dist), model)))


def loglike_fd_grad(alignment, tree, log_exch, pi, h=1e-4, wrt="distances", idx=None, pool=None):
    """Central finite differences (FP64) of sum_c logL_c, for adjoint checks.

    ``idx``: the components to difference (default all; the others stay 0);
    ``pool``: a multiprocessing pool (spawn context) that evaluates the
    perturbed likelihoods in parallel.
    """
    dist = np.array(tree.distanceToParent, dtype=np.float64)
    le = np.array(log_exch, dtype=np.float64)
    parent = np.asarray(tree.parentIndex)
    base = dist if wrt == "distances" else le
    if idx is None:
        idx = range(1, len(dist)) if wrt == "distances" else range(len(le))
    idx = list(idx)
    work = []
    for i in idx:
        for sgn in (1.0, -1.0):
            x = base.copy()
            x[i] += sgn * h
            work.append((alignment, parent, x, le, pi) if wrt == "distances" else (alignment, parent, dist, x, pi))
    vals = pool.map(_fd_total, work) if pool is not None else list(map(_fd_total, work))
    g = np.zeros(len(base))
    for j, i in enumerate(idx):
        g[i] = (vals[2 * j] - vals[2 * j + 1]) / (2 * h)
    return g


# ---------------------------------------------------------------------------
# Batched models — rate categories, mixtures, per-column model lists
# ---------------------------------------------------------------------------

def gamma_rate_categories(alpha, K):
    """Yang (1994) discrete gamma: quantile medians by 64 bisection steps,
    mean-normalised rates, uniform weights; oracle.py:208-241."""
    from scipy.special import gammainc
    mids = 0.5 * (np.linspace(0, 1, K + 1)[:-1] + np.linspace(0, 1, K + 1)[1:])
    rates = np.zeros(K)
    for i, p in enumerate(mids):
        lo, hi = 0.0, max(50.0, 10.0 / alpha)
        for _ in range(64):
            mid = 0.5 * (lo + hi)
            if float(gammainc(alpha, mid * alpha)) < p:
                lo = mid
            else:
                hi = mid
        rates[i] = 0.5 * (lo + hi)
    return rates * K / np.sum(rates), np.ones(K) / K


def scale_model(model, rate_multiplier):
    """Eigenvalues times the rate; oracle.py:244-262."""
    m = dict(model)
    m['eigenvalues'] = np.asarray(model['eigenvalues']) * rate_multiplier
    return m


def mixture_posterior(log_likes, log_weights):
    """softmax_k(log_likes[k, c] + log_weights[k]); oracle.py:1334-1365."""
    lj = np.asarray(log_likes, dtype=np.float64) + np.asarray(log_weights, dtype=np.float64)[:, None]
    lj = lj - np.max(lj, axis=0, keepdims=True)
    e = np.exp(lj)
    return e / np.sum(e, axis=0, keepdims=True)


def MixturePosterior(alignment, tree, models, log_weights):
    """(K, C) posterior over mixture components; oracle.py:1598-1615."""
    return mixture_posterior(np.stack([LogLike(alignment, tree, m) for m in models]), log_weights)


def LogLike_per_column(alignment, tree, models):
    """Per-column models (subby/jax/__init__.py:267-277): column c uses
    models[c]'s M(t); the root prior is models[0]'s pi for every column."""
    alignment = np.asarray(alignment)
    out = np.zeros(alignment.shape[1])
    for c in range(alignment.shape[1]):
        M = _sub_matrices(models[c], tree.distanceToParent)
        out[c] = upward_pass(alignment[:, c:c + 1], tree, M, models[0]['pi'])[2][0]
    return out


def RootProb_per_column(alignment, tree, models):
    """subby/jax/__init__.py:617-633: pi_c * U_root e^{lnU - lnL}, with lnL
    from the root prior models[0]['pi'] (columns need not sum to one when
    the pis differ)."""
    alignment = np.asarray(alignment)
    A = len(models[0]['pi'])
    out = np.zeros((A, alignment.shape[1]))
    for c in range(alignment.shape[1]):
        M = _sub_matrices(models[c], tree.distanceToParent)
        U, lnU, lnL = upward_pass(alignment[:, c:c + 1], tree, M, models[0]['pi'])
        out[:, c] = np.asarray(models[c]['pi']) * U[0, 0] * np.exp(lnU[0, 0] - lnL[0])
    return out


def Counts_per_column(alignment, tree, models, f81_fast=False, branch_mask="auto"):
    """subby/jax/__init__.py:396-411: column by column with its own model."""
    alignment = np.asarray(alignment)
    cols = []
    for c in range(alignment.shape[1]):
        bm = branch_mask if (branch_mask is None or isinstance(branch_mask, str)) else \
            np.asarray(branch_mask)[:, c:c + 1]
        cols.append(Counts(alignment[:, c:c + 1], tree, models[c], f81_fast=f81_fast, branch_mask=bm))
    return np.concatenate(cols, axis=-1)


def _rows_sub_matrices(models_row, distances):
    """M_n from node n's own model (subby/jax/__init__.py:74-101)."""
    d = np.asarray(distances, dtype=np.float64)
    return np.stack([_sub_matrices(models_row[n], d[n:n + 1])[0] for n in range(len(d))])


def LogLike_rows(alignment, tree, models_row):
    """Per-branch models, the (1, R) model grid (subby/jax/__init__.py:
    230-244): root prior models_row[0]['pi']."""
    M = _rows_sub_matrices(models_row, tree.distanceToParent)
    return upward_pass(alignment, tree, M, models_row[0]['pi'])[2]


def RootProb_rows(alignment, tree, models_row):
    M = _rows_sub_matrices(models_row, tree.distanceToParent)
    pi0 = np.asarray(models_row[0]['pi'])
    U, lnU, lnL = upward_pass(alignment, tree, M, pi0)
    return (pi0[None, :] * U[0] * np.exp(lnU[0] - lnL)[:, None]).T


def BranchCounts_rows(alignment, tree, models_row):
    """Per-branch counts, each branch in its own model's eigenbasis, unmasked
    (subby/jax/__init__.py:104-152)."""
    M = _rows_sub_matrices(models_row, tree.distanceToParent)
    U, lnU, lnL = upward_pass(alignment, tree, M, models_row[0]['pi'])
    D, lnD = downward_pass(U, lnU, tree, M, models_row[0]['pi'], alignment)
    R, C, A = U.shape
    out = np.zeros((R, A, A, C))
    d = tree.distanceToParent
    for n in range(1, R):
        m = models_row[n]
        J = compute_J(m['eigenvalues'], d[n:n + 1])[0]
        Ut, Dt = eigenbasis_project(U[n], D[n], m)
        s = np.exp(lnD[n] + lnU[n] - lnL)
        Cn = np.einsum('ck,kl,cl->klc', Dt * s[:, None], J, Ut)
        out[n] = back_transform(Cn, m)
    return out


def Counts_rows(alignment, tree, models_row, branch_mask="auto"):
    """Per-branch counts times the mask, summed (subby/jax/__init__.py:
    356-369)."""
    bc = BranchCounts_rows(alignment, tree, models_row)
    A = bc.shape[1]
    if isinstance(branch_mask, str) and branch_mask == "auto":
        branch_mask = compute_branch_mask(alignment, tree.parentIndex, A)
    if branch_mask is not None:
        bc = bc * np.asarray(branch_mask)[:, None, None, :]
    return bc.sum(0)
