"""Alphabets run inside a larger kernel alphabet (subby_gb300/embed.py):
the embedded model, the token map and the output slicing, checked on the CPU
by running the embedded A2-state model through the FP64 oracle (as the inner
plan) and comparing with the oracle on the A-state model itself."""
import numpy as np
import pytest

import oracle
from subby_gb300 import embed, models, synth


class _OraclePlan:
    """Stand-in for the GPU plan: the FP64 oracle on the (embedded) model."""

    def __init__(self, tree, model, device=None):
        self.t = oracle.Tree(tree.parentIndex, tree.distanceToParent)
        self.m = model._asdict()
        self.R = len(tree.parentIndex)

    def run(self, aln, loglike=True, counts=False, rootprob=False, branch_mask="auto", bt64=None, stream=None,
            exact_irreversible=False):
        r = {}
        if loglike:
            r['logLike'] = oracle.LogLike(aln, self.t, self.m)
        if counts:
            r['counts'] = oracle.Counts(aln, self.t, self.m, branch_mask=branch_mask, irrev_exact=exact_irreversible)
        if rootprob:
            r['rootProb'] = oracle.RootProb(aln, self.t, self.m)
        return r

    def branch_counts(self, aln, branch_mask=None, stream=None, exact_irreversible=False):
        return oracle.BranchCounts(aln, self.t, self.m, branch_mask=branch_mask, irrev_exact=exact_irreversible)

    def posteriors(self, aln, node=None, want_node=True, want_branch=False, stream=None):
        r = {}
        if want_node:
            r['node'] = oracle.NodePosterior(aln, self.t, self.m, node=node)
        if want_branch:
            r['branch'] = oracle.BranchPosterior(aln, self.t, self.m, node=node)
        return r


def test_kernel_alphabet_and_token_map():
    assert [embed.kernel_alphabet(a) for a in (2, 8, 9, 16, 17, 21, 33, 61, 64, 65)] == \
        [2, 8, 16, 16, 20, 32, 64, 64, 64, None]
    t = np.array([[-1, -3, 0, 60, 61, 62, 63, 64, 99]], np.int32)
    assert embed.embed_tokens(t, 61, 64).tolist() == [[-1, -3, 0, 60, 64, 65, 65, 65, 65]]


@pytest.mark.parametrize("A,irrev", [(61, False), (13, True), (26, False)])
def test_embedded_plan_equals_the_model_itself(A, irrev):
    rng = np.random.default_rng(A)
    m = models.random_irreversible(A, rng) if irrev else models.random_reversible(A, rng)[0]
    tree = synth.random_tree(6, 0.2, rng)
    R = len(tree.parentIndex)
    aln = rng.integers(-1, A + 4, size=(R, 25)).astype(np.int32)
    aln[:, 0] = A + 1
    p = embed.EmbeddedPlan(tree, m, plan_cls=_OraclePlan)
    assert (p.A, p.A2) == (A, embed.kernel_alphabet(A))
    t, md = oracle.Tree(tree.parentIndex, tree.distanceToParent), m._asdict()
    r = p.run(aln, loglike=True, counts=True, rootprob=True, branch_mask=None)
    np.testing.assert_allclose(r['logLike'], oracle.LogLike(aln, t, md), rtol=1e-12, atol=1e-12)
    for mask in (None, "auto"):
        c = p.run(aln, loglike=False, counts=True, branch_mask=mask)['counts']
        assert c.shape == (A, A, 25)
        np.testing.assert_allclose(c, oracle.Counts(aln, t, md, branch_mask=mask), rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(r['rootProb'], oracle.RootProb(aln, t, md), rtol=1e-10, atol=1e-13)
    np.testing.assert_allclose(p.branch_counts(aln), oracle.BranchCounts(aln, t, md), rtol=1e-9, atol=1e-11)
    post = p.posteriors(aln, want_node=True, want_branch=True)
    np.testing.assert_allclose(post['node'], oracle.NodePosterior(aln, t, md), rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(post['branch'], oracle.BranchPosterior(aln, t, md), rtol=1e-9, atol=1e-12)
    one = p.posteriors(aln, node=2, want_node=True, want_branch=True)
    np.testing.assert_allclose(one['branch'], post['branch'][2], rtol=1e-12, atol=1e-15)
    out = {'counts': np.empty((A, A, 25)), 'logLike': np.empty(25)}
    r2 = p.run(aln, loglike=True, counts=True, out=out)
    assert r2['counts'] is out['counts'] and np.allclose(out['counts'], r2['counts'])
    with pytest.raises(NotImplementedError):
        p.run(aln, counts=True, f81=True)


def _counts_fp32(aln, tree, md):
    """The eigenbasis Counts algorithm (unmasked) with every array in FP32,
    the arithmetic of the FP32 kernels; back-transform in FP64."""
    f = np.float32
    mu, pi = np.asarray(md['eigenvalues'], np.float64), np.asarray(md['pi'], np.float64)
    M = oracle.compute_sub_matrices(md, tree.distanceToParent).astype(f)
    J = oracle.compute_J(mu, tree.distanceToParent).astype(f)
    R, C = aln.shape
    A = len(pi)
    L = oracle.token_to_likelihood(aln, A).astype(f)
    par = tree.parentIndex
    sib = oracle.children_of(par)[2]
    U, lnU = L.copy(), np.zeros((R, C), f)
    for n in range(R - 1, 0, -1):
        p = par[n]
        U[p] *= U[n] @ M[n].T
        mx = np.maximum(U[p].max(-1), f(1e-30))
        U[p] /= mx[:, None]
        lnU[p] += lnU[n] + np.log(mx)
    lnL = lnU[0] + np.log(U[0] @ pi.astype(f))
    D, lnD = np.zeros((R, C, A), f), np.zeros((R, C), f)
    for n in range(1, R):
        p, s = par[n], sib[n]
        pv = np.broadcast_to(pi.astype(f), (C, A)) if p == 0 else D[p] @ M[p]
        raw = (U[s] @ M[s].T) * pv * L[p]
        mx = np.maximum(raw.max(-1), f(1e-30))
        D[n] = raw / mx[:, None]
        lnD[n] = lnU[s] + (lnD[p] if p else 0) + np.log(mx)
    sp, V = np.sqrt(pi).astype(f), np.asarray(md['eigenvectors']).astype(f)
    Ut, Dt = (U * sp) @ V, (D / sp) @ V
    Cm = np.zeros((A, A, C), f)
    for n in range(1, R):
        Cm += np.einsum('ck,kl,cl,c->klc', Dt[n], J[n], Ut[n], np.exp(lnD[n] + lnU[n] - lnL))
    return oracle.back_transform(Cm.astype(np.float64), md)


def test_embedding_changes_nothing_in_fp32_arithmetic():
    """In FP32 arithmetic the embedded model's real-state counts equal the
    A-state model's up to summation order (the extra states meet the real
    ones only through exact zeros of the block-diagonal eigenvectors), so the
    GPU error of an embedded model is that of the A-state input itself.  The
    same input class is FP32-hard without embedding too: a random 61-state
    model (pi ~ Dirichlet(1)) with uniformly random tokens carries ~1e-4
    column-wise FP32 error against FP64 either way."""
    rng = np.random.default_rng(561)
    m = models.random_reversible(61, rng)[0]
    tree = synth.random_tree(5, 0.15, rng)
    t = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    aln = rng.integers(-1, 64, size=(len(tree.parentIndex), 12)).astype(np.int32)
    direct = _counts_fp32(aln, t, m._asdict())
    emb = _counts_fp32(embed.embed_tokens(aln, 61, 64), t, embed.embed_model(m, 64)._asdict())[:61, :61]
    np.testing.assert_allclose(emb, direct, rtol=1e-5, atol=1e-9)
    ref = oracle.Counts(aln, t, m._asdict(), branch_mask=None)
    scale = np.maximum(np.abs(ref).max(axis=(0, 1)), 1e-3)
    e_direct = (np.abs(direct - ref).max(axis=(0, 1)) / scale).max()
    e_emb = (np.abs(emb - ref).max(axis=(0, 1)) / scale).max()
    assert e_emb <= 1.01 * e_direct + 1e-7
