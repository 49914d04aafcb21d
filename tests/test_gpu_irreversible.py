"""Irreversible (complex eigensystem) models through every entry point vs
the FP64 oracle's restatement of subby/oracle/oracle.py:474-740 and the
reference oracle's fixtures (irrev_4, irrev_8, irrev_16).

Tolerances as for reversible models (tests/_tol.py): LogLike 1e-5 relative,
RootProb / posteriors 1e-4 column-wise norm-wise.  Counts: 1e-4 x max(1,
cond(V) / 10).  The counts are Re V C V^-1 with |C| a few hundred times the
counts when V is far from orthogonal, so the FP32 rounding of the inside /
outside vectors and of their projections is amplified by about cond(V)^2
(cyclic test models: cond(V) = 1.6 at A = 4, 8 at A = 16, 29 at A = 32, 59
at A = 64); the A = 64 back-transform itself runs in FP64."""
import numpy as np
import pytest

import oracle
from tests import _golden
from tests._tol import COUNTS_RTOL, POSTERIOR_RTOL, ROOTPROB_RTOL, assert_cols, assert_loglike

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import synth, models, _lib  # noqa: E402


def _per_branch(x):
    """(R, A, A, C) -> (A, A, R * C): every (branch, column) is a column."""
    x = np.asarray(x, np.float64)
    R, A, _, C = x.shape
    return x.transpose(1, 2, 0, 3).reshape(A, A, R * C)


def _nodes(x):
    x = np.asarray(x, np.float64)
    return np.moveaxis(x, 0, -2).reshape(*x.shape[1:-1], -1)


def _counts_tol(md):
    return COUNTS_RTOL * max(1.0, np.linalg.cond(md['eigenvectors']) / 10.0)


def _check_all(plan, aln, ot, md, what, branch=True):
    tol = _counts_tol(md)
    res = plan.run(aln, loglike=True, counts=True, rootprob=True)
    assert_loglike(res['logLike'], oracle.LogLike(aln, ot, md), what=what + " logLike")
    assert_cols(res['counts'], oracle.Counts(aln, ot, md), tol, what + " counts (auto mask)")
    assert_cols(res['rootProb'], oracle.RootProb(aln, ot, md), ROOTPROB_RTOL, what + " rootProb")
    c0 = plan.run(aln, loglike=False, counts=True, branch_mask=None)['counts']
    assert_cols(c0, oracle.Counts(aln, ot, md, branch_mask=None), tol, what + " counts (no mask)")
    cx = plan.run(aln, loglike=False, counts=True, exact_irreversible=True)['counts']
    assert_cols(cx, oracle.Counts(aln, ot, md, irrev_exact=True), tol, what + " counts (exact)")
    if branch:
        bc = plan.branch_counts(aln)
        assert_cols(_per_branch(bc), _per_branch(oracle.BranchCounts(aln, ot, md)), tol,
                    what + " branch counts")
        np.testing.assert_array_equal(bc[0], 0.0)
        bx = plan.branch_counts(aln, exact_irreversible=True)
        assert_cols(_per_branch(bx), _per_branch(oracle.BranchCounts(aln, ot, md, irrev_exact=True)), tol,
                    what + " branch counts (exact)")
    post = plan.posteriors(aln, want_node=True, want_branch=branch)
    assert_cols(_nodes(post['node']), _nodes(oracle.NodePosterior(aln, ot, md)), POSTERIOR_RTOL, what + " node post")
    if branch:
        assert_cols(_nodes(post['branch']), _nodes(oracle.BranchPosterior(aln, ot, md)), POSTERIOR_RTOL,
                    what + " branch post")


@pytest.mark.parametrize("name", [n for n in _golden.names() if n.startswith("irrev_")])
def test_golden_irreversible(name):
    g = _golden.load(name)
    m = sg.models.ensure_diag(_golden.model_dict(g))
    assert isinstance(m, sg.IrrevDiagModel)
    tree = sg.Tree(g['parentIndex'], g['distanceToParent'])
    plan = sg.Plan(tree, m)
    aln = g['alignment']
    res = plan.run(aln, loglike=True, counts=True, rootprob=True, branch_mask=None)
    assert_loglike(res['logLike'], g['logLike'], what=name)
    assert_cols(res['counts'], g['counts'], COUNTS_RTOL, name + " counts")
    assert_cols(res['rootProb'], g['root_prob'], ROOTPROB_RTOL, name + " rootProb")
    assert_cols(plan.run(aln, loglike=False, counts=True)['counts'], g['counts_masked'], COUNTS_RTOL,
                name + " counts masked")
    if 'branch_counts' in g:
        assert_cols(_per_branch(plan.branch_counts(aln)), _per_branch(g['branch_counts']), COUNTS_RTOL,
                    name + " branch counts")
    post = plan.posteriors(aln, want_node=True, want_branch=True)
    assert_cols(_nodes(post['node']), _nodes(g['node_posterior']), POSTERIOR_RTOL, name + " node post")
    assert_cols(_nodes(post['branch']), _nodes(g['branch_posterior']), POSTERIOR_RTOL, name + " branch post")
    plan.close()


@pytest.mark.parametrize("A,leaves,C", [(4, 16, 300), (8, 9, 80), (16, 9, 45), (20, 7, 33), (32, 6, 20),
                                        (64, 6, 40)])
def test_random_irreversible_vs_oracle(A, leaves, C):
    """Complex eigenvalue pairs (cyclic rate component); the walk with raw
    staging + the complex accumulation kernel; tensor-core walk at A = 64."""
    rng = np.random.default_rng(70 + A)
    m = models.random_irreversible(A, rng)
    assert np.any(np.abs(m.eigenvalues.imag) > 1e-3)
    tree = synth.random_tree(leaves, 0.15, rng)
    aln = synth.simulated_alignment(tree, m, C, 0.1, rng) if A <= 8 else \
        rng.integers(0, A + 2, size=(len(tree.parentIndex), C)).astype(np.int32)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    plan = sg.Plan(tree, m)
    _check_all(plan, aln, ot, m._asdict(), f"A={A}", branch=(A <= 32 or C <= 8))
    plan.close()


def test_given_mask_api_functions_and_errors():
    rng = np.random.default_rng(5)
    m = models.random_irreversible(4, rng)
    tree = synth.random_tree(10, 0.2, rng)
    R = len(tree.parentIndex)
    aln = synth.simulated_alignment(tree, m, 100, 0.1, rng)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    md = m._asdict()
    mask = rng.random((R, 100)) < 0.7
    assert_cols(sg.Counts(aln, tree, m, branch_mask=mask), oracle.Counts(aln, ot, md, branch_mask=mask),
                COUNTS_RTOL, "given mask")
    assert_loglike(sg.LogLike(aln, tree, m), oracle.LogLike(aln, ot, md))
    assert_cols(sg.RootProb(aln, tree, m), oracle.RootProb(aln, ot, md), ROOTPROB_RTOL, "RootProb")
    io = sg.InsideOutside(aln, tree, m)
    assert_cols(_nodes(io.node_posterior()), _nodes(oracle.NodePosterior(aln, ot, md)), POSTERIOR_RTOL, "io")
    # a dict with eigenvectors_inv is an irreversible model too
    d = dict(md, reversible=False)
    np.testing.assert_array_equal(sg.Counts(aln, tree, d), sg.Counts(aln, tree, m))
    with pytest.raises(_lib.SubbyError):
        sg.Counts(aln, tree, m, f81_fast_flag=True)
    plan = sg.Plan(tree, m)
    # device pointers give the host-pointer results
    dev = plan.run(torch.as_tensor(aln).cuda(), loglike=True, counts=True)
    host = plan.run(aln, loglike=True, counts=True)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev['counts'].cpu().numpy(), host['counts'])
    np.testing.assert_array_equal(dev['logLike'].cpu().numpy(), host['logLike'])
    plan.close()


def test_per_branch_fp64_back_transform_a64():
    """A = 64 per-branch counts: C buffered branch by branch and
    back-transformed in FP64."""
    rng = np.random.default_rng(99)
    m = models.random_irreversible(64, rng)
    tree = synth.random_tree(4, 0.15, rng)
    aln = rng.integers(0, 66, size=(len(tree.parentIndex), 9)).astype(np.int32)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    plan = sg.Plan(tree, m)
    bc = plan.branch_counts(aln)
    tol = _counts_tol(m._asdict())
    assert_cols(_per_branch(bc), _per_branch(oracle.BranchCounts(aln, ot, m._asdict())), tol, "A=64 per-branch")
    tot = plan.run(aln, loglike=False, counts=True, branch_mask=None)['counts']
    assert_cols(bc.astype(np.float64).sum(0), tot, tol, "A=64 branches sum to Counts")
    plan.close()


def test_reversible_model_as_irreversible_gives_the_same_counts():
    """A reversible model written as V = diag(pi)^-1/2 W, V^-1 = W^T diag(pi)^1/2
    (real eigenvalues) through the complex path with ``exact_irreversible``
    equals the reversible path (the reference's irreversible formula does
    not: it gives the transposed process's counts, tests/test_irrev_math.py)."""
    w = synth.plain_small(seed=2, C=200)
    aln, tree, m = w['alignment'], w['tree'], w['model']
    sp = np.sqrt(m.pi)
    V = m.eigenvectors / sp[:, None]
    Vi = m.eigenvectors.T * sp[None, :]
    mi = sg.IrrevDiagModel(m.eigenvalues.astype(np.complex128), V.astype(np.complex128),
                           Vi.astype(np.complex128), m.pi)
    a = sg.Plan(tree, m).run(aln, loglike=True, counts=True, rootprob=True)
    b = sg.Plan(tree, mi).run(aln, loglike=True, counts=True, rootprob=True, exact_irreversible=True)
    assert_loglike(b['logLike'], a['logLike'])
    assert_cols(b['counts'], a['counts'], COUNTS_RTOL, "counts")
    assert_cols(b['rootProb'], a['rootProb'], ROOTPROB_RTOL, "rootProb")


@pytest.mark.parametrize("A,leaves,C", [(4, 10, 200), (20, 6, 40), (64, 5, 30)])
def test_distance_gradient_vs_oracle(A, leaves, C):
    """d(sum g logL)/dt for irreversible models (subby/jax/vjp.py:62-133:
    D V and V^-1 U projections, real part): walk raw staging + the
    gradient kernel vs the oracle; through LogLikeCustomGrad with autograd."""
    rng = np.random.default_rng(90 + A)
    m = models.random_irreversible(A, rng)
    tree = synth.random_tree(leaves, 0.2, rng)
    aln = synth.simulated_alignment(tree, m, C, 0.1, rng)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    g = rng.uniform(0.5, 1.5, C)
    ref = oracle.loglike_distance_grad(aln, ot, m._asdict(), g=g)
    plan = sg.Plan(tree, m)
    ll, dldt, dldS = plan.grad(aln, g=g.astype(np.float32))
    plan.close()
    assert_loglike(ll, oracle.LogLike(aln, ot, m._asdict()))
    scale = max(np.abs(ref).max(), 1e-3)
    assert np.abs(dldt - ref).max() / scale <= 1e-4, (dldt, ref)
    assert dldt[0] == 0.0 and not np.any(dldS)
    d = torch.as_tensor(tree.distanceToParent.copy(), dtype=torch.float64).requires_grad_(True)
    out = sg.LogLikeCustomGrad(aln, sg.Tree(tree.parentIndex, d), m)
    (out * torch.as_tensor(g)).sum().backward()
    assert np.abs(d.grad.numpy() - ref).max() / scale <= 1e-4
