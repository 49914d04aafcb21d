"""Node and branch posteriors (subby_plan_posteriors, sg.InsideOutside) vs
the FP64 oracle's restatement of InsideOutside.node_posterior /
branch_posterior (subby/oracle/oracle.py:1755-1905), vs the reference
oracle's fixtures, and the identities the reference's tests check
(tests/test_api.py:971-1090 of ihh/subby): rows sum to one, the root row is
RootProb, a single node equals its slice of the all-node result, the
branch marginals are the parent's and the child's node posteriors.

Tolerance: per (node, column), max |d| / max(max |ref|, 1e-3) <= 1e-4 over
the states (node) or state pairs (branch)."""
import numpy as np
import pytest

import oracle
from tests import _golden
from tests._tol import POSTERIOR_RTOL, ROOTPROB_RTOL, assert_cols

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import synth, models, _lib  # noqa: E402


def _err(got, ref, floor=1e-3):
    """Worst (node, column) norm-wise error; states on the middle axes."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    R, C = ref.shape[0], ref.shape[-1]
    g = np.moveaxis(got, 0, -2).reshape(-1, R * C)
    r = np.moveaxis(ref, 0, -2).reshape(-1, R * C)
    num = np.max(np.abs(g - r), axis=0)
    den = np.maximum(np.max(np.abs(r), axis=0), floor)
    return float(np.max(num / den))


def _check(got, ref, what):
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    assert np.all(np.isfinite(got)), what
    e = _err(got, ref)
    assert e <= POSTERIOR_RTOL, f"{what}: posterior error {e:.2e} > {POSTERIOR_RTOL:.0e}"


def _model(g):
    return sg.models.ensure_diag(_golden.model_dict(g))


@pytest.mark.parametrize("name", [n for n in _golden.names() if 'node_posterior' in _golden.load(n)])
def test_golden_posteriors(name):
    g = _golden.load(name)
    tree = sg.Tree(g['parentIndex'], g['distanceToParent'])
    plan = sg.Plan(tree, _model(g))
    res = plan.posteriors(g['alignment'], want_node=True, want_branch=True)
    _check(res['node'], g['node_posterior'], name + " node")
    _check(res['branch'], g['branch_posterior'], name + " branch")
    np.testing.assert_array_equal(res['branch'][0], 0.0)
    plan.close()


def _identities(plan, aln, res, what):
    node, br = res['node'].astype(np.float64), res['branch'].astype(np.float64)
    R = node.shape[0]
    np.testing.assert_allclose(node.sum(1), 1.0, atol=1e-5, err_msg=what)
    np.testing.assert_allclose(br[1:].sum((1, 2)), 1.0, atol=1e-5, err_msg=what)
    assert node.min() >= -1e-6 and br.min() >= -1e-6, what
    root = plan.run(aln, loglike=False, rootprob=True)['rootProb']
    assert_cols(node[0], root, ROOTPROB_RTOL, what + " root = RootProb")
    parent = plan.parentIndex
    for n in range(1, R):
        assert_cols(br[n].sum(1), node[parent[n]], POSTERIOR_RTOL, f"{what} parent marginal n={n}")
        assert_cols(br[n].sum(0), node[n], POSTERIOR_RTOL, f"{what} child marginal n={n}")


def test_plain_workloads_vs_oracle_and_identities():
    for w in (synth.plain_small(seed=3, C=300), synth.plain_large(seed=4, C=257, f81=True)):
        aln, tree, m = w['alignment'], w['tree'], w['model']
        ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
        plan = sg.Plan(tree, m)
        res = plan.posteriors(aln, want_node=True, want_branch=True)
        _check(res['node'], oracle.NodePosterior(aln, ot, m._asdict()), "node")
        _check(res['branch'], oracle.BranchPosterior(aln, ot, m._asdict()), "branch")
        _identities(plan, aln, res, "plain")
        # one node: the slice of the all-node result (same kernels, same arithmetic)
        for n in (0, 1, 5, tree.parentIndex.shape[0] - 1):
            one = plan.posteriors(aln, node=n, want_node=True, want_branch=(n > 0))
            np.testing.assert_array_equal(one['node'], res['node'][n])
            if n > 0:
                np.testing.assert_array_equal(one['branch'], res['branch'][n])
        plan.close()


def test_a4_walk_route_matches_tree_kernel_route():
    """A = 4 posteriors come from the tree-program kernel; with it switched
    off (kernel selector 1) the walk + branch-posterior kernel serve them.
    Both match the oracle, eigen and F81 models, all nodes and one node."""
    for w in (synth.plain_small(seed=9, C=333), synth.plain_large(seed=10, C=200, f81=True)):
        aln, tree, m = w['alignment'], w['tree'], w['model']
        ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
        ref_n = oracle.NodePosterior(aln, ot, m._asdict())
        ref_b = oracle.BranchPosterior(aln, ot, m._asdict())
        plan = sg.Plan(tree, m)
        got = {}
        try:
            for sel in (0, 1):
                _lib.load().subby_debug_set_kernel(sel)
                got[sel] = plan.posteriors(aln, want_node=True, want_branch=True)
                one = plan.posteriors(aln, node=3, want_node=True, want_branch=True)
                np.testing.assert_array_equal(one['node'], got[sel]['node'][3])
                np.testing.assert_array_equal(one['branch'], got[sel]['branch'][3])
                root = plan.posteriors(aln, node=0)['node']
                np.testing.assert_array_equal(root, got[sel]['node'][0])
        finally:
            _lib.load().subby_debug_set_kernel(0)
        for sel in (0, 1):
            _check(got[sel]['node'], ref_n, f"selector {sel} node")
            _check(got[sel]['branch'], ref_b, f"selector {sel} branch")
        plan.close()


@pytest.mark.parametrize("A,leaves,C", [(8, 9, 70), (16, 9, 45), (20, 7, 33), (32, 5, 17), (64, 6, 140)])
def test_large_alphabets_vs_oracle(A, leaves, C):
    """The walk's raw staging at A = 8 .. 64 (tensor-core walk at A = 64), a
    general reversible model and an F81 model (closed-form walk products)."""
    rng = np.random.default_rng(40 + A)
    for m in (models.near_degenerate_reversible(A, rng)[0], models.f81_model(rng.dirichlet(np.ones(A)))):
        tree = synth.random_tree(leaves, 0.1, rng)
        aln = synth.simulated_alignment(tree, m, C, 0.1, rng)
        ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
        plan = sg.Plan(tree, m)
        res = plan.posteriors(aln, want_node=True, want_branch=True)
        md = sg.models.ensure_diag(m)._asdict()
        _check(res['node'], oracle.NodePosterior(aln, ot, md), f"A={A} node")
        _check(res['branch'], oracle.BranchPosterior(aln, ot, md), f"A={A} branch")
        _identities(plan, aln, res, f"A={A}")
        plan.close()


def test_device_pointers_and_inside_outside_api():
    w = synth.plain_small(seed=6, C=200)
    aln, tree, m = w['alignment'], w['tree'], w['model']
    plan = sg.Plan(tree, m)
    host = plan.posteriors(aln, want_node=True, want_branch=True)
    dev = plan.posteriors(torch.as_tensor(aln).cuda(), want_node=True, want_branch=True)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev['node'].cpu().numpy(), host['node'])
    np.testing.assert_array_equal(dev['branch'].cpu().numpy(), host['branch'])
    io = sg.InsideOutside(aln, tree, m)
    np.testing.assert_array_equal(io.node_posterior(), host['node'])
    np.testing.assert_array_equal(io.node_posterior(4), host['node'][4])
    np.testing.assert_array_equal(io.branch_posterior(), host['branch'])
    np.testing.assert_array_equal(io.branch_posterior(7), host['branch'][7])
    np.testing.assert_array_equal(io.log_likelihood, sg.LogLike(aln, tree, m))
    np.testing.assert_array_equal(io.counts(), sg.Counts(aln, tree, m))
    np.testing.assert_array_equal(io.branch_counts(), sg.BranchCounts(aln, tree, m))
    with pytest.raises(ValueError):
        io.branch_posterior(0)
    with pytest.raises(IndexError):
        plan.posteriors(aln, node=tree.parentIndex.shape[0])
    plan.close()


def test_unsupported_alphabet_raises():
    rng = np.random.default_rng(2)
    m = models.random_reversible(6, rng)[0]
    tree = synth.random_tree(6, 0.1, rng)
    aln = synth.simulated_alignment(tree, m, 8, 0.1, rng)
    plan = sg.Plan(tree, m)
    with pytest.raises(_lib.SubbyError):
        plan.posteriors(aln)
    plan.close()


@pytest.mark.parametrize("A,leaves,C", [(4, 14, 300), (16, 9, 160)])
def test_inside_outside_over_per_column_models_with_different_pi(A, leaves, C):
    """InsideOutside over a per-column model list whose pis differ
    (subby/jax/__init__.py:721-774): the passes of every column take the
    first model's pi at the root, the root's own posterior row the column's
    own pi.  Each group runs on a plan with that root prior
    (subby_plan_set_root_prior); compared with the oracle restated the same
    way, node and branch posteriors, every node."""
    rng = np.random.default_rng(70 + A)
    if A == 4:
        ms = [models.hky85_diag(2.0, rng.dirichlet(np.ones(4))) for _ in range(3)]
    else:
        ms = [models.random_reversible(A, rng, 0.5, 2.0)[0] for _ in range(3)]
    tree = synth.random_tree(leaves, 0.1, rng)
    aln = synth.simulated_alignment(tree, ms[0], C, 0.1, rng)
    which = rng.integers(0, 3, size=C)
    which[0] = 0
    per_col = [ms[k] for k in which]
    io = sg.InsideOutside(aln, tree, per_col)
    node = np.asarray(io.node_posterior())
    br = np.asarray(io.branch_posterior())
    t = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    pi0 = np.asarray(ms[0].pi, np.float64)
    ref_n = np.zeros_like(node, dtype=np.float64)
    ref_b = np.zeros_like(br, dtype=np.float64)
    for k in range(3):
        idx = np.nonzero(which == k)[0]
        if idx.size == 0:
            continue
        sub = np.ascontiguousarray(aln[:, idx])
        md = ms[k]._asdict()
        rn = oracle.NodePosterior(sub, t, md, root_prob=pi0)
        rn[0] = oracle.NodePosterior(sub, t, md)[0]
        ref_n[..., idx] = rn
        ref_b[..., idx] = oracle.BranchPosterior(sub, t, md, root_prob=pi0)
    _check(node, ref_n, f"A={A} node posteriors, per-column pis")
    _check(br, ref_b, f"A={A} branch posteriors, per-column pis")
    # the shared-pi columns equal the plain single-model run
    one = np.nonzero(which == 0)[0]
    _check(node[..., one], oracle.NodePosterior(np.ascontiguousarray(aln[:, one]), t, ms[0]._asdict()),
           "first-model columns")
