"""Per-branch counts (subby_plan_branch_counts / sg.BranchCounts) vs the FP64
oracle's BranchCounts (subby/oracle/oracle.py:1517-1568 restated in
oracle/) and vs the reference oracle's fixtures.

Tolerance: each (branch, column) is one "column" of the norm-wise measure
of tests/_tol.py (max_ij |d| / max(max_ij |ref|, 1e-3) <= 1e-4)."""
import numpy as np
import pytest

import oracle
from tests import _golden
from tests._tol import COUNTS_RTOL

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import synth, models, _lib  # noqa: E402


def _branch_err(got, ref, floor=1e-3):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    R, A, _, C = ref.shape
    g = got.transpose(1, 2, 0, 3).reshape(A * A, R * C)
    r = ref.transpose(1, 2, 0, 3).reshape(A * A, R * C)
    num = np.max(np.abs(g - r), axis=0)
    den = np.maximum(np.max(np.abs(r), axis=0), floor)
    return float(np.max(num / den))


def _assert_bc(got, ref, what):
    assert got.shape == ref.shape, (got.shape, ref.shape)
    e = _branch_err(got, ref)
    assert e <= COUNTS_RTOL, f"{what}: per-branch column-wise error {e:.2e} > {COUNTS_RTOL:.0e}"
    np.testing.assert_array_equal(got[0], 0.0)


def _model(g):
    return sg.models.ensure_diag(_golden.model_dict(g))


@pytest.mark.parametrize("name", [n for n in _golden.names() if 'branch_counts' in _golden.load(n)])
def test_golden_branch_counts(name):
    g = _golden.load(name)
    tree = sg.Tree(g['parentIndex'], g['distanceToParent'])
    plan = sg.Plan(tree, _model(g))
    _assert_bc(plan.branch_counts(g['alignment']), g['branch_counts'], name)
    if 'branch_counts_masked' in g:
        _assert_bc(plan.branch_counts(g['alignment'], branch_mask="auto"), g['branch_counts_masked'],
                   name + " masked")
    if 'branch_counts_f81' in g:
        _assert_bc(plan.branch_counts(g['alignment'], f81=True), g['branch_counts_f81'], name + " f81")
    plan.close()


def test_plain_workloads_vs_oracle_and_sum_equals_counts():
    for w, f81 in ((synth.plain_small(seed=3, C=300), False),
                   (synth.plain_large(seed=4, C=257, f81=True), True)):
        aln, tree, m = w['alignment'], w['tree'], w['model']
        md = m._asdict()
        ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
        plan = sg.Plan(tree, m)
        for bm in (None, "auto"):
            got = plan.branch_counts(aln, f81=f81, branch_mask=bm)
            _assert_bc(got, oracle.BranchCounts(aln, ot, md, f81_fast=f81, branch_mask=bm), f"bm={bm}")
            # the branches sum to Counts
            tot = plan.run(aln, loglike=False, counts=True, f81=f81, branch_mask=bm)['counts']
            s = got.astype(np.float64).sum(0)
            den = np.maximum(np.abs(tot).max(axis=(0, 1)), 1e-3)
            assert np.max(np.abs(s - tot).max(axis=(0, 1)) / den) <= COUNTS_RTOL
        plan.close()


def test_given_mask_device_pointers_and_api():
    w = synth.plain_small(seed=5, C=130)
    aln, tree, m = w['alignment'], w['tree'], w['model']
    R = aln.shape[0]
    mask = np.random.default_rng(1).random((R, 130)) < 0.6
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    plan = sg.Plan(tree, m)
    host = plan.branch_counts(aln, branch_mask=mask)
    _assert_bc(host, oracle.BranchCounts(aln, ot, m._asdict(), branch_mask=mask), "given mask")
    dev = plan.branch_counts(torch.as_tensor(aln).cuda(), branch_mask=torch.as_tensor(mask).cuda())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev.cpu().numpy(), host)
    np.testing.assert_array_equal(sg.BranchCounts(aln, tree, m), plan.branch_counts(aln))
    plan.close()


@pytest.mark.parametrize("A,leaves,C", [(16, 9, 45), (20, 7, 33), (32, 5, 17), (64, 6, 21)])
def test_large_alphabets_vs_oracle(A, leaves, C):
    """Walk staging + the per-branch accumulation kernel (A >= 16), eigen
    and F81 counts, unmasked and masked; tensor-core walk at A = 64."""
    rng = np.random.default_rng(30 + A)
    m = models.near_degenerate_reversible(A, rng)[0]
    tree = synth.random_tree(leaves, 0.1, rng)
    aln = synth.simulated_alignment(tree, m, C, 0.1, rng)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    plan = sg.Plan(tree, m)
    for f81, bm in ((False, None), (False, "auto"), (True, None)):
        got = plan.branch_counts(aln, f81=f81, branch_mask=bm)
        _assert_bc(got, oracle.BranchCounts(aln, ot, m._asdict(), f81_fast=f81, branch_mask=bm),
                   f"A={A} f81={f81} mask={bm}")
    plan.close()


def test_unsupported_alphabet_raises():
    rng = np.random.default_rng(2)
    m = models.random_reversible(6, rng)[0]
    tree = synth.random_tree(6, 0.1, rng)
    aln = synth.simulated_alignment(tree, m, 8, 0.1, rng)
    plan = sg.Plan(tree, m)
    with pytest.raises(_lib.SubbyError):
        plan.branch_counts(aln)
    plan.close()
