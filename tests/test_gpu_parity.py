"""GPU parity: the CUDA path through the C ABI vs the FP64 oracle.

Every case compares LogLike, Counts (unmasked, Steiner-masked, F81 fast
path) and RootProb with the tolerances of tests/_tol.py, on
* the golden fixtures made by the reference oracle (tests/golden/*.npz), and
* seeded synthetic workloads at sizes the oracle finishes in seconds.
"""
import numpy as np
import pytest

import oracle
from tests import _golden
from tests._tol import (assert_cols, assert_loglike, COUNTS_RTOL, ROOTPROB_RTOL)

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import synth, models, _lib  # noqa: E402


KERNELS = {"auto": 0, "thread": 1, "tree_smem": 2, "tree_global": 3, "tree_tmem": 4}


@pytest.fixture(params=["auto", "thread", "tree_smem"])
def big_kernel(request):
    """Large alphabets: tree walk + staged accumulation (auto: tensor cores
    at A = 64), warp per column (thread), FP32 CUDA-core walk (tree_smem)."""
    _lib.load().subby_debug_set_kernel(KERNELS[request.param])
    yield request.param
    _lib.load().subby_debug_set_kernel(0)


@pytest.fixture(params=list(KERNELS))
def kernel(request):
    """Run a test through every kernel / slot-storage variant for A <= 8."""
    _lib.load().subby_debug_set_kernel(KERNELS[request.param])
    yield request.param
    _lib.load().subby_debug_set_kernel(0)


def _model_dict(m):
    return {'eigenvalues': np.asarray(m.eigenvalues), 'eigenvectors': np.asarray(m.eigenvectors),
            'pi': np.asarray(m.pi)}


def _check_all(aln, tree, model, f81=False, masked=True, rp=True, bt64=None):
    """Run every output through one plan and compare with the oracle."""
    md = _model_dict(model)
    otree = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    plan = sg.Plan(tree, model)
    r = plan.run(aln, loglike=True, counts=True, rootprob=rp, branch_mask=None, bt64=bt64)
    assert_loglike(r['logLike'], oracle.LogLike(aln, otree, md))
    assert_cols(r['counts'], oracle.Counts(aln, otree, md, branch_mask=None), COUNTS_RTOL, "counts")
    if rp:
        assert_cols(r['rootProb'], oracle.RootProb(aln, otree, md), ROOTPROB_RTOL, "rootProb")
    if masked:
        rm = plan.run(aln, loglike=False, counts=True, branch_mask="auto", bt64=bt64)
        assert_cols(rm['counts'], oracle.Counts(aln, otree, md), COUNTS_RTOL, "masked counts")
    if f81:
        rf = plan.run(aln, loglike=False, counts=True, f81=True, branch_mask=None)
        assert_cols(rf['counts'], oracle.Counts(aln, otree, md, f81_fast=True, branch_mask=None),
                    COUNTS_RTOL, "f81 counts")
        if masked:
            rfm = plan.run(aln, loglike=False, counts=True, f81=True, branch_mask="auto")
            assert_cols(rfm['counts'], oracle.Counts(aln, otree, md, f81_fast=True), COUNTS_RTOL,
                        "f81 masked counts")
    plan.close()


@pytest.mark.parametrize("name", _golden.names())
def test_golden(name, kernel):
    g = _golden.load(name)
    tree = sg.Tree(g['parentIndex'], g['distanceToParent'])
    model = sg.models.ensure_diag(_golden.model_dict(g))   # IrrevDiagModel for the irrev_* fixtures
    plan = sg.Plan(tree, model)
    r = plan.run(g['alignment'], loglike=True, counts=True, rootprob=True, branch_mask=None)
    assert_loglike(r['logLike'], g['logLike'])
    assert_cols(r['counts'], g['counts'], COUNTS_RTOL, "counts")
    assert_cols(r['rootProb'], g['root_prob'], ROOTPROB_RTOL, "rootProb")
    if 'counts_masked' in g:
        rm = plan.run(g['alignment'], loglike=False, counts=True, branch_mask="auto")
        assert_cols(rm['counts'], g['counts_masked'], COUNTS_RTOL, "masked counts")
    if 'counts_f81' in g:
        rf = plan.run(g['alignment'], loglike=False, counts=True, f81=True, branch_mask=None)
        assert_cols(rf['counts'], g['counts_f81'], COUNTS_RTOL, "f81 counts")
    if 'counts_f81_masked' in g:
        rf = plan.run(g['alignment'], loglike=False, counts=True, f81=True, branch_mask="auto")
        assert_cols(rf['counts'], g['counts_f81_masked'], COUNTS_RTOL, "f81 masked counts")
    # the given-mask mode reproduces "auto" when handed the reference's own mask
    if 'counts_masked' in g:
        rg = plan.run(g['alignment'], loglike=False, counts=True, branch_mask=g['branch_mask'])
        assert_cols(rg['counts'], g['counts_masked'], COUNTS_RTOL, "given-mask counts")
    plan.close()


def test_plain_small_full(kernel):
    w = synth.plain_small(seed=1, C=1024)
    _check_all(w['alignment'], w['tree'], w['model'])


def test_plain_large_subset_hky_and_f81(kernel):
    for f81 in (False, True):
        w = synth.plain_large(seed=2, C=3000, f81=f81)
        _check_all(w['alignment'], w['tree'], w['model'], f81=f81)


@pytest.mark.parametrize("A,leaves,C", [(16, 12, 40), (20, 9, 33), (32, 6, 20), (64, 10, 24), (64, 30, 300),
                                        (16, 40, 1000)])
def test_reversible_larger_alphabets(A, leaves, C, big_kernel):
    rng = np.random.default_rng(100 + A)
    m, _, _, _ = models.near_degenerate_reversible(A, rng)
    tree = synth.random_tree(leaves, 0.1, rng)
    aln = synth.simulated_alignment(tree, m, C, 0.1, rng)
    _check_all(aln, tree, m)


def test_precision64_subset(big_kernel):
    w = synth.precision64(seed=3, C=48)
    ev = np.sort(np.asarray(w['model'].eigenvalues))
    gaps = np.abs(ev[:, None] - ev[None, :])[np.triu_indices(len(ev), 1)]
    assert np.mean(gaps < 1e-7) >= 0.04          # ~5% near-degenerate pairs
    assert np.any(gaps < 1e-8) and np.any((gaps > 1e-8) & (gaps < 1e-7))
    _check_all(w['alignment'], w['tree'], w['model'], masked=False)


def test_f81_counts_general_model_large_alphabet(big_kernel):
    """F81 counts requested with a general reversible model (the reference
    applies the F81 formulas to the model's own inside/outside vectors): the
    tensor-core walk stages F81 vectors and, at A = 64, the tensor-core F81
    accumulation runs; vs the oracle, masked and unmasked, with ragged
    column counts (last group short)."""
    rng = np.random.default_rng(17)
    for A, C in ((64, 37), (20, 29)):
        m, _, _ = models.random_reversible(A, rng, 0.5, 2.0)
        tree = synth.random_tree(21, 0.1, rng)
        aln = synth.simulated_alignment(tree, m, C, 0.1, rng)
        otree = oracle.Tree(tree.parentIndex, tree.distanceToParent)
        plan = sg.Plan(tree, m)
        for bm in (None, "auto"):
            got = plan.run(aln, loglike=False, counts=True, f81=True, branch_mask=bm)['counts']
            ref = oracle.Counts(aln, otree, _model_dict(m), f81_fast=True, branch_mask=bm)
            assert_cols(got, ref, COUNTS_RTOL, f"A={A} f81 counts mask={bm}")
        plan.close()


@pytest.mark.parametrize("A", [2, 3, 4, 5, 6, 8])
def test_small_alphabets(A, kernel):
    rng = np.random.default_rng(200 + A)
    base, _, _ = models.random_reversible(A, rng)
    tree = synth.random_tree(20, 0.2, rng)
    aln = synth.simulated_alignment(tree, base, 77, 0.1, rng)
    _check_all(aln, tree, base)


def test_jc_and_f81_fast_paths_large_alphabet(big_kernel):
    """F81 / JC models: the large-alphabet walk detects the closed form of
    M(t) and uses it for LogLike-only and F81-count runs (general products
    for eigen counts); every output against the oracle."""
    rng = np.random.default_rng(7)
    tree = synth.random_tree(14, 0.1, rng)
    otree = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    for m in (models.jukes_cantor_model(64), models.f81_model(rng.dirichlet(np.ones(20))),
              models.f81_model(rng.dirichlet(np.ones(64))), models.jukes_cantor_model(16),
              models.f81_model(rng.dirichlet(np.ones(32)))):
        aln = synth.simulated_alignment(tree, m, 19, 0.1, rng)
        _check_all(aln, tree, m, f81=True)
        plan = sg.Plan(tree, m)
        ll = plan.run(aln, loglike=True)['logLike']
        assert_loglike(ll, oracle.LogLike(aln, otree, _model_dict(m)))
        plan.close()


def test_edge_cases(kernel):
    rng = np.random.default_rng(9)
    m = models.hky85_diag(2.0, [0.3, 0.2, 0.25, 0.25])
    # R = 1 (root only) and R = 3
    for tree in (sg.Tree(np.array([-1], np.int32), np.array([0.0])),
                 sg.Tree(np.array([-1, 0, 0], np.int32), np.array([0.0, 0.3, 0.05]))):
        R = len(tree.parentIndex)
        aln = rng.integers(-1, 6, size=(R, 37)).astype(np.int32)
        _check_all(aln, tree, m)
    # C = 1, C not a multiple of 32, all-gap columns, all-unobserved columns
    tree = synth.random_tree(30, 0.1, rng)
    for C in (1, 31, 33, 129):
        aln = synth.simulated_alignment(tree, m, C, 0.2, rng)
        aln[:, 0] = -1
        _check_all(aln, tree, m)
    # BFS-numbered balanced tree (not DFS order), as in the reference tests
    R = 31
    parent = np.array([-1] + [(i - 1) // 2 for i in range(1, R)], np.int32)
    dist = rng.uniform(0.01, 0.5, R)
    dist[0] = 0
    tree = sg.Tree(parent, dist)
    aln = rng.integers(-1, 5, size=(R, 50)).astype(np.int32)
    _check_all(aln, tree, m)


def test_device_pointer_path_matches_host_path():
    w = synth.plain_large(seed=2, C=2048)
    plan = sg.Plan(w['tree'], w['model'])
    host = plan.run(w['alignment'], loglike=True, counts=True, rootprob=True)
    dev = plan.run(torch.as_tensor(w['alignment']).cuda(), loglike=True, counts=True, rootprob=True)
    torch.cuda.synchronize()
    for k in host:
        np.testing.assert_array_equal(dev[k].cpu().numpy(), host[k])


@pytest.mark.parametrize("A,waves", [(4, 3.3), (20, 5.0)])
def test_chunked_host_pipeline_matches_device_path(A, waves):
    """Host buffers large enough to be split into column chunks (copy-in,
    kernel and copy-out of neighbouring chunks overlap on three queues) give
    bit-identical results to one device-pointer call over all columns."""
    W = torch.cuda.get_device_properties(0).multi_processor_count * 256
    C = int(waves * W) + 77
    rng = np.random.default_rng(5 + A)
    tree = synth.random_tree(24, 0.1, rng)
    model = models.random_reversible(A, rng, 0.5, 2.0)[0] if A > 4 else models.hky85_diag(2.0, np.full(4, 0.25))
    R = len(tree.parentIndex)
    aln = rng.integers(-1, A + 2, size=(R, C)).astype(np.int32)
    mask = (rng.random((R, C)) < 0.7).astype(np.uint8)
    plan = sg.Plan(tree, model)
    d_aln = torch.as_tensor(aln).cuda()
    for bm in ("auto", mask):
        host = plan.run(aln, loglike=True, counts=True, rootprob=True, branch_mask=bm)
        dbm = torch.as_tensor(bm).cuda() if isinstance(bm, np.ndarray) else bm
        dev = plan.run(d_aln, loglike=True, counts=True, rootprob=True, branch_mask=dbm)
        torch.cuda.synchronize()
        for k in host:
            np.testing.assert_array_equal(dev[k].cpu().numpy(), host[k], err_msg=k)
    plan.close()


def test_deterministic_repeat():
    w = synth.plain_large(seed=2, C=4096)
    plan = sg.Plan(w['tree'], w['model'])
    a = plan.run(w['alignment'], counts=True, rootprob=True)
    b = plan.run(w['alignment'], counts=True, rootprob=True)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])


def test_subby_jax_style_api():
    w = synth.plain_small(seed=1, C=256)
    aln, tree, m = w['alignment'], w['tree'], w['model']
    md = _model_dict(m)
    otree = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    assert_loglike(sg.LogLike(aln, tree, m), oracle.LogLike(aln, otree, md))
    assert_cols(sg.Counts(aln, tree, m), oracle.Counts(aln, otree, md), COUNTS_RTOL, "Counts")
    assert_cols(sg.Counts(aln, tree, m, branch_mask=None),
                oracle.Counts(aln, otree, md, branch_mask=None), COUNTS_RTOL, "Counts unmasked")
    assert_cols(sg.RootProb(aln, tree, m), oracle.RootProb(aln, otree, md), ROOTPROB_RTOL, "RootProb")
    # RateModel input is diagonalised on the host
    Q = models.reversible_rate_matrix(np.zeros(6), m.pi)
    rm = sg.RateModel(Q, m.pi)
    dm = models.diagonalize_rate_matrix(Q, m.pi)
    np.testing.assert_allclose(sg.LogLike(aln, tree, rm), sg.LogLike(aln, tree, dm), rtol=1e-6)


def test_fp32_vs_fp64_back_transform_both_within_tolerance():
    w = synth.plain_small(seed=1, C=512)
    md = _model_dict(w['model'])
    otree = oracle.Tree(w['tree'].parentIndex, w['tree'].distanceToParent)
    ref = oracle.Counts(w['alignment'], otree, md, branch_mask=None)
    plan = sg.Plan(w['tree'], w['model'])
    for bt in (True, False):
        r = plan.run(w['alignment'], loglike=False, counts=True, branch_mask=None, bt64=bt)
        assert_cols(r['counts'], ref, COUNTS_RTOL, f"counts bt64={bt}")


@pytest.mark.parametrize("sel", [0, 2], ids=["tensor_core_walk", "fp32_walk"])
@pytest.mark.parametrize("mask", ["auto", None], ids=["masked", "unmasked"])
def test_tensor_core_walk_repeatable_small_tree(sel, mask):
    """A=64 reversible model, 6-leaf tree, 314 columns (three 128-column
    tiles, the last one ragged), where a stored child's step directly
    follows the step that writes its slot word: 30 runs agree bit for bit
    and every run matches the oracle.  (Before each column half kept its own
    slot word, the half in warp w + 4 could read the word before warp w wrote
    it, and columns 0-31 of a tile came out wrong.)"""
    rng = np.random.default_rng(77)
    m = models.random_reversible(64, rng)[0]
    tree = sg.Tree(np.array([-1, 0, 1, 2, 2, 1, 5, 5, 7, 7, 0], dtype=np.int32),
                   rng.exponential(0.1, 11))
    aln = synth.simulated_alignment(tree, m, 314, 0.05, rng)
    oref = oracle.Counts(aln, oracle.Tree(tree.parentIndex, tree.distanceToParent), _model_dict(m),
                         branch_mask=mask)
    lib = _lib.load()
    plan = sg.Plan(tree, m)
    try:
        lib.subby_debug_set_kernel(sel)
        ref = plan.run(aln, loglike=True, counts=True, branch_mask=mask)['counts']
        assert_cols(ref, oref, COUNTS_RTOL, "first run vs oracle")
        for _ in range(30):
            got = plan.run(aln, loglike=True, counts=True, branch_mask=mask)['counts']
            assert_cols(got, oref, COUNTS_RTOL, "repeat vs oracle")
            np.testing.assert_array_equal(got, ref)
    finally:
        lib.subby_debug_set_kernel(0)
        plan.close()


@pytest.mark.parametrize("A", [4, 20])
def test_zero_columns(A):
    """C = 0 gives empty outputs of the reference's shapes (the reference
    oracle returns them too) through every entry point, on host arrays and on
    CUDA tensors (whose data pointer is null when empty); the gradient of the
    empty sum is zero."""
    rng = np.random.default_rng(4)
    m = models.hky85_diag(2.0, [0.3, 0.2, 0.25, 0.25]) if A == 4 else models.random_reversible(A, rng)[0]
    tree = synth.random_tree(6, 0.1, rng)
    R = len(tree.parentIndex)
    otree = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    md = _model_dict(m)
    empty = np.zeros((R, 0), np.int32)
    assert oracle.Counts(empty, otree, md).shape == (A, A, 0)
    plan = sg.Plan(tree, m)
    for aln in (empty, torch.zeros((R, 0), dtype=torch.int32, device="cuda")):
        r = plan.run(aln, loglike=True, counts=True, rootprob=True)
        assert tuple(r['logLike'].shape) == (0,)
        assert tuple(r['counts'].shape) == (A, A, 0)
        assert tuple(r['rootProb'].shape) == (A, 0)
        r = plan.run(aln, loglike=False, counts=True, branch_mask=np.zeros((R, 0), bool))
        assert tuple(r['counts'].shape) == (A, A, 0)
        assert tuple(plan.branch_counts(aln).shape) == (R, A, A, 0)
        post = plan.posteriors(aln, want_node=True, want_branch=True)
        assert tuple(post['node'].shape) == (R, A, 0) and tuple(post['branch'].shape) == (R, A, A, 0)
        assert tuple(sg.MixturePosterior(aln, tree, [m, m], np.log([0.25, 0.75])).shape) == (2, 0)
    torch.cuda.synchronize()
    ll, dldt, dldS = plan.grad(empty)
    assert ll.shape == (0,) and dldt.shape == (R,) and not dldt.any() and not dldS.any()
    plan.close()


def test_padded_tree_and_alignment_are_neutral():
    """subby.jax's padding workflow (pad_tree_and_alignment, then LogLike /
    RootProb / MixturePosterior on the padded inputs, then unpad_columns):
    the real columns equal the unpadded results and the gap columns have
    logLike 0, as in the reference's padding tests."""
    rng = np.random.default_rng(12)
    m = models.hky85_diag(2.0, [0.3, 0.2, 0.25, 0.25])
    m2 = models.hky85_diag(4.0, [0.25, 0.25, 0.25, 0.25])
    tree = synth.random_tree(40, 0.1, rng)
    aln = synth.simulated_alignment(tree, m, 300, 0.1, rng)
    ptree, paln, R, C = sg.pad_tree_and_alignment(tree, aln)
    assert len(ptree.parentIndex) > R and paln.shape[1] > C
    ll = sg.LogLike(paln, ptree, m)
    assert_loglike(sg.unpad_columns(ll, C), sg.LogLike(aln, tree, m))
    assert np.abs(ll[C:]).max() <= 1e-5
    assert_cols(sg.unpad_columns(sg.RootProb(paln, ptree, m), C), sg.RootProb(aln, tree, m), ROOTPROB_RTOL,
                "RootProb")
    lw = np.log([0.3, 0.7])
    assert_cols(sg.unpad_columns(sg.MixturePosterior(paln, ptree, [m, m2], lw), C),
                sg.MixturePosterior(aln, tree, [m, m2], lw), 1e-5, "MixturePosterior")
    dev = sg.LogLike(torch.as_tensor(paln).cuda(), ptree, m)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev.cpu().numpy(), ll)
    with pytest.raises(_lib.TreeError):          # Counts keeps the reference's binary-tree rule
        sg.Counts(paln, ptree, m)
