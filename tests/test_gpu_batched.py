"""Batched models on the GPU: ``*H`` batches (discrete-gamma rate
categories), per-column model lists and MixturePosterior, vs the FP64
oracle (subby/oracle/oracle.py:208-262, 1334-1365, 1598-1615 restated;
per-column list semantics of subby/jax/__init__.py:267-277, 396-411,
617-633) and the reference oracle's mixture fixtures; the identities of the
reference's own tests (tests/test_api.py TestPerColumnModel: a list of one
model equals that model; a list of rate-scaled models equals the column-by-
column result).  Tolerances as everywhere (tests/_tol.py); mixture
posteriors 1e-4 absolute."""
import os

import numpy as np
import pytest

import oracle
from tests._tol import COUNTS_RTOL, ROOTPROB_RTOL, assert_cols, assert_loglike

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import synth, models  # noqa: E402

MIX = os.path.join(os.path.dirname(__file__), "golden", "mixture")


@pytest.mark.parametrize("name", ["ref_7node_mixture_jc4", "gamma4_hky"])
def test_mixture_fixtures(name):
    with np.load(os.path.join(MIX, name + ".npz")) as z:
        g = {k: z[k] for k in z.files}
    tree = sg.Tree(g['parentIndex'], g['distanceToParent'])
    base = sg.DiagModel(g['eigenvalues'], g['eigenvectors'], g['pi'])
    ms = [sg.scale_model(base, r) for r in g['rates']]
    post = sg.MixturePosterior(g['alignment'], tree, ms, g['log_weights'])
    np.testing.assert_allclose(post, g['posteriors'], atol=1e-4)
    # the same through one batched model: LogLike (K, C)
    ll = sg.LogLike(g['alignment'], tree, sg.scale_model(base, g['rates']))
    assert ll.shape == g['log_likes'].shape
    assert_loglike(ll, g['log_likes'])


def test_h_batch_all_outputs_and_device():
    w = synth.plain_small(seed=11, C=257)
    aln, tree, base = w['alignment'], w['tree'], w['model']
    rates, _ = sg.gamma_rate_categories(0.7, 4)
    mb = sg.scale_model(base, rates)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    ll = sg.LogLike(aln, tree, mb)
    cnt = sg.Counts(aln, tree, mb)
    rp = sg.RootProb(aln, tree, mb)
    bc = sg.BranchCounts(aln, tree, mb)
    assert ll.shape == (4, 257) and cnt.shape == (4, 4, 4, 257) and rp.shape == (4, 4, 257)
    assert bc.shape == (4, len(tree.parentIndex), 4, 4, 257)
    for k, r in enumerate(rates):
        md = oracle.scale_model(base._asdict(), r)
        assert_loglike(ll[k], oracle.LogLike(aln, ot, md))
        assert_cols(cnt[k], oracle.Counts(aln, ot, md), COUNTS_RTOL, f"counts k={k}")
        assert_cols(rp[k], oracle.RootProb(aln, ot, md), ROOTPROB_RTOL, f"rootprob k={k}")
    dev = sg.LogLike(torch.as_tensor(aln).cuda(), tree, mb)
    torch.cuda.synchronize()
    assert dev.is_cuda and tuple(dev.shape) == (4, 257)
    np.testing.assert_array_equal(dev.cpu().numpy(), ll)


def test_per_column_lists_vs_oracle():
    rng = np.random.default_rng(12)
    tree = synth.random_tree(12, 0.2, rng)
    base = models.hky85_diag(2.0, [0.25, 0.25, 0.25, 0.25])
    C = 60
    aln = synth.simulated_alignment(tree, base, C, 0.1, rng)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    # three distinct models over the columns, different pi (root prior rule)
    palette = [models.hky85_diag(2.0, [0.25] * 4), models.hky85_diag(3.0, [0.1, 0.2, 0.3, 0.4]),
               models.scale_model(models.hky85_diag(1.5, [0.4, 0.3, 0.2, 0.1]), 1.7)]
    ms = [palette[rng.integers(0, 3)] for _ in range(C)]
    ms[0] = palette[1]
    mds = [m._asdict() for m in ms]
    assert_loglike(sg.LogLike(aln, tree, ms), oracle.LogLike_per_column(aln, ot, mds))
    assert_cols(sg.RootProb(aln, tree, ms), oracle.RootProb_per_column(aln, ot, mds), ROOTPROB_RTOL, "rootprob")
    cnt = sg.Counts(aln, tree, ms)
    assert_cols(cnt, oracle.Counts_per_column(aln, ot, mds), COUNTS_RTOL, "counts")
    assert_cols(sg.Counts(aln, tree, ms, branch_mask=None), oracle.Counts_per_column(aln, ot, mds, branch_mask=None),
                COUNTS_RTOL, "counts unmasked")
    bc = sg.BranchCounts(aln, tree, ms, branch_mask="auto")
    assert_cols(bc.astype(np.float64).sum(0), cnt, COUNTS_RTOL, "branches sum to counts")
    # device inputs: same results, results on the device
    dl = sg.LogLike(torch.as_tensor(aln).cuda(), tree, ms)
    torch.cuda.synchronize()
    assert dl.is_cuda
    assert_loglike(dl.cpu().numpy(), oracle.LogLike_per_column(aln, ot, mds))


def test_reference_identities():
    """[model] * C equals the single model; rate-scaled models per column equal
    the column-by-column computation (tests/test_api.py:397-430 of ihh/subby)."""
    w = synth.plain_small(seed=13, C=40)
    aln, tree, base = w['alignment'], w['tree'], w['model']
    np.testing.assert_allclose(sg.LogLike(aln, tree, [base] * 40), sg.LogLike(aln, tree, base), atol=1e-6)
    ms = [sg.scale_model(base, r) for r in np.linspace(0.5, 2.0, 40)]
    by_col = np.array([sg.LogLike(aln[:, c:c + 1], tree, ms[c])[0] for c in range(40)])
    np.testing.assert_allclose(sg.LogLike(aln, tree, ms), by_col, atol=1e-5)
    # a (1, R) grid of one model is that model
    np.testing.assert_allclose(sg.LogLike(aln, tree, [[base] * len(tree.parentIndex)]), sg.LogLike(aln, tree, base),
                               atol=1e-5)


def test_mixture_posterior_device_and_oracle():
    w = synth.plain_small(seed=14, C=500)
    aln, tree, base = w['alignment'], w['tree'], w['model']
    rates, weights = sg.gamma_rate_categories(0.4, 6)
    ms = [sg.scale_model(base, r) for r in rates]
    lw = np.log(weights)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    ref = oracle.MixturePosterior(aln, ot, [oracle.scale_model(base._asdict(), r) for r in rates], lw)
    host = sg.MixturePosterior(aln, tree, ms, lw)
    np.testing.assert_allclose(host, ref, atol=1e-4)
    np.testing.assert_allclose(host.sum(0), 1.0, atol=1e-5)
    dev = sg.MixturePosterior(torch.as_tensor(aln).cuda(), tree, ms, lw)
    torch.cuda.synchronize()
    np.testing.assert_allclose(dev.cpu().numpy(), host, atol=1e-6)


def _hky_rows(R, rng):
    return [models.hky85_diag(float(rng.uniform(1.0, 4.0)), rng.dirichlet(np.full(4, 5.0))) for _ in range(R)]


def test_per_branch_models_vs_oracle():
    """(1, R) model grid: each branch its own HKY85 model (three distinct
    models over the branches), A = 4; identical rows equal the single model."""
    rng = np.random.default_rng(15)
    tree = synth.random_tree(10, 0.2, rng)
    R = len(tree.parentIndex)
    palette = _hky_rows(3, rng)
    rows = [palette[rng.integers(0, 3)] for _ in range(R)]
    aln = synth.simulated_alignment(tree, palette[0], 90, 0.1, rng)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    rd = [m._asdict() for m in rows]
    assert_loglike(sg.LogLike(aln, tree, [rows]), oracle.LogLike_rows(aln, ot, rd))
    assert_cols(sg.RootProb(aln, tree, [rows]), oracle.RootProb_rows(aln, ot, rd), ROOTPROB_RTOL, "rootprob")
    cnt = sg.Counts(aln, tree, [rows])
    assert_cols(cnt, oracle.Counts_rows(aln, ot, rd), COUNTS_RTOL, "counts")
    assert_cols(sg.Counts(aln, tree, [rows], branch_mask=None), oracle.Counts_rows(aln, ot, rd, branch_mask=None),
                COUNTS_RTOL, "counts unmasked")
    bc = sg.BranchCounts(aln, tree, [rows])
    ref = oracle.BranchCounts_rows(aln, ot, rd)
    assert_cols(bc.transpose(1, 2, 0, 3).reshape(4, 4, -1), ref.transpose(1, 2, 0, 3).reshape(4, 4, -1),
                COUNTS_RTOL, "branch counts")
    # identical rows: the single-model results
    same = [rows[0]] * R
    assert_loglike(sg.LogLike(aln, tree, [same]), sg.LogLike(aln, tree, rows[0]))
    assert_cols(sg.Counts(aln, tree, [same]), sg.Counts(aln, tree, rows[0]), COUNTS_RTOL, "same rows")


def test_per_branch_models_large_alphabet_and_column_grid():
    rng = np.random.default_rng(16)
    tree = synth.random_tree(7, 0.15, rng)
    R = len(tree.parentIndex)
    pal = [models.random_reversible(20, rng, 0.5, 2.0)[0] for _ in range(2)]
    rows = [pal[n % 2] for n in range(R)]
    aln = rng.integers(0, 22, size=(R, 37)).astype(np.int32)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    rd = [m._asdict() for m in rows]
    assert_loglike(sg.LogLike(aln, tree, [rows]), oracle.LogLike_rows(aln, ot, rd))
    assert_cols(sg.Counts(aln, tree, [rows]), oracle.Counts_rows(aln, ot, rd), COUNTS_RTOL, "A=20 rows counts")
    # (C, R): two row sets over the columns
    rows2 = [pal[(n + 1) % 2] for n in range(R)]
    grid = [rows if c % 3 else rows2 for c in range(37)]
    ll = sg.LogLike(aln, tree, grid)
    ref = np.array([oracle.LogLike_rows(aln[:, c:c + 1], ot, [m._asdict() for m in grid[c]])[0] for c in range(37)])
    assert_loglike(ll, ref)
    cnt = sg.Counts(aln, tree, grid)
    refc = np.concatenate([oracle.Counts_rows(aln[:, c:c + 1], ot, [m._asdict() for m in grid[c]])
                           for c in range(37)], axis=-1)
    assert_cols(cnt, refc, COUNTS_RTOL, "column grid counts")


def test_inside_outside_batched_and_lists():
    w = synth.plain_small(seed=17, C=120)
    aln, tree, base = w['alignment'], w['tree'], w['model']
    rates = np.array([0.5, 1.0, 2.0])
    io = sg.InsideOutside(aln, tree, sg.scale_model(base, rates))
    npost = io.node_posterior()
    assert npost.shape == (3, len(tree.parentIndex), 4, 120)
    for k, r in enumerate(rates):
        one = sg.InsideOutside(aln, tree, sg.scale_model(base, r))
        np.testing.assert_array_equal(npost[k], one.node_posterior())
        np.testing.assert_array_equal(io.branch_posterior(3)[k], one.branch_posterior(3))
    # per-column list sharing pi: grouped posteriors equal the per-model ones
    ms = [sg.scale_model(base, rates[c % 3]) for c in range(120)]
    iol = sg.InsideOutside(aln, tree, ms)
    got = iol.node_posterior()
    for k in range(3):
        cols = np.arange(k, 120, 3)
        ref = sg.InsideOutside(aln[:, cols], tree, sg.scale_model(base, rates[k])).node_posterior()
        np.testing.assert_array_equal(got[..., cols], ref)
    assert_loglike(iol.log_likelihood, sg.LogLike(aln, tree, ms))
    with pytest.raises(NotImplementedError):
        sg.InsideOutside(aln, tree, [[base] * len(tree.parentIndex)])
