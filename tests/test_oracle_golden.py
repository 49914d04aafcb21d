"""Pins the FP64 oracle (oracle/oracle.py) to the reference.

* against fixtures made by running the reference's own oracle
  (tests/golden/make_golden.py), including every intermediate for the small
  cases, and
* against the reference's golden JSON files directly when the reference tree
  is mounted (skipped otherwise).
"""
import json
import os

import numpy as np
import pytest

import oracle
from tests import _golden

CASES = _golden.names()


def _tree(g):
    return oracle.Tree(g['parentIndex'], g['distanceToParent'])


def _model(g):
    return _golden.model_dict(g)


@pytest.mark.parametrize("name", CASES)
def test_outputs_match_reference_oracle(name):
    g = _golden.load(name)
    aln, tree, model = g['alignment'], _tree(g), _model(g)
    np.testing.assert_allclose(oracle.LogLike(aln, tree, model), g['logLike'], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(oracle.Counts(aln, tree, model, branch_mask=None), g['counts'],
                               rtol=1e-9, atol=1e-11)
    if 'counts_masked' in g:
        np.testing.assert_allclose(oracle.Counts(aln, tree, model), g['counts_masked'],
                                   rtol=1e-9, atol=1e-11)
    if 'counts_f81' in g:
        np.testing.assert_allclose(oracle.Counts(aln, tree, model, f81_fast=True, branch_mask=None),
                                   g['counts_f81'], rtol=1e-9, atol=1e-11)
    if 'counts_f81_masked' in g:
        np.testing.assert_allclose(oracle.Counts(aln, tree, model, f81_fast=True),
                                   g['counts_f81_masked'], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(oracle.RootProb(aln, tree, model), g['root_prob'], rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(
        oracle.compute_branch_mask(aln, g['parentIndex'], int(g['A'])), g['branch_mask'])
    if 'branch_counts' in g:
        np.testing.assert_allclose(oracle.BranchCounts(aln, tree, model), g['branch_counts'],
                                   rtol=1e-9, atol=1e-11)
    if 'branch_counts_masked' in g:
        np.testing.assert_allclose(oracle.BranchCounts(aln, tree, model, branch_mask="auto"),
                                   g['branch_counts_masked'], rtol=1e-9, atol=1e-11)
    if 'branch_counts_f81' in g:
        np.testing.assert_allclose(oracle.BranchCounts(aln, tree, model, f81_fast=True),
                                   g['branch_counts_f81'], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(oracle.NodePosterior(aln, tree, model), g['node_posterior'],
                               rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(oracle.BranchPosterior(aln, tree, model), g['branch_posterior'],
                               rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("name", [n for n in CASES if 'U' in _golden.load(n)])
def test_intermediates_match_reference_oracle(name):
    g = _golden.load(name)
    p = oracle.pipeline(g['alignment'], _tree(g), _model(g))
    for k in ('sub_matrices', 'U', 'logNormU', 'D', 'logNormD', 'J', 'U_tilde', 'D_tilde', 'C_eigen'):
        np.testing.assert_allclose(p[k], g[k], rtol=1e-11, atol=1e-12, err_msg=k)


REF_GOLDEN = "/root/reference/tests/golden"


@pytest.mark.skipif(not os.path.isdir(REF_GOLDEN), reason="reference tree not mounted")
@pytest.mark.parametrize("fname", ["5node_jc4", "7node_hky85_4", "7node_jc4_mixed_gaps",
                                   "7node_jc4_all_gaps", "7node_jc64"])
def test_reference_golden_json(fname):
    with open(os.path.join(REF_GOLDEN, fname + ".json")) as f:
        gj = json.load(f)
    inp = gj['inputs']
    aln = np.asarray(inp['alignment'], dtype=np.int32)
    tree = oracle.Tree(inp['parentIndex'], inp['distanceToParent'])
    model = {k: np.asarray(v) for k, v in inp['model'].items()}
    p = oracle.pipeline(aln, tree, model)
    out = gj['outputs']
    np.testing.assert_allclose(p['logLike'], out['logLike'], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(p['counts'], out['counts'], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(oracle.RootProb(aln, tree, model), out['root_prob'], rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(oracle.compute_branch_mask(aln, tree.parentIndex, inp['A']),
                                  np.asarray(out['branch_mask']))
    inter = gj['intermediates']
    for k in ('sub_matrices', 'U', 'logNormU', 'D', 'logNormD', 'J', 'U_tilde', 'D_tilde', 'C_eigen'):
        np.testing.assert_allclose(p[k], np.asarray(inter[k]), rtol=1e-10, atol=1e-12, err_msg=k)


def test_validate_binary_tree_rejects():
    with pytest.raises(ValueError):
        oracle.validate_binary_tree([-1, 0, 0, 0])
    oracle.validate_binary_tree([-1, 0, 0, 1, 1])


MIXTURE_DIR = os.path.join(os.path.dirname(__file__), "golden", "mixture")


@pytest.mark.parametrize("name", ["ref_7node_mixture_jc4", "gamma4_hky"])
def test_mixture_matches_reference_oracle(name):
    with np.load(os.path.join(MIXTURE_DIR, name + ".npz")) as z:
        g = {k: z[k] for k in z.files}
    tree = oracle.Tree(g['parentIndex'], g['distanceToParent'])
    base = {k: g[k] for k in ('eigenvalues', 'eigenvectors', 'pi')}
    ms = [oracle.scale_model(base, r) for r in g['rates']]
    np.testing.assert_allclose(np.stack([oracle.LogLike(g['alignment'], tree, m) for m in ms]), g['log_likes'],
                               rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(oracle.MixturePosterior(g['alignment'], tree, ms, g['log_weights']),
                               g['posteriors'], rtol=1e-12, atol=1e-14)


def test_gamma_rate_categories_match_reference_oracle():
    with np.load(os.path.join(MIXTURE_DIR, "gamma_categories.npz")) as z:
        for a, r in zip(z['alpha'], z['rates']):
            np.testing.assert_allclose(oracle.gamma_rate_categories(float(a), 4)[0], r, rtol=1e-14)


@pytest.mark.skipif(not os.path.isdir(REF_GOLDEN), reason="reference tree not mounted")
def test_reference_mixture_json():
    with open(os.path.join(REF_GOLDEN, "7node_mixture_jc4.json")) as f:
        gj = json.load(f)
    inp, out = gj['inputs'], gj['outputs']
    base = {k: np.asarray(v) for k, v in inp['base_model'].items()}
    ms = [oracle.scale_model(base, r) for r in inp['rates']]
    tree = oracle.Tree(inp['parentIndex'], inp['distanceToParent'])
    aln = np.asarray(inp['alignment'], dtype=np.int32)
    np.testing.assert_allclose(oracle.MixturePosterior(aln, tree, ms, np.asarray(inp['log_weights'])),
                               np.asarray(out['posteriors']), rtol=1e-12, atol=1e-14)
