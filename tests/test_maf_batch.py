"""MAF batch pipeline host logic (subby_gb300/maf_batch.py) against the
reference batch script's own outputs (tests/golden/maf, made by
make_maf_golden.py from scripts/batch_eigensub_maf.py): block parsing
(plain and gzip), tree pruning, token mapping, tree expansion, feature
layout, diagnostics, processing order, and the whole pipeline with the FP64
oracle's Counts in place of the GPU's.  CPU only."""
import gzip
import json
import os
import shutil

import numpy as np
import pytest

import oracle
from subby_gb300 import formats, maf_batch
from tests._tol import assert_cols

D = os.path.join(os.path.dirname(__file__), "golden", "maf")
with open(os.path.join(D, "expected.json")) as f:
    E = json.load(f)
Z = np.load(os.path.join(D, "expected.npz"))
MAF = os.path.join(D, "blocks.maf")


def _guide():
    with open(os.path.join(D, "guide.nh")) as f:
        return formats.parse_newick("".join(f.read().split()))


def _scan():
    return maf_batch.scan_blocks(MAF, _guide(), E["exclude"], E["min_species"], E["min_cols"], E["max_cols"])


@pytest.mark.parametrize("gz", [False, True])
def test_iter_maf_blocks(gz, tmp_path):
    path = MAF
    if gz:
        path = str(tmp_path / "blocks.maf.gz")
        with open(MAF, "rb") as src, gzip.open(path, "wb") as dst:
            shutil.copyfileobj(src, dst)
    assert list(maf_batch.iter_maf_blocks(path)) == E["blocks"]


def test_prune_tree():
    guide = _guide()
    for case in E["prune"]:
        got = maf_batch.prune_tree(guide, set(case["keep"]))
        exp = case["result"]
        if exp is None:
            assert got is None, case["keep"]
            continue
        assert got["parentIndex"].dtype == np.int32
        assert got["parentIndex"].tolist() == exp["parentIndex"]
        np.testing.assert_allclose(got["distanceToParent"], exp["distanceToParent"], rtol=1e-15, atol=0)
        assert got["leaf_names"] == exp["leaf_names"] and got["node_names"] == exp["node_names"]


def test_tokens_and_features():
    for case in E["tokens"]:
        assert maf_batch.maf_tokens(case["seqs"]).tolist() == case["alignment"]
    with pytest.raises(IndexError):
        maf_batch.maf_tokens(["AC", "ACG"])
    cnt = Z["features_of_random_counts_in"]
    np.testing.assert_array_equal(maf_batch.counts_to_features(cnt, cnt.shape[2]), Z["features_of_random_counts_out"])


def test_scan_matches_reference_pass_one():
    kept, pruned, skipped = _scan()
    assert len(kept) == len(E["manifest"]) and skipped == len(E["blocks"]) - len(kept)
    for (g, species, aln, n_orig), meta in zip(kept, E["per_block"]):
        assert species == meta["species"] and n_orig == meta["n_species_original"]
        np.testing.assert_array_equal(aln, Z[f"expanded_{g:06d}"])
        assert aln.shape[1] == meta["length"]


def test_processing_order_and_diagnostics():
    kept, _, _ = _scan()
    order = [i for _, idx in maf_batch._group_order(kept) for i in idx]
    assert sorted(order) == list(range(len(kept)))
    assert [i for i in order if i < E["validate"]] == [d["block_idx"] for d in E["diagnostics"]]
    for d in E["diagnostics"]:
        g = d["block_idx"]
        got = maf_batch.validate_block(Z[f"features_{g:06d}"], d["n_species"], g)
        for k, v in got.items():
            np.testing.assert_allclose(v, d[k], rtol=1e-9, atol=1e-12, err_msg=k)


def test_pipeline_with_oracle_counts():
    """Pass 1 + the oracle's Counts (Steiner mask) + the feature layout give
    the reference pipeline's per-block features (FP32 rounding apart)."""
    kept, pruned, _ = _scan()
    model = oracle.hky85_diag(E["kappa"], np.asarray(E["pi"]))
    for g, species, aln, _ in kept:
        tr = pruned[tuple(sorted(species))]
        c = oracle.Counts(aln, oracle.Tree(tr["parentIndex"], tr["distanceToParent"]), model)
        got = maf_batch.counts_to_features(c, aln.shape[1])
        assert_cols(got.T, Z[f"features_{g:06d}"].T, 1e-6, f"block {g}")
