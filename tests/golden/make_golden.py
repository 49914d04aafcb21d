"""Generate the golden fixtures under tests/golden/ from the REFERENCE oracle.

Run in a container where ihh/subby is mounted (default /root/reference):

    python tests/golden/make_golden.py [--reference /root/reference]

It imports the reference's own CPU oracle (``subby.oracle``, numpy + scipy)
and runs it on

* the inputs of the reference's golden files ``tests/golden/*.json``
  (5node_jc4, 7node_hky85_4, 7node_jc4_mixed_gaps, 7node_jc4_all_gaps,
  7node_jc64), and
* seeded synthetic cases of this repository (plain_small column subsets,
  legacy -1 gaps, F81 with non-uniform pi, zero-length branches, random
  reversible A=16 / A=20 models with near-degenerate eigenvalue pairs,
  irreversible A=4 / 8 / 16 models with complex eigenvalue pairs),

and writes one ``.npz`` per case holding the inputs, the reference oracle's
outputs (logLike, unmasked and Steiner-masked Counts, F81 fast-path Counts
where the model is F81/JC, per-branch counts for A <= 8, RootProb, node and
branch posteriors of InsideOutside, branch mask) and, for the small A=4 cases, its intermediates.  The fixtures travel with the repository; the
reference itself is never read by the GPU tests.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))


def _ref(path):
    sys.path.insert(0, path)
    import subby.oracle as oracle          # noqa: E402  (reference)
    from subby.formats import Tree         # noqa: E402  (reference)
    return oracle, Tree


def run_case(oracle, RTree, name, alignment, parent, dist, model, f81_ok,
             intermediates=False, masked=True):
    alignment = np.asarray(alignment, dtype=np.int32)
    parent = np.asarray(parent, dtype=np.int32)
    dist = np.asarray(dist, dtype=np.float64)
    if 'eigenvectors_inv' in model:
        # irreversible: complex eigensystem (subby/oracle/oracle.py:265-301)
        m = {k: np.asarray(model[k], dtype=np.complex128) for k in ('eigenvalues', 'eigenvectors',
                                                                   'eigenvectors_inv')}
        m['pi'] = np.asarray(model['pi'], dtype=np.float64)
        m['reversible'] = False
    else:
        m = {k: np.asarray(model[k], dtype=np.float64) for k in ('eigenvalues', 'eigenvectors', 'pi')}
    tree = RTree(parentIndex=parent, distanceToParent=dist)
    A = len(m['pi'])
    out = dict(alignment=alignment, parentIndex=parent, distanceToParent=dist,
               eigenvalues=m['eigenvalues'], eigenvectors=m['eigenvectors'], pi=m['pi'],
               A=np.int64(A))
    if 'eigenvectors_inv' in m:
        out['eigenvectors_inv'] = m['eigenvectors_inv']
    out['logLike'] = oracle.LogLike(alignment, tree, m)
    out['counts'] = oracle.Counts(alignment, tree, m, branch_mask=None)
    if masked:
        out['counts_masked'] = oracle.Counts(alignment, tree, m, branch_mask="auto")
    if f81_ok:
        out['counts_f81'] = oracle.Counts(alignment, tree, m, f81_fast=True, branch_mask=None)
        if masked:
            out['counts_f81_masked'] = oracle.Counts(alignment, tree, m, f81_fast=True,
                                                     branch_mask="auto")
    if A <= 8:
        # per-branch outputs (the reference's loops are O(R C A^4): small A only)
        out['branch_counts'] = oracle.BranchCounts(alignment, tree, m, branch_mask=None)
        if masked:
            out['branch_counts_masked'] = oracle.BranchCounts(alignment, tree, m, branch_mask="auto")
        if f81_ok:
            out['branch_counts_f81'] = oracle.BranchCounts(alignment, tree, m, f81_fast=True, branch_mask=None)
    out['root_prob'] = oracle.RootProb(alignment, tree, m)
    # posteriors of InsideOutside (loops O(R C A^2))
    io = oracle.InsideOutside(alignment, tree, m)
    out['node_posterior'] = io.node_posterior()
    out['branch_posterior'] = io.branch_posterior()
    out['branch_mask'] = oracle.compute_branch_mask(alignment, parent, A)
    if intermediates:
        M = oracle.compute_sub_matrices(m, dist)
        U, lnU, lnL = oracle.upward_pass(alignment, tree, M, m['pi'])
        D, lnD = oracle.downward_pass(U, lnU, tree, M, m['pi'], alignment)
        J = oracle.compute_J(m['eigenvalues'], dist)
        Ut, Dt = oracle.eigenbasis_project(U, D, m)
        Ce = oracle.accumulate_C(Dt, Ut, J, lnU, lnD, lnL, parent)
        out.update(sub_matrices=M, U=U, logNormU=lnU, D=D, logNormD=lnD, J=J,
                   U_tilde=Ut, D_tilde=Dt, C_eigen=Ce)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"  {name}: R={len(parent)} C={alignment.shape[1]} A={A} -> {os.path.basename(path)}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    oracle, RTree = _ref(args.reference)
    from subby_gb300 import synth, models

    gdir = os.path.join(args.reference, "tests", "golden")
    for fname, f81_ok, inter in [("5node_jc4", True, True), ("7node_hky85_4", False, True),
                                 ("7node_jc4_mixed_gaps", True, True),
                                 ("7node_jc4_all_gaps", True, True), ("7node_jc64", True, False)]:
        with open(os.path.join(gdir, fname + ".json")) as f:
            inp = json.load(f)['inputs']
        run_case(oracle, RTree, "ref_" + fname, inp['alignment'], inp['parentIndex'],
                 inp['distanceToParent'], inp['model'], f81_ok, intermediates=inter,
                 masked=(fname != "7node_jc64"))

    # plain_small column subset (R=31, A=4 HKY85, 5% unobserved split A/A+1)
    w = synth.plain_small(seed=1, C=1024)
    sel = np.random.default_rng(11).choice(1024, size=96, replace=False)
    aln = w['alignment'][:, np.sort(sel)]
    mm = w['model']._asdict()
    run_case(oracle, RTree, "plain_small_sub96", aln, w['tree'].parentIndex,
             w['tree'].distanceToParent, mm, False)

    # legacy -1 gaps, observed internal tokens, an all-gap and an all-unobserved column
    rng = np.random.default_rng(12)
    tr = synth.random_tree(16, 0.1, rng)
    R = len(tr.parentIndex)
    aln = rng.integers(-1, 6, size=(R, 40)).astype(np.int32)
    aln[:, 0] = -1
    aln[:, 1] = 4
    aln[:, 2] = 5
    run_case(oracle, RTree, "legacy_gaps_hky", aln, tr.parentIndex, tr.distanceToParent,
             models.hky85_diag(3.0, [0.1, 0.4, 0.3, 0.2])._asdict(), False)

    # F81 non-uniform pi: fast path and general path on the same input
    rng = np.random.default_rng(13)
    tr = synth.random_tree(24, 0.2, rng)
    m = models.f81_model(rng.dirichlet(np.ones(4)))
    aln = synth.simulated_alignment(tr, m, 64, 0.1, rng)
    run_case(oracle, RTree, "f81_4", aln, tr.parentIndex, tr.distanceToParent, m._asdict(), True)

    # zero-length branches
    rng = np.random.default_rng(14)
    tr = synth.random_tree(10, 0.1, rng)
    d = tr.distanceToParent.copy()
    d[3] = 0.0
    d[len(d) - 1] = 0.0
    m = models.hky85_diag(2.0, [0.25, 0.25, 0.3, 0.2])
    aln = synth.simulated_alignment(tr, m, 32, 0.1, rng)
    run_case(oracle, RTree, "zero_branch_hky", aln, tr.parentIndex, d, m._asdict(), False)

    # random reversible A=16 and A=20 with near-degenerate eigenvalue pairs
    for A, L, C, seed in [(16, 8, 8, 15), (20, 6, 5, 16)]:
        rng = np.random.default_rng(seed)
        m, _, _, _ = models.near_degenerate_reversible(A, rng, target_fraction=0.08)
        tr = synth.random_tree(L, 0.1, rng)
        aln = synth.simulated_alignment(tr, m, C, 0.1, rng)
        run_case(oracle, RTree, f"reversible_{A}", aln, tr.parentIndex, tr.distanceToParent,
                 m._asdict(), False)

    # irreversible models with complex eigenvalue pairs (cyclic rate
    # component), A = 4, 8 and 16; gaps and unobserved cells included
    for A, L, C, seed in [(4, 8, 24, 17), (8, 6, 10, 18), (16, 5, 4, 19)]:
        rng = np.random.default_rng(seed)
        m = models.random_irreversible(A, rng)
        tr = synth.random_tree(L, 0.2, rng)
        R = len(tr.parentIndex)
        aln = rng.integers(0, A + 2, size=(R, C)).astype(np.int32)
        aln[:, 0] = A + 1
        run_case(oracle, RTree, f"irrev_{A}", aln, tr.parentIndex, tr.distanceToParent,
                 m._asdict(), False)

    # mixtures of rate-scaled models (subby/oracle/oracle.py:208-262, 1334-1365,
    # 1598-1615): the reference's 7node_mixture_jc4 inputs and a discrete-gamma
    # HKY85 case; written to golden/mixture/ (not a single-model case)
    mdir = os.path.join(HERE, "mixture")
    os.makedirs(mdir, exist_ok=True)
    with open(os.path.join(gdir, "7node_mixture_jc4.json")) as f:
        inp = json.load(f)['inputs']
    cases = [("ref_7node_mixture_jc4", np.asarray(inp['alignment'], np.int32), np.asarray(inp['parentIndex']),
              np.asarray(inp['distanceToParent']), {k: np.asarray(v, np.float64) for k, v in inp['base_model'].items()},
              np.asarray(inp['rates'], np.float64), np.asarray(inp['log_weights'], np.float64))]
    rng = np.random.default_rng(21)
    tr = synth.random_tree(12, 0.2, rng)
    base = models.hky85_diag(2.5, [0.3, 0.2, 0.2, 0.3])
    rates, weights = oracle.gamma_rate_categories(0.5, 4)
    aln = synth.simulated_alignment(tr, base, 48, 0.1, rng)
    cases.append(("gamma4_hky", aln, tr.parentIndex, tr.distanceToParent, base._asdict(), np.asarray(rates),
                  np.log(np.asarray(weights))))
    for name, aln, parent, dist, bm, rates, lw in cases:
        tree = RTree(parentIndex=np.asarray(parent, np.int32), distanceToParent=np.asarray(dist, np.float64))
        bm = {k: np.asarray(bm[k], np.float64) for k in ('eigenvalues', 'eigenvectors', 'pi')}
        ms = [oracle.scale_model(bm, r) for r in rates]
        ll = np.stack([oracle.LogLike(aln, tree, m) for m in ms])
        post = oracle.MixturePosterior(aln, tree, ms, lw)
        np.savez_compressed(os.path.join(mdir, name + ".npz"), alignment=aln, parentIndex=np.asarray(parent, np.int32),
                            distanceToParent=np.asarray(dist, np.float64), rates=rates, log_weights=lw,
                            log_likes=ll, posteriors=post, **bm)
        print(f"  mixture/{name}: K={len(rates)} C={aln.shape[1]}")
    g_rates, g_w = oracle.gamma_rate_categories(0.5, 4)
    np.savez_compressed(os.path.join(mdir, "gamma_categories.npz"), alpha=np.array([0.5, 1.0, 2.0]),
                        rates=np.stack([oracle.gamma_rate_categories(a, 4)[0] for a in (0.5, 1.0, 2.0)]),
                        weights=g_w)


if __name__ == "__main__":
    main()
