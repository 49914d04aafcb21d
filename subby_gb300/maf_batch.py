"""MAF batch pipeline: per-block substitution features from a multiple
alignment (MAF) file and a guide tree, computed on the GPU.

Mirrors the reference's batch script (scripts/batch_eigensub_maf.py) —
same inputs, filters, tree pruning, token mapping, feature layout and
output files:

* ``iter_maf_blocks`` (:67-119): one block per 'a' line, its 's' lines as
  rows (species = source name up to the first '.'); plain or gzip text.
* ``maf_tokens`` (:127-158): A/C/G/T (either case) -> 0..3, N -> A,
  '-' / '.' -> A + 1, any other character -> A (unobserved, not an error).
* ``prune_tree`` (:161-253): the guide tree restricted to the kept leaves,
  single-child internal nodes collapsed (branch lengths summed), preorder
  renumbered; None below two leaves.
* ``expand_to_tree`` (:256-293): alignment rows placed at their leaves,
  every other node the gap token 5.
* ``counts_to_features`` (:311-323): (L, 20) = the 16 counts c[i, j]
  row-major, then the 4 dwell times c[i, i].
* ``validate_block`` (:326-380): the script's sanity statistics.
* ``precompute_maf`` (:423-693): filters (columns in [min_cols, max_cols],
  excluded species, at least min_species rows, a pruned tree), Counts with
  the Steiner branch mask, ``features_NNNNNN.npz`` per kept block (features,
  species, n_species, n_species_original, length), the manifest, and
  ``validation_diagnostics.json`` for the first ``validate_n`` blocks.
  ``main`` is the same command line (:701-798).

GB300 design.  The reference pads groups of blocks to 128-column bins and
vmaps Counts over stacks of groups that share a node count.  Here each
distinct species set (which fixes the pruned tree) has one resident plan
(cached), the columns of all its blocks are concatenated and run by one
fused Counts call, with no padding; columns are independent, so each block
gets exactly its own counts.  Blocks are processed in the reference's order
(buckets by node count, most blocks first; groups by column count), so the
diagnostics come out in the same order too.
"""
from __future__ import annotations

import argparse
import gzip
import json
import os
import time
from collections import OrderedDict

import numpy as np

GAP_TOKEN = 5
DEFAULT_KAPPA = 4.0
DEFAULT_PI = [0.295, 0.205, 0.205, 0.295]


def iter_maf_blocks(maf_path: str):
    """Blocks of a MAF file as dicts: species, seqs, srcs, starts, sizes,
    strands, src_sizes (one entry per 's' line).  ``.gz`` paths are read
    through gzip.  Lines other than 'a' and 's' lines are ignored."""
    opener = gzip.open if maf_path.endswith(".gz") else open
    keys = ("species", "seqs", "srcs", "starts", "sizes", "strands", "src_sizes")
    block = None
    with opener(maf_path, "rt") as f:
        for line in f:
            line = line.rstrip("\n\r")
            if line.startswith("a"):
                if block is not None and block["species"]:
                    yield block
                block = {k: [] for k in keys}
            elif line.startswith("s") and block is not None:
                _, src, start, size, strand, src_size, seq = line.split()[:7]
                block["species"].append(src.split(".")[0])
                block["seqs"].append(seq)
                block["srcs"].append(src)
                block["starts"].append(int(start))
                block["sizes"].append(int(size))
                block["strands"].append(strand)
                block["src_sizes"].append(int(src_size))
    if block is not None and block["species"]:
        yield block


def _token_table(A: int) -> np.ndarray:
    t = np.full(256, A, dtype=np.int32)
    for i, ch in enumerate("ACGT"):
        t[ord(ch)] = t[ord(ch.lower())] = i
    t[ord("N")] = t[ord("n")] = A
    t[ord("-")] = t[ord(".")] = A + 1
    return t


def maf_tokens(seqs, alphabet_size: int = 4) -> np.ndarray:
    """(R, C) int32 tokens of aligned sequence strings, C = the first
    sequence's length; a shorter row is gap-filled, a longer one raises
    IndexError (as the reference's element-wise fill does)."""
    A = int(alphabet_size)
    table = _token_table(A)
    R, C = len(seqs), len(seqs[0])
    out = np.full((R, C), A + 1, dtype=np.int32)
    for r, s in enumerate(seqs):
        if len(s) > C:
            raise IndexError(f"index {C} is out of bounds for axis 1 with size {C}")
        b = np.frombuffer(s.encode("latin-1", errors="replace"), dtype=np.uint8)
        out[r, :len(b)] = table[b]
    return out


def prune_tree(tree_data: dict, keep_leaves) -> dict | None:
    """The guide tree (a parse_newick dict, node 0 the root) restricted to
    the leaves named in ``keep_leaves``: unary internal nodes are collapsed
    into their child (lengths added; a collapsed root's length is dropped),
    nodes renumbered in preorder (children in index order).  Returns the
    same keys (parentIndex, distanceToParent, leaf_names, node_names), or
    None when fewer than two leaves remain."""
    parent = np.asarray(tree_data["parentIndex"])
    dist = np.asarray(tree_data["distanceToParent"], dtype=np.float64)
    names = tree_data["node_names"]
    R = len(parent)
    kids = [[] for _ in range(R)]
    for i in range(1, R):
        kids[int(parent[i])].append(i)
    keep = np.zeros(R, dtype=bool)
    order, stack = [], [0]
    while stack:                       # preorder from the root
        n = stack.pop()
        order.append(n)
        stack.extend(reversed(kids[n]))
    for n in reversed(order):          # children before parents
        keep[n] = (names[n] in keep_leaves) if not kids[n] else any(keep[c] for c in kids[n])
    if not keep[0]:
        return None
    new_parent, new_dist, new_names, leaves = [], [], [], []
    stack = [(0, -1, 0.0)]
    while stack:
        n, p, extra = stack.pop()
        live = [c for c in kids[n] if keep[c]]
        total = dist[n] + extra
        if kids[n] and len(live) == 1:
            stack.append((live[0], p, total))
            continue
        idx = len(new_parent)
        new_parent.append(p)
        new_dist.append(total if p >= 0 else 0.0)
        new_names.append(names[n])
        if not kids[n]:
            leaves.append(names[n])
        stack.extend((c, idx, 0.0) for c in reversed(live))
    if len(leaves) < 2:
        return None
    return {"parentIndex": np.array(new_parent, dtype=np.int32),
            "distanceToParent": np.array(new_dist, dtype=np.float64),
            "leaf_names": leaves, "node_names": new_names}


def expand_to_tree(alignment: np.ndarray, species, pruned: dict) -> np.ndarray:
    """(nodes, L) int32: the row of each leaf's species (the last row when a
    species repeats), the gap token 5 at internal nodes and at leaves
    without a row."""
    parent = np.asarray(pruned["parentIndex"])
    n = len(parent)
    out = np.full((n, alignment.shape[1]), GAP_TOKEN, dtype=np.int32)
    row = {sp: i for i, sp in enumerate(species)}
    internal = np.zeros(n, dtype=bool)
    internal[parent[1:]] = True
    for i in np.flatnonzero(~internal):
        r = row.get(pruned["node_names"][i])
        if r is not None:
            out[i] = alignment[r]
    return out


def counts_to_features(counts: np.ndarray, L: int) -> np.ndarray:
    """(A, A, L) counts -> (L, A*A + A): counts[i, j] row-major, then the
    dwell times counts[i, i]."""
    c = np.asarray(counts)
    A = c.shape[0]
    per_col = np.moveaxis(c, 2, 0)
    return np.concatenate([per_col.reshape(L, A * A), per_col[:, np.arange(A), np.arange(A)]], axis=1)


def validate_block(features: np.ndarray, n_species: int, block_idx: int) -> dict:
    """Sanity statistics of one block's (L, 20) features: mean count matrix,
    symmetry ratio (mean of the strict upper triangle's entries over the
    strict lower triangle's, each in np.triu_indices / np.tril_indices order,
    as the reference pairs them), dwell per column, Ti/Tv ratio, coefficient
    of variation of the per-column substitution totals, and the
    dominant-base dwell share in the lowest-quartile (conserved) columns."""
    L = features.shape[0]
    trans = features[:, :16].reshape(L, 4, 4)
    dwell = features[:, 16:]
    mean = trans.mean(axis=0)
    iu, il = np.triu_indices(4, 1), np.tril_indices(4, -1)
    sym = (mean[iu] / np.maximum(mean[il], 1e-10)).mean()
    ti = mean[0, 2] + mean[2, 0] + mean[1, 3] + mean[3, 1]                  # A<->G, C<->T
    tv = (mean[0, 1] + mean[1, 0] + mean[0, 3] + mean[3, 0]                 # A<->C, A<->T,
          + mean[2, 1] + mean[1, 2] + mean[2, 3] + mean[3, 2])              # G<->C, G<->T
    tot = trans[:, ~np.eye(4, dtype=bool)].sum(axis=1)
    cons = tot < np.percentile(tot, 25)
    if cons.any():
        d = dwell[cons]
        dom = float((d.max(axis=1) / np.maximum(d.sum(axis=1), 1e-10)).mean())
    else:
        dom = float("nan")
    return {"block_idx": block_idx, "n_species": n_species, "n_cols": L, "mean_trans_matrix": mean.tolist(),
            "symmetry_ratio": float(sym), "total_dwell_per_col": float(dwell.sum(axis=1).mean()),
            "ti_tv_ratio": float(ti / max(tv, 1e-10)),
            "count_cv": float(tot.std() / max(tot.mean(), 1e-10)), "conserved_dominant_frac": dom,
            "total_counts_mean": float(tot.mean()), "total_counts_std": float(tot.std())}


def scan_blocks(maf_path: str, guide_tree: dict, exclude_species=None, min_species: int = 3,
                min_cols: int = 10, max_cols: int = 2048):
    """Pass 1: the kept blocks as (index, species, expanded alignment,
    species count before exclusion), numbered in file order, and the pruned
    tree of every species set (key: the sorted species tuple)."""
    exclude = set(exclude_species or ())
    pruned, kept, skipped = {}, [], 0
    for blk in iter_maf_blocks(maf_path):
        seqs = blk["seqs"]
        L = len(seqs[0]) if seqs else 0
        rows = [i for i, sp in enumerate(blk["species"]) if sp not in exclude]
        if L < min_cols or L > max_cols or len(rows) < min_species:
            skipped += 1
            continue
        species = [blk["species"][i] for i in rows]
        key = tuple(sorted(species))
        if key not in pruned:
            pruned[key] = prune_tree(guide_tree, set(species))
        if pruned[key] is None:
            skipped += 1
            continue
        aln = expand_to_tree(maf_tokens([seqs[i] for i in rows]), species, pruned[key])
        kept.append((len(kept), species, aln, len(blk["species"])))
    return kept, pruned, skipped


def _group_order(kept):
    """Species groups in the reference's processing order: buckets by node
    count, most blocks first (ties by first appearance); within a bucket,
    groups by concatenated column count (ties by first appearance)."""
    buckets = OrderedDict()
    for i, (_, species, aln, _) in enumerate(kept):
        buckets.setdefault(aln.shape[0], OrderedDict()).setdefault(tuple(sorted(species)), []).append(i)
    order = []
    for groups in sorted(buckets.values(), key=lambda g: -sum(len(v) for v in g.values())):
        order.extend(sorted(groups.items(), key=lambda kv: sum(kept[i][2].shape[1] for i in kv[1])))
    return order


def precompute_maf(maf_path: str, output_dir: str, model, guide_tree: dict, exclude_species=None,
                   min_species: int = 3, min_cols: int = 10, max_cols: int = 2048, validate_n: int = 0,
                   device=None, verbose: bool = True) -> list:
    """Features of every kept block of a MAF file, one fused Counts call per
    species set; writes ``features_NNNNNN.npz`` per block into output_dir
    (and ``validation_diagnostics.json`` when validate_n > 0) and returns
    the manifest (one entry per kept block, in file order)."""
    from .api import get_plan
    from .types import Tree
    os.makedirs(output_dir, exist_ok=True)
    t0 = time.time()
    kept, pruned, skipped = scan_blocks(maf_path, guide_tree, exclude_species, min_species, min_cols, max_cols)
    if verbose:
        print(f"  pass 1: {len(kept)} blocks kept, {skipped} skipped, {len(pruned)} species sets")
    manifest = [None] * len(kept)
    diagnostics = []
    cols = 0
    t1 = time.time()
    for key, idx in _group_order(kept):
        tr = pruned[key]
        plan = get_plan(Tree(tr["parentIndex"], tr["distanceToParent"]), model, device)
        lengths = [kept[i][2].shape[1] for i in idx]
        counts = plan.run(np.concatenate([kept[i][2] for i in idx], axis=1), loglike=False, counts=True,
                          branch_mask="auto")["counts"]
        off = 0
        for i, L in zip(idx, lengths):
            g, species, _, n_orig = kept[i]
            feats = counts_to_features(counts[:, :, off:off + L], L)
            off += L
            if g < validate_n:
                d = validate_block(feats, len(species), g)
                d["n_species_excluded"] = n_orig - len(species)
                diagnostics.append(d)
            name = f"features_{g:06d}.npz"
            np.savez_compressed(os.path.join(output_dir, name), features=feats, species=np.array(species),
                                n_species=len(species), n_species_original=n_orig, length=L)
            manifest[g] = {"file": name, "n_species": len(species), "n_species_original": n_orig, "length": L}
            cols += L
    if verbose:
        dt = time.time() - t1
        print(f"  pass 2: {len(kept)} blocks, {cols} columns in {dt:.2f} s "
              f"({cols / max(dt, 1e-9):.0f} columns/s; {time.time() - t0:.2f} s in all)")
    if diagnostics:
        with open(os.path.join(output_dir, "validation_diagnostics.json"), "w") as f:
            json.dump(diagnostics, f, indent=2)
    return manifest


def main(argv=None):
    from . import formats, models
    ap = argparse.ArgumentParser(description="Per-block substitution features of a MAF file on the GPU")
    ap.add_argument("maf_path")
    ap.add_argument("output_dir")
    ap.add_argument("--tree", required=True, help="Newick guide tree file")
    ap.add_argument("--exclude-species", default="", help="comma-separated species to leave out")
    ap.add_argument("--min-species", type=int, default=3)
    ap.add_argument("--min-cols", type=int, default=10)
    ap.add_argument("--max-cols", type=int, default=2048)
    ap.add_argument("--kappa", type=float, default=DEFAULT_KAPPA)
    ap.add_argument("--pi", default=None, help="A,C,G,T equilibrium frequencies")
    ap.add_argument("--validate", type=int, default=0, help="diagnostics for the first N blocks")
    a = ap.parse_args(argv)
    pi = DEFAULT_PI if a.pi is None else [float(x) for x in a.pi.split(",")]
    if len(pi) != 4 or abs(sum(pi) - 1.0) >= 0.01:
        raise SystemExit(f"--pi needs 4 values summing to 1, got {pi}")
    with open(a.tree) as f:
        guide = formats.parse_newick("".join(f.read().split()))
    exclude = set(a.exclude_species.split(",")) if a.exclude_species else set()
    t0 = time.time()
    manifest = precompute_maf(a.maf_path, a.output_dir, models.hky85_diag(a.kappa, np.asarray(pi)), guide,
                              exclude, a.min_species, a.min_cols, a.max_cols, a.validate)
    with open(os.path.join(a.output_dir, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=2)
    cols = sum(m["length"] for m in manifest)
    print(f"{len(manifest)} blocks, {cols} columns in {time.time() - t0:.1f} s -> {a.output_dir}")


if __name__ == "__main__":
    main()
