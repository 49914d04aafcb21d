"""Generate tests/golden/maf/ from the REFERENCE MAF batch script.

    python tests/golden/make_maf_golden.py [--reference /root/reference]

Writes a small synthetic MAF file (``blocks.maf``: ragged species sets,
excluded species, species missing from the guide tree, a duplicated
species, soft-masked bases, gaps, N and IUPAC codes, blocks below / at /
above the column limits, i/e/q lines) and a guide tree (``guide.nh``), then
runs the reference's own functions from scripts/batch_eigensub_maf.py on
them: ``iter_maf_blocks``, ``prune_tree``, ``_seqs_to_subby_alignment``,
``_expand_alignment_to_tree``, ``_counts_to_features``, ``validate_block``
and the whole ``precompute_maf_gpu`` (filters, pruning, grouping,
per-block feature files, manifest).  That script imports jax, which is not
installed here: ``jax``, ``jax.numpy`` and ``subby.jax`` are replaced by
small stand-ins (vmap as a loop, arrays as numpy) whose ``Counts`` is the
reference's FP64 oracle ``subby.oracle.Counts`` — the same expected counts
as subby.jax computes.  Outputs: ``expected.json`` (parsed blocks, pruned
trees, tokens, manifest, per-block metadata, diagnostics) and
``expected.npz`` (expanded alignments and features per block).
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "maf")

GUIDE = ("((((sp01:0.01,sp02:0.012):0.005,sp03:0.02):0.01,sp04:0.03):0.04,\n"
         "(((sp05:0.08,sp06:0.09)anc56:0.1,sp07:0.15):0.05,((sp08:0.12,sp09:0.13):0.04,sp10:0.3):0.06):0.02)root;\n")
EXCLUDE = {"sp03"}
MIN_SPECIES, MIN_COLS, MAX_COLS, VALIDATE = 3, 10, 150, 3

# (species rows, length); "spXX" / "spYY" are not in the guide tree
ALL = [f"sp{i:02d}" for i in range(1, 11)]
BLOCKS = [
    (ALL, 60),
    (["sp01", "sp02", "sp04", "sp05"], 40),
    (["sp05", "sp04", "sp02", "sp01"], 25),          # same species set, other row order
    (["sp01", "sp03", "sp02"], 30),                  # two species left after exclusion
    (["sp01", "sp02", "sp04"], 5),                   # too short
    (["sp01", "sp02", "sp04"], 200),                 # too long
    (["sp05", "sp06", "sp07", "spXX"], 33),          # one species not in the tree
    (["spXX", "spYY", "sp01"], 22),                  # prunes to one leaf
    (ALL[::-1], 77),
    (["sp08", "sp09", "sp10", "sp05", "sp05"], 50),  # duplicated species
    (["sp05", "sp06", "sp08"], 18),                  # root collapses
    (["sp02", "sp06", "sp09", "sp10"], 150),         # at the column maximum
    (["sp01", "sp02", "sp04", "sp05"], 10),          # at the column minimum
    (["sp07", "sp08", "sp09"], 20),
]
PRUNE_SETS = [ALL, ["sp01", "sp02"], ["sp05", "sp06", "sp08"], ["sp01"], ["spXX"], ["sp01", "sp04", "sp10", "spXX"],
              ["sp03", "sp07", "sp09", "sp10"]]
TOKEN_CASES = [["ACGTN-.", "acgtn-.", "RYKMSWB"], ["AC", "G?"]]


def _maf_text(rng):
    lines = ["##maf version=1 scoring=none", "# synthetic blocks", ""]
    for b, (species, L) in enumerate(BLOCKS):
        lines.append(f"a score={1000 + 7 * b}.0")
        anc = rng.choice(list("ACGT"), size=L)
        for r, sp in enumerate(species):
            seq = anc.copy()
            mut = rng.random(L) < 0.15
            seq[mut] = rng.choice(list("ACGT"), size=int(mut.sum()))
            gap0 = int(rng.integers(0, L))
            seq[gap0:gap0 + int(rng.integers(0, 4))] = "-"
            seq[rng.random(L) < 0.03] = "N"
            if rng.random() < 0.5:
                s0 = int(rng.integers(0, L))
                seq[s0:s0 + 6] = np.char.lower(seq[s0:s0 + 6])
            if b == 0 and r == 2:
                seq[:3] = ["R", "Y", "."]
            text = "".join(seq)
            size = sum(ch not in "-." for ch in text)
            strand = "-" if (b + r) % 3 == 0 else "+"
            chrom = f"chr{1 + (r % 5)}" if not (b == 9 and r == 4) else "chr9_random"
            lines.append(f"s {sp}.{chrom} {100 * b + r} {size} {strand} {10000 + r} {text}")
            if r == 0:
                lines.append(f"i {sp}.{chrom} C 0 C 0")
        if b == 1:
            lines.append("e sp10.chr3 500 12 + 9000 I")
            lines.append("q sp01.chr1 " + "9" * L)
        if b != len(BLOCKS) - 1:
            lines.append("")
    return "\n".join(lines) + "\n"


def _stub_modules(ro):
    """Stand-ins for jax / subby.jax so the reference batch script imports
    without jax; Counts is the reference oracle's."""
    jax = types.ModuleType("jax")
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
    jax.devices = lambda: ["cpu"]
    jax.default_backend = lambda: "cpu"

    def vmap(f):
        def g(*xs):
            return np.stack([f(*[x[i] for x in xs]) for i in range(len(xs[0]))])
        return g
    jax.vmap = vmap
    jnp = types.ModuleType("jax.numpy")
    jnp.array = lambda x, dtype=None: np.asarray(x, dtype=dtype)
    jnp.float64 = np.float64
    jax.numpy = jnp
    sj = types.ModuleType("subby.jax")
    sj.Counts = lambda aln, tree, model, maxChunkSize=128, branch_mask="auto": ro.Counts(
        np.asarray(aln), tree, model, branch_mask=branch_mask)
    sj.pad_alignment = sj.unpad_columns = None
    sjm = types.ModuleType("subby.jax.models")
    sjm.hky85_diag = ro.hky85_diag
    sj.models = sjm
    sys.modules.update({"jax": jax, "jax.numpy": jnp, "subby.jax": sj, "subby.jax.models": sjm})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    from subby.oracle import oracle as ro   # noqa: E402  (reference)
    from subby import formats as F          # noqa: E402  (reference)
    _stub_modules(ro)
    spec = importlib.util.spec_from_file_location(
        "ref_batch_maf", os.path.join(args.reference, "scripts", "batch_eigensub_maf.py"))
    B = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(B)

    os.makedirs(OUT, exist_ok=True)
    rng = np.random.default_rng(2024)
    maf_path = os.path.join(OUT, "blocks.maf")
    with open(maf_path, "w") as f:
        f.write(_maf_text(rng))
    with open(os.path.join(OUT, "guide.nh"), "w") as f:
        f.write(GUIDE)
    guide = F.parse_newick("".join(GUIDE.split()))

    exp = {"exclude": sorted(EXCLUDE), "min_species": MIN_SPECIES, "min_cols": MIN_COLS, "max_cols": MAX_COLS,
           "validate": VALIDATE, "kappa": B.DEFAULT_KAPPA, "pi": list(B.DEFAULT_PI)}
    exp["blocks"] = list(B.iter_maf_blocks(maf_path))
    exp["prune"] = []
    for keep in PRUNE_SETS:
        p = B.prune_tree(guide, set(keep))
        exp["prune"].append({"keep": keep, "result": None if p is None else {
            "parentIndex": p["parentIndex"].tolist(), "distanceToParent": p["distanceToParent"].tolist(),
            "leaf_names": p["leaf_names"], "node_names": p["node_names"]}})
    exp["tokens"] = [{"seqs": s, "alignment": B._seqs_to_subby_alignment(s).tolist()} for s in TOKEN_CASES]
    arrays = {}
    cnt = np.random.default_rng(5).random((4, 4, 9)).astype(np.float32)
    arrays["features_of_random_counts_in"] = cnt
    arrays["features_of_random_counts_out"] = B._counts_to_features(cnt, 9)

    model = ro.hky85_diag(B.DEFAULT_KAPPA, np.asarray(B.DEFAULT_PI))
    with tempfile.TemporaryDirectory() as td:
        manifest = B.precompute_maf_gpu(maf_path, td, model, guide, exclude_species=set(EXCLUDE),
                                        min_species=MIN_SPECIES, min_cols=MIN_COLS, max_cols=MAX_COLS,
                                        validate_n=VALIDATE)
        exp["manifest"] = manifest
        exp["per_block"] = []
        for m in manifest:
            z = np.load(os.path.join(td, m["file"]))
            exp["per_block"].append({"species": z["species"].tolist(), "n_species": int(z["n_species"]),
                                     "n_species_original": int(z["n_species_original"]),
                                     "length": int(z["length"])})
            arrays[m["file"][:-4]] = z["features"]
        with open(os.path.join(td, "validation_diagnostics.json")) as f:
            exp["diagnostics"] = json.load(f)
    # pass 1 of the reference: the kept blocks' tree-expanded alignments
    kept = 0
    for blk in exp["blocks"]:
        L = len(blk["seqs"][0])
        keep = [i for i, sp in enumerate(blk["species"]) if sp not in EXCLUDE]
        if L < MIN_COLS or L > MAX_COLS or len(keep) < MIN_SPECIES:
            continue
        sp = [blk["species"][i] for i in keep]
        pr = B.prune_tree(guide, set(sp))
        if pr is None:
            continue
        arrays[f"expanded_{kept:06d}"] = B._expand_alignment_to_tree(
            B._seqs_to_subby_alignment([blk["seqs"][i] for i in keep]), sp, pr)
        kept += 1
    assert kept == len(exp["manifest"])
    with open(os.path.join(OUT, "expected.json"), "w") as f:
        json.dump(exp, f, indent=1)
    np.savez_compressed(os.path.join(OUT, "expected.npz"), **arrays)
    print(f"wrote {OUT}: {len(exp['blocks'])} blocks, {kept} kept")


if __name__ == "__main__":
    main()
