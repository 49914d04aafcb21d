"""Generate tests/golden/padding.json from the REFERENCE padding helpers.

    python tests/golden/make_padding_golden.py [--reference /root/reference]

Runs subby/jax/_utils.py's GEOM_BINS, pad_to_geom_bin, pad_alignment,
pad_tree, pad_tree_and_alignment and unpad_columns on small inputs.  jax is
not installed here: ``jax.numpy`` is numpy for the duration (these helpers
only build arrays), and the module is loaded from its file with the
reference package around it.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    import subby  # noqa: F401  (reference package, for the relative import of subby.formats)
    jax = types.ModuleType("jax")
    jax.numpy = np
    sys.modules.update({"jax": jax, "jax.numpy": np})
    pkg = types.ModuleType("subby.jax")
    pkg.__path__ = [os.path.join(args.reference, "subby", "jax")]
    sys.modules["subby.jax"] = pkg
    spec = importlib.util.spec_from_file_location("subby.jax._utils",
                                                  os.path.join(args.reference, "subby", "jax", "_utils.py"))
    U = importlib.util.module_from_spec(spec)
    sys.modules["subby.jax._utils"] = U
    spec.loader.exec_module(U)
    from subby.formats import Tree

    out = {"GEOM_BINS": list(U.GEOM_BINS)}
    ns = [1, 2, 3, 5, 6, 9, 100, 129, 255, 1000, 4097, 10 ** 6, 10 ** 9, 10 ** 10]
    out["geom"] = [[n, int(U.pad_to_geom_bin(n))] for n in ns]
    rng = np.random.default_rng(8)
    aln = rng.integers(-1, 6, size=(5, 7)).astype(np.int32)
    out["alignment"] = aln.tolist()
    out["pad_alignment"] = []
    for kw in ({}, {"bin_size": 4}, {"bin_size": 7}, {"bin_fn": U.pad_to_geom_bin}):
        p, c = U.pad_alignment(aln, **kw)
        out["pad_alignment"].append({"kw": {k: (v if not callable(v) else "geom") for k, v in kw.items()},
                                     "out": np.asarray(p).tolist(), "C": int(c)})
    tree = Tree(parentIndex=np.array([-1, 0, 0, 1, 1, 2, 2, 3, 3], np.int32),
                distanceToParent=np.array([0.0, 0.1, 0.2, 0.3, 0.05, 0.15, 0.25, 0.12, 0.07]))
    pt = U.pad_tree(tree, 12)
    out["tree"] = {"parentIndex": tree.parentIndex.tolist(), "distanceToParent": tree.distanceToParent.tolist()}
    out["pad_tree_12"] = {"parentIndex": np.asarray(pt.parentIndex).tolist(),
                          "distanceToParent": np.asarray(pt.distanceToParent).tolist()}
    a9 = rng.integers(0, 4, size=(9, 20)).astype(np.int32)
    ptree, paln, R, C = U.pad_tree_and_alignment(tree, a9)
    out["pad_both"] = {"alignment": a9.tolist(), "parentIndex": np.asarray(ptree.parentIndex).tolist(),
                       "distanceToParent": np.asarray(ptree.distanceToParent).tolist(),
                       "padded": np.asarray(paln).tolist(), "R": int(R), "C": int(C)}
    out["unpad"] = np.asarray(U.unpad_columns(np.arange(24).reshape(2, 3, 4), 3)).tolist()
    with open(os.path.join(HERE, "padding.json"), "w") as f:
        json.dump(out, f)
    print("wrote padding.json")


if __name__ == "__main__":
    main()
