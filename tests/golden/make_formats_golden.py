"""Generate tests/golden/formats/formats.json from the REFERENCE front-end.

    python tests/golden/make_formats_golden.py [--reference /root/reference]

Runs the reference's own parsers (``subby.formats``: parse_newick,
parse_fasta, parse_stockholm, parse_maf, parse_strings, parse_dict,
combine_tree_alignment, detect_alphabet) and JSON request runner
(``subby.io.run``, FP64 oracle) on small synthetic inputs written here,
and stores inputs, outputs and error messages as JSON.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

NEWICK = [
    "((A:0.1,B:0.2):0.3,(C:0.4,D:0.5)E:0.6)root;",
    "(('a b':1,'it''s':2)[a comment]:3,c:4);",
    "((A,B),(C,(D,E)));",
    "((x:1e-2,y:2.5E-1):0.125,z:7);",
    "A;",
]
FASTA = [
    ">s1 first\nACGT-A\n>s2\nacgt..\n>s3\nAC\nGTAA\n",
    ">p1\nMKV-LA\n>p2\nmkvwla\n",
    ">r1\nACGU\n>r2\nAC-U\n",
]
STOCKHOLM = ["# STOCKHOLM 1.0\n#=GF ID test\nseqA ACG-T\nseqB ACGAT\n\nseqA TTA\nseqB TTC\n//\n"]
MAF = ["##maf version=1\na score=1\ns hg38.chr1 10 5 + 1000 ACGTA\ns mm10.chr2 20 5 + 900 ACG-A\n\n"
       "a score=2\ns hg38.chr1 30 3 + 1000 TTG\ns rn6.chr3 5 3 - 800 TAG\n"]
STRINGS = [["ACGT", "AC-T", "acgt"], ["ACDE", "FGHI"]]
DICTS = [{"human": "ACGTT", "mouse": "AC.TT", "rat": "ACGTA"}]
BAD = [("fasta", ">a\nACGX\n>b\nACGT\n", ["A", "C", "G", "T"]), ("fasta", ">a\nACG\n>b\nACGT\n", None),
       ("strings", ["ACGJ", "ACGT"], ["A", "C", "G", "T"]), ("newick", "((A,B);", None), ("newick", "", None)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    from subby import formats as F   # noqa: E402  (reference)
    from subby import io as IO       # noqa: E402  (reference)

    def aln_out(d):
        return {k: (np.asarray(v).tolist() if k == "alignment" else v) for k, v in d.items()}

    out = {"newick": [], "fasta": [], "stockholm": [], "maf": [], "strings": [], "dict": [], "errors": [],
           "combine": [], "detect": [], "requests": []}
    for s in NEWICK:
        r = F.parse_newick(s)
        out["newick"].append({"input": s, "parentIndex": r["parentIndex"].tolist(),
                              "distanceToParent": r["distanceToParent"].tolist(),
                              "leaf_names": r["leaf_names"], "node_names": r["node_names"]})
    for s in FASTA:
        out["fasta"].append({"input": s, "output": aln_out(F.parse_fasta(s))})
    for s in STOCKHOLM:
        out["stockholm"].append({"input": s, "output": aln_out(F.parse_stockholm(s))})
    for s in MAF:
        out["maf"].append({"input": s, "output": aln_out(F.parse_maf(s))})
    for s in STRINGS:
        out["strings"].append({"input": s, "output": aln_out(F.parse_strings(s))})
    for s in DICTS:
        out["dict"].append({"input": s, "output": aln_out(F.parse_dict(s))})
    for kind, s, alpha in BAD:
        fn = {"fasta": F.parse_fasta, "strings": F.parse_strings, "newick": F.parse_newick}[kind]
        try:
            fn(s, alpha) if kind != "newick" else fn(s)
            msg = None
        except Exception as e:  # noqa: BLE001
            msg = f"{type(e).__name__}: {e}"
        out["errors"].append({"kind": kind, "input": s, "alphabet": alpha, "error": msg})
    t = F.parse_newick("((human:0.1,mouse:0.2):0.05,rat:0.3);")
    a = F.parse_dict({"rat": "ACG-T", "human": "ACGTT", "mouse": "AC.TA"})
    c = F.combine_tree_alignment(t, a)
    out["combine"].append({"newick": "((human:0.1,mouse:0.2):0.05,rat:0.3);",
                           "sequences": {"rat": "ACG-T", "human": "ACGTT", "mouse": "AC.TA"},
                           "alignment": c.alignment.tolist(), "alphabet": c.alphabet, "leaf_names": c.leaf_names})
    for chars in (["A", "C", "g"], ["A", "C", "G", "U"], ["M", "K", "V"], ["0", "1"]):
        out["detect"].append({"chars": chars, "alphabet": F.detect_alphabet(set(chars))})
    rng = np.random.default_rng(31)
    reqs = [
        {"model": {"name": "hky85", "kappa": 2.0, "pi": [0.1, 0.2, 0.3, 0.4], "alphabet": ["A", "C", "G", "T"]},
         "tree": {"parentIndex": [-1, 0, 0, 1, 1], "distanceToParent": [0.0, 0.1, 0.2, 0.15, 0.3]},
         "alignment": ["ACGTAC", "ACG-AC", "TTGTAC", "ACGTTC", "AAGTAG"]},
        {"model": {"name": "jukes-cantor", "alphabetSize": 4},
         "tree": {"parentIndex": [-1, 0, 0], "distanceToParent": [0.0, 0.3, 0.2]},
         "alignment": rng.integers(0, 6, size=(3, 8)).tolist(), "compute": ["logLike", "rootProb"]},
    ]
    Q = rng.uniform(0.1, 1.0, (4, 4))
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(1))
    reqs.append({"model": {"subRate": Q.tolist(), "rootProb": [0.25] * 4, "reversible": None},
                 "tree": {"parentIndex": [-1, 0, 0, 2, 2], "distanceToParent": [0.0, 0.2, 0.1, 0.3, 0.25]},
                 "alignment": rng.integers(0, 6, size=(5, 7)).tolist()})
    for r in reqs:
        out["requests"].append({"request": r, "result": IO.run(r)})
    with open(os.path.join(HERE, "formats", "formats.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote formats/formats.json")


if __name__ == "__main__":
    main()
