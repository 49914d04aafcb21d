"""Generate tests/golden/formats/formats.json from the REFERENCE front-end.

    python tests/golden/make_formats_golden.py [--reference /root/reference]

Runs the reference's own parsers (``subby.formats``: parse_newick,
parse_fasta, parse_stockholm, parse_maf, parse_strings, parse_dict,
combine_tree_alignment, detect_alphabet; sliding_windows,
all_column_ktuples, kmer_tokenize, codon_to_sense, split_paired_columns,
merge_paired_columns) and JSON request runner
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


def _err(fn, *a, **k):
    try:
        fn(*a, **k)
    except Exception as e:  # noqa: BLE001
        return f"{type(e).__name__}: {e}"
    return None


def _transforms(F):
    """k-mer, codon and paired-column transforms (subby/formats.py:628-1098)."""
    rng = np.random.default_rng(77)
    t = {"sliding": [], "ktuples": [], "kmer": [], "codon": [], "paired": []}
    for C, k, stride, offset, edge in [(10, 3, None, 0, "truncate"), (10, 3, None, 0, "pad"), (10, 4, 2, 1, "pad"),
                                       (5, 6, None, 0, "truncate"), (7, 2, 3, 0, "truncate"), (6, 2, 1, 2, "pad")]:
        t["sliding"].append({"args": [C, k, stride, offset, edge],
                             "out": F.sliding_windows(C, k, stride, offset, edge).tolist()})
    t["sliding_error"] = _err(F.sliding_windows, 10, 3, edge="wrap")
    for C, k, ordered in [(4, 2, True), (5, 3, False), (1, 2, True), (3, 1, False)]:
        t["ktuples"].append({"args": [C, k, ordered], "out": F.all_column_ktuples(C, k, ordered).tolist()})
    a4 = rng.integers(-1, 6, size=(5, 12))
    cases = [(a4, 4, 2, "any", None), (a4, 4, 3, "all", ["A", "C", "G", "T"]),
             (a4, 4, F.sliding_windows(12, 5, 3, 0, "pad"), "any", None),
             (a4, 4, F.sliding_windows(12, 5, 3, 0, "pad"), "all", None),
             (a4, 4, [[0, 11], [3, 3], [7, 1]], "all", list("ACGT")), (a4, 4, np.zeros((0, 2)), "any", list("AC")),
             (rng.integers(-1, 22, size=(4, 6)), 20, [[0, 1, 2], [5, 4, 3]], "any", None)]
    for aln, A, kt, mode, alpha in cases:
        r = F.kmer_tokenize(aln, A, kt, gap_mode=mode, alphabet=alpha)
        t["kmer"].append({"alignment": np.asarray(aln).tolist(), "A": A,
                          "k_or_tuples": kt if isinstance(kt, int) else np.asarray(kt).tolist(),
                          "k": int(r["index"].tuples.shape[1]),
                          "gap_mode": mode, "alphabet": alpha, "out": r["alignment"].tolist(), "A_kmer": r["A_kmer"],
                          "tuples": r["index"].tuples.tolist(), "repr": repr(r["index"]),
                          "labels": r.get("alphabet")})
    t["kmer_errors"] = [_err(F.kmer_tokenize, a4, 4, 5), _err(F.kmer_tokenize, a4, 4, [0, 1, 2]),
                        _err(F.kmer_tokenize, a4, 4, 2, gap_mode="some")]
    codon = rng.integers(-2, 68, size=(3, 40))
    t["codon"] = {"alignment": codon.tolist(), "out": F.codon_to_sense(codon)["alignment"].tolist(),
                  "out_A63": F.codon_to_sense(codon, A=63)["alignment"].tolist(),
                  "alphabet": F.codon_to_sense(codon)["alphabet"]}
    a20 = rng.integers(-1, 22, size=(4, 8))
    for pairs in ([(0, 3), (5, 2)], [], [(0, 1), (2, 3), (4, 5), (6, 7)], [(7, 0)]):
        sp = F.split_paired_columns(a20, pairs, A=20)
        P, S = len(pairs), len(sp["single_columns"])
        pp = np.round(rng.random((400, P)), 3)
        ss = np.round(rng.random((20, S)), 3)
        t["paired"].append({"alignment": a20.tolist(), "pairs": [list(p) for p in pairs],
                            "paired_alignment": sp["paired_alignment"].tolist(),
                            "singles_alignment": sp["singles_alignment"].tolist(),
                            "single_columns": sp["single_columns"], "A_paired": sp["A_paired"],
                            "paired_post": pp.tolist(), "singles_post": ss.tolist(),
                            "merged": F.merge_paired_columns(pp, ss, sp).tolist()})
    return t


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
    out["transforms"] = _transforms(F)
    with open(os.path.join(HERE, "formats", "formats.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote formats/formats.json")


if __name__ == "__main__":
    main()
