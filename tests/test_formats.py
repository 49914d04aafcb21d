"""Front-end parsers (subby_gb300.formats, subby_gb300.io) against the
reference's own front-end run on the same inputs
(tests/golden/formats/formats.json, made by make_formats_golden.py):
Newick, FASTA, Stockholm, MAF, strings, dicts, combine_tree_alignment,
detect_alphabet, the error messages, and JSON request parsing.  CPU only;
the device tokeniser and request execution are in test_gpu_front.py."""
import json
import os

import numpy as np
import pytest

from subby_gb300 import formats, io

with open(os.path.join(os.path.dirname(__file__), "golden", "formats", "formats.json")) as f:
    G = json.load(f)


@pytest.mark.parametrize("case", G["newick"], ids=lambda c: c["input"][:20])
def test_newick(case):
    r = formats.parse_newick(case["input"])
    assert r["parentIndex"].tolist() == case["parentIndex"]
    np.testing.assert_array_equal(r["distanceToParent"], case["distanceToParent"])
    assert r["leaf_names"] == case["leaf_names"] and r["node_names"] == case["node_names"]


@pytest.mark.parametrize("kind,fn", [("fasta", formats.parse_fasta), ("stockholm", formats.parse_stockholm),
                                     ("maf", formats.parse_maf), ("strings", formats.parse_strings),
                                     ("dict", formats.parse_dict)])
def test_alignment_parsers(kind, fn):
    for case in G[kind]:
        r = fn(case["input"])
        exp = case["output"]
        assert r["alignment"].dtype == np.int32
        assert r["alignment"].tolist() == exp["alignment"]
        assert r["alphabet"] == exp["alphabet"]
        if "leaf_names" in exp:
            assert r["leaf_names"] == exp["leaf_names"]


@pytest.mark.parametrize("case", G["errors"], ids=lambda c: c["kind"])
def test_errors(case):
    fn = {"fasta": formats.parse_fasta, "strings": formats.parse_strings, "newick": formats.parse_newick}[case["kind"]]
    if case["error"] is None:
        fn(case["input"]) if case["kind"] == "newick" else fn(case["input"], case["alphabet"])
        return
    etype, msg = case["error"].split(": ", 1)
    with pytest.raises(Exception) as ei:
        fn(case["input"]) if case["kind"] == "newick" else fn(case["input"], case["alphabet"])
    assert type(ei.value).__name__ == etype
    assert str(ei.value) == msg


def test_combine_and_detect():
    c = G["combine"][0]
    r = formats.combine_tree_alignment(formats.parse_newick(c["newick"]), formats.parse_dict(c["sequences"]))
    assert r.alignment.tolist() == c["alignment"]
    assert r.alphabet == c["alphabet"] and r.leaf_names == c["leaf_names"]
    for d in G["detect"]:
        assert formats.detect_alphabet(set(d["chars"])) == d["alphabet"]


def test_deep_newick_no_recursion_limit():
    depth = 5000
    s = "(" * depth + "a" + "".join(f",b{i})" for i in range(depth)) + ";"
    r = formats.parse_newick(s)
    assert len(r["parentIndex"]) == 2 * depth + 1


def test_request_parsing():
    for case in G["requests"]:
        aln, tree, model, compute = io.load_input(case["request"])
        assert aln.dtype == np.int32 and aln.shape[0] == len(tree.parentIndex)
        assert compute == case["request"].get("compute", ["logLike", "counts", "rootProb"])
    m, _ = io._parse_model(G["requests"][2]["request"]["model"])
    assert type(m).__name__ == "IrrevDiagModel"   # random rate matrix: detailed balance fails



def test_command_line_validate(tmp_path):
    """``python -m subby_gb300 --validate``: exit 0 and "Valid." for a good
    request, exit 1 and "Invalid: <reason>" for a bad one (subby/__main__.py)."""
    import subprocess
    import sys
    good = tmp_path / "good.json"
    good.write_text(json.dumps(G["requests"][0]["request"]))
    bad = tmp_path / "bad.json"
    bad.write_text(json.dumps(dict(G["requests"][0]["request"], model={"name": "wag"})))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-m", "subby_gb300", str(good), "--validate"], capture_output=True,
                       text=True, cwd=root)
    assert r.returncode == 0 and r.stderr.strip() == "Valid."
    r = subprocess.run([sys.executable, "-m", "subby_gb300", "--validate"], input=bad.read_text(),
                       capture_output=True, text=True, cwd=root)
    assert r.returncode == 1 and r.stderr.strip() == "Invalid: Unknown model name: wag"


T = G["transforms"]


def test_sliding_windows_and_ktuples():
    for c in T["sliding"]:
        got = formats.sliding_windows(*c["args"])
        assert got.dtype == np.int64 and got.shape[1] == c["args"][1] and got.tolist() == c["out"]
    with pytest.raises(ValueError) as ei:
        formats.sliding_windows(10, 3, edge="wrap")
    assert f"ValueError: {ei.value}" == T["sliding_error"]
    for c in T["ktuples"]:
        got = formats.all_column_ktuples(*c["args"])
        assert got.dtype == np.int64 and got.shape[1] == c["args"][1] and got.tolist() == c["out"]


def test_kmer_tokenize():
    for c in T["kmer"]:
        kt = c["k_or_tuples"]
        kt = kt if isinstance(kt, int) else np.array(kt, dtype=np.int64).reshape(-1, c["k"])
        r = formats.kmer_tokenize(np.array(c["alignment"]), c["A"], kt,
                                  gap_mode=c["gap_mode"], alphabet=c["alphabet"])
        assert r["alignment"].dtype == np.int32 and r["alignment"].tolist() == c["out"]
        assert r["A_kmer"] == c["A_kmer"] and r["index"].tuples.tolist() == c["tuples"]
        assert repr(r["index"]) == c["repr"] and r.get("alphabet") == c["labels"]
        for i, t in enumerate(c["tuples"]):
            assert r["index"].tuple_to_idx(t) == i and list(r["index"].idx_to_tuple(i)) == t
        assert r["index"].tuple_to_idx((99, 98)) == -1
    a = np.array(T["kmer"][0]["alignment"])
    for args, kw, exp in zip(([a, 4, 5], [a, 4, [0, 1, 2]], [a, 4, 2]), ({}, {}, {"gap_mode": "some"}),
                             T["kmer_errors"]):
        with pytest.raises(ValueError) as ei:
            formats.kmer_tokenize(*args, **kw)
        assert f"ValueError: {ei.value}" == exp


def test_codon_to_sense_and_genetic_code():
    c = T["codon"]
    aln = np.array(c["alignment"])
    r = formats.codon_to_sense(aln)
    assert r["alignment"].tolist() == c["out"] and r["A_sense"] == 61 and r["alphabet"] == c["alphabet"]
    assert formats.codon_to_sense(aln, A=63)["alignment"].tolist() == c["out_A63"]
    gc = formats.genetic_code()
    assert len(gc["sense_codons"]) == 61 and [gc["codons"][i] for i in (48, 50, 56)] == ["TAA", "TAG", "TGA"]
    assert gc["amino_acids"][gc["codons"].index("ATG")] == "M" and gc["sense_codons"] == c["alphabet"]


def test_split_and_merge_paired_columns():
    for c in T["paired"]:
        pairs = [tuple(p) for p in c["pairs"]]
        sp = formats.split_paired_columns(np.array(c["alignment"]), pairs, A=20)
        assert sp["paired_alignment"].tolist() == c["paired_alignment"]
        assert sp["singles_alignment"].tolist() == c["singles_alignment"]
        assert sp["single_columns"] == c["single_columns"] and sp["A_paired"] == c["A_paired"]
        merged = formats.merge_paired_columns(np.array(c["paired_post"]).reshape(400, -1),
                                              np.array(c["singles_post"]).reshape(20, -1), sp)
        np.testing.assert_allclose(merged, np.array(c["merged"]).reshape(20, -1), rtol=1e-14, atol=0)


def test_request_field_parsing():
    """The request fields as the reference's tests/test_cli.py checks them:
    integer and character alignments, '-' -> A + 1, the missing-alphabet and
    model-spec errors."""
    acgt = ["A", "C", "G", "T"]
    a = io._parse_alignment([[0, 1], [2, 3]], None)
    assert a.dtype == np.int32 and a.shape == (2, 2)
    assert io._parse_alignment(["AC", "GT"], acgt).tolist() == [[0, 1], [2, 3]]
    assert io._parse_alignment(["A-", "GT"], acgt)[0, 1] == 5
    assert io._parse_alignment([["A", "C"], ["G", "T"]], acgt).tolist() == [[0, 1], [2, 3]]
    with pytest.raises(ValueError, match="Alphabet required"):
        io._parse_alignment(["AC", "GT"], None)
    with pytest.raises(ValueError, match="Unknown model"):
        io._parse_model({"name": "bogus", "alphabetSize": 4})
    with pytest.raises(ValueError, match="must have"):
        io._parse_model({"alphabet": ["A", "C"]})
    m, alpha = io._parse_model({"name": "hky85", "kappa": 2.0, "pi": [0.3, 0.2, 0.2, 0.3]})
    assert alpha is None and np.allclose(m.pi, [0.3, 0.2, 0.2, 0.3])
