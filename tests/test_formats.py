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
