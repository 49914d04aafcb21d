"""Shape padding helpers (subby_gb300/padding.py) against the reference's
subby/jax/_utils.py outputs (tests/golden/padding.json, made by
make_padding_golden.py), and the host-side removal of the dummy leaves that
padded trees hang under the root.  CPU only."""
import json
import os

import numpy as np
import pytest

import subby_gb300 as sg
from subby_gb300.padding import strip_dummy_leaves

with open(os.path.join(os.path.dirname(__file__), "golden", "padding.json")) as f:
    G = json.load(f)


def test_geometric_bins():
    assert sg.GEOM_BINS == G["GEOM_BINS"]
    for n, b in G["geom"]:
        assert sg.pad_to_geom_bin(n) == b


def test_pad_alignment_tree_and_unpad():
    aln = np.array(G["alignment"], np.int32)
    for case in G["pad_alignment"]:
        kw = {k: (sg.pad_to_geom_bin if v == "geom" else v) for k, v in case["kw"].items()}
        p, C = sg.pad_alignment(aln, **kw)
        assert C == case["C"] and p.dtype == np.int32 and p.tolist() == case["out"]
    t = sg.Tree(np.array(G["tree"]["parentIndex"], np.int32), np.array(G["tree"]["distanceToParent"]))
    pt = sg.pad_tree(t, 12)
    assert pt.parentIndex.tolist() == G["pad_tree_12"]["parentIndex"]
    assert pt.distanceToParent.tolist() == G["pad_tree_12"]["distanceToParent"]
    assert sg.pad_tree(t, 5) is t
    b = G["pad_both"]
    ptree, paln, R, C = sg.pad_tree_and_alignment(t, np.array(b["alignment"], np.int32))
    assert (R, C) == (b["R"], b["C"]) and paln.tolist() == b["padded"]
    assert ptree.parentIndex.tolist() == b["parentIndex"]
    assert ptree.distanceToParent.tolist() == b["distanceToParent"]
    assert sg.unpad_columns(np.arange(24).reshape(2, 3, 4), 3).tolist() == G["unpad"]


def test_strip_dummy_leaves():
    torch = pytest.importorskip("torch")
    b = G["pad_both"]
    t = sg.Tree(np.array(G["tree"]["parentIndex"], np.int32), np.array(G["tree"]["distanceToParent"]))
    aln = np.array(b["alignment"], np.int32)
    big = sg.Tree(*[np.concatenate([x, y]) for x, y in zip(t, (np.zeros(4, np.int32), np.zeros(4)))])
    big_aln = np.concatenate([aln, np.full((4, 20), -1, np.int32)])
    big_aln[-2, 3] = 5                        # A + 1: still no data for A = 4
    for ptree, paln in [sg.pad_tree_and_alignment(t, aln)[:2], (big, big_aln)]:
        a, s = strip_dummy_leaves(paln, ptree, 4)
        assert s.parentIndex.tolist() == t.parentIndex.tolist()
        assert s.distanceToParent.tolist() == t.distanceToParent.tolist()
        np.testing.assert_array_equal(a, paln[:9])
        ta, ts = strip_dummy_leaves(torch.as_tensor(paln), sg.Tree(torch.as_tensor(ptree.parentIndex),
                                                                    torch.as_tensor(ptree.distanceToParent)), lambda: 4)
        assert ta.tolist() == paln[:9].tolist() and ts.parentIndex.tolist() == t.parentIndex.tolist()
    # untouched: a binary tree; a dummy with data (only the rows after it go); a dummy with a branch length
    a, s = strip_dummy_leaves(aln, t, lambda: 1 / 0)
    assert a is aln and s is t
    data = big_aln.copy()
    data[10, 0] = 2
    a, s = strip_dummy_leaves(data, big, 4)
    assert len(s.parentIndex) == 11 and a.shape[0] == 11
    far = sg.Tree(big.parentIndex, np.concatenate([t.distanceToParent, [0, 0, 0, 0.1]]))
    a, s = strip_dummy_leaves(big_aln, far, 4)
    assert s is far
    # the root keeps two children even when every child is a dummy
    star = sg.Tree(np.array([-1, 0, 0, 0, 0], np.int32), np.zeros(5))
    a, s = strip_dummy_leaves(np.full((5, 3), -1, np.int32), star, 4)
    assert s.parentIndex.tolist() == [-1, 0, 0] and a.shape == (3, 3)
