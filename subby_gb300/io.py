"""JSON requests: the reference's input specification (subby/io.py:20-183,
subby/schema.json) run through the GPU path.

``load_input(data)`` -> (alignment (R, C) int32, Tree, model, compute list);
``run(data)`` -> {"logLike", "counts", "dwellTimes", "rootProb"} as nested
lists, computed by one fused plan run; ``load_json`` / ``format_output`` as
in the reference.  Model specs: {"name": "jukes-cantor", "alphabetSize"},
{"name": "hky85", "kappa", "pi"}, {"name": "f81", "pi"}, or {"subRate",
"rootProb", "reversible": true / false / null (detailed-balance check)};
an optional "alphabet" lets the alignment be given as character strings or
a character matrix ('-' = gap, token A+1).
"""
from __future__ import annotations

import json

import numpy as np

from . import models
from .types import Tree


def _parse_model(spec):
    if "name" in spec:
        name = spec["name"].lower().replace("-", "").replace("_", "")
        alphabet = spec.get("alphabet")
        if name == "jukescantor":
            return models.jukes_cantor_model(int(spec["alphabetSize"])), alphabet
        if name == "hky85":
            return models.hky85_diag(float(spec["kappa"]), np.asarray(spec["pi"], dtype=np.float64)), alphabet
        if name == "f81":
            return models.f81_model(np.asarray(spec["pi"], dtype=np.float64)), alphabet
        raise ValueError(f"Unknown model name: {spec['name']}")
    if "subRate" in spec:
        m = models.model_from_rate_matrix(np.asarray(spec["subRate"], dtype=np.float64),
                                          np.asarray(spec["rootProb"], dtype=np.float64),
                                          reversible=spec.get("reversible"))
        return m, spec.get("alphabet")
    raise ValueError("Model spec must have 'name' (named model) or 'subRate' (rate matrix)")


def _char_rows(rows, alphabet, what):
    if alphabet is None:
        raise ValueError(f"Alphabet required when alignment uses {what}")
    idx = {ch: i for i, ch in enumerate(alphabet)}
    gap = len(alphabet) + 1
    C = len(rows[0])
    out = np.zeros((len(rows), C), dtype=np.int32)
    for r, row in enumerate(rows):
        if len(row) != C:
            raise ValueError(f"Row {r} has length {len(row)}, expected {C}")
        for c, ch in enumerate(row):
            if ch == "-":
                out[r, c] = gap
            elif ch in idx:
                out[r, c] = idx[ch]
            else:
                raise ValueError(f"Unknown character '{ch}' at row {r}, col {c}")
    return out


def _parse_alignment(raw, alphabet):
    if not raw:
        raise ValueError("Alignment is empty")
    first = raw[0]
    if isinstance(first, str):
        return _char_rows(raw, alphabet, "character strings")
    if isinstance(first, list):
        if first and isinstance(first[0], str):
            return _char_rows(raw, alphabet, "characters")
        return np.array(raw, dtype=np.int32)
    raise ValueError("Alignment must be a list of strings or a 2D integer array")


def load_input(data):
    model, alphabet = _parse_model(data["model"])
    t = data["tree"]
    tree = Tree(np.asarray(t["parentIndex"], dtype=np.int32), np.asarray(t["distanceToParent"], dtype=np.float64))
    alignment = _parse_alignment(data["alignment"], alphabet)
    return alignment, tree, model, data.get("compute", ["logLike", "counts", "rootProb"])


def run(data):
    """Outputs of one request, all from a single plan run."""
    from .api import get_plan
    alignment, tree, model, compute = load_input(data)
    want_counts = "counts" in compute
    res = get_plan(tree, model).run(alignment, loglike="logLike" in compute, counts=want_counts,
                                    rootprob="rootProb" in compute)
    out = {}
    if "logLike" in compute:
        out["logLike"] = res["logLike"].astype(np.float64).tolist()
    if want_counts:
        c = res["counts"].astype(np.float64)
        out["counts"] = c.tolist()
        out["dwellTimes"] = np.array([c[a, a, :] for a in range(c.shape[0])]).tolist()
    if "rootProb" in compute:
        out["rootProb"] = res["rootProb"].astype(np.float64).tolist()
    return out


def load_json(path_or_file):
    if isinstance(path_or_file, str):
        with open(path_or_file) as f:
            return json.load(f)
    return json.load(path_or_file)


def format_output(result, indent=2):
    return json.dumps(result, indent=indent)
