"""Front-end: alignment and tree text formats to the hot path's inputs.

Same names, arguments, return values and errors as subby/formats.py
(``detect_alphabet`` :37-60, ``parse_newick`` :150-225, ``parse_fasta``
:228-315, ``parse_stockholm`` :318-410, ``parse_maf`` :413-507,
``parse_strings`` :510-564, ``parse_dict`` :567-625,
``combine_tree_alignment`` :1101-1169).  Differences are in how, not what:

* characters are tokenised through a 256-entry lookup table over the raw
  bytes (numpy on the host; ``tokenize(..., device=...)`` runs the CUDA
  kernel ``subby_tokenize`` on a device byte buffer, so a large alignment
  crosses the host link as 1 byte per cell instead of 4);
* the Newick parser is iterative (no recursion limit on deep trees).

Token convention (subby/oracle/oracle.py:69-96): 0..A-1 the alphabet
(case-insensitive), A+1 for the gap characters '-' and '.', A for the
internal rows ``combine_tree_alignment`` adds.
"""
from __future__ import annotations

import ctypes as ct
from typing import NamedTuple

import numpy as np

from .types import Tree

_DNA = list("ACGT")
_RNA = list("ACGU")
_PROTEIN = list("ACDEFGHIKLMNPQRSTVWY")
_GAP_CHARS = {"-", "."}
_BAD = -1


class CombinedResult(NamedTuple):
    alignment: np.ndarray
    tree: Tree
    alphabet: list
    leaf_names: list


def detect_alphabet(chars):
    """DNA, RNA or protein when the (upper-cased, gap-free) characters fit,
    else the sorted characters."""
    upper = {ch.upper() for ch in chars} - _GAP_CHARS
    for alpha in (_DNA, _RNA, _PROTEIN):
        if upper <= set(alpha):
            return list(alpha)
    return sorted(upper)


# ---------------------------------------------------------------- tokenising
def lookup_table(alphabet, lowercase=True):
    """int32[256]: byte -> token (alphabet index; A+1 for '-' and '.'; -1
    for any other byte)."""
    lut = np.full(256, _BAD, dtype=np.int32)
    for i, ch in enumerate(alphabet):
        for c in ({ch, ch.lower()} if lowercase else {ch}):
            b = c.encode("latin-1")
            if len(b) == 1:
                lut[b[0]] = i
    for g in _GAP_CHARS:
        lut[ord(g)] = len(alphabet) + 1
    return lut


def _as_bytes(sequences, names=None):
    C = len(sequences[0])
    try:
        buf = np.frombuffer("".join(sequences).encode("latin-1"), dtype=np.uint8)
    except UnicodeEncodeError as e:
        # a character outside one byte is in no alphabet: report it as such
        _unknown(e.object[e.start], e.start // C, e.start % C, names)
    return buf.reshape(len(sequences), C)


def tokenize(chars, alphabet, device=None, names=None):
    """(N, C) uint8 characters -> (N, C) int32 tokens.  With ``device`` (or a
    CUDA uint8 tensor) the mapping runs on the GPU and the result stays
    there.  Unknown characters raise ValueError naming the first one."""
    lut = lookup_table(alphabet)
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    on_dev = torch is not None and (device is not None or (isinstance(chars, torch.Tensor) and chars.is_cuda))
    if not on_dev:
        chars = np.ascontiguousarray(np.asarray(chars, dtype=np.uint8))
        out = lut[chars]
        bad = np.argwhere(out == _BAD)
        if bad.size:
            r, c = (int(x) for x in bad[0])
            _unknown(chr(chars[r, c]), r, c, names)
        return out
    from . import _lib
    lib = _lib.load()
    dev = torch.device(device) if device is not None else chars.device
    src = torch.as_tensor(np.asarray(chars, dtype=np.uint8) if not isinstance(chars, torch.Tensor) else chars,
                          device=dev).to(torch.uint8).contiguous()
    if src.data_ptr() % 16:
        src = src.clone()     # the kernel reads 16-byte words
    dlut = torch.as_tensor(lut, device=dev)
    out = torch.empty(src.shape, dtype=torch.int32, device=dev)
    first_bad = torch.full((1,), -1, dtype=torch.int64, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    with torch.cuda.device(dev):
        _lib.check(lib.subby_tokenize(ct.c_void_p(src.data_ptr()), ct.c_int64(src.numel()),
                                      ct.c_void_p(dlut.data_ptr()), ct.c_void_p(out.data_ptr()),
                                      ct.c_void_p(first_bad.data_ptr()), ct.c_void_p(st)), "subby_tokenize")
    fb = int(first_bad.item())
    if fb >= 0:
        C = int(src.shape[-1])
        r, c = divmod(fb, C)
        _unknown(chr(int(src.reshape(-1)[fb].item())), r, c, names)
    return out


def _unknown(ch, r, c, names):
    if names is not None:
        raise ValueError(f"Unknown character '{ch}' in sequence '{names[r]}' at position {c}")
    raise ValueError(f"Unknown character '{ch}' at row {r}, col {c}")


def _encode(sequences, alphabet, names, empty_msg, unequal_msg, zero_msg):
    if not sequences:
        raise ValueError(empty_msg)
    lengths = {len(s) for s in sequences}
    if len(lengths) > 1:
        raise ValueError(f"{unequal_msg}: {sorted(lengths)}")
    if lengths.pop() == 0:
        raise ValueError(zero_msg)
    if alphabet is None:
        seen = set()
        for s in sequences:
            seen.update(s.upper())
        alphabet = detect_alphabet(seen - _GAP_CHARS)
    return tokenize(_as_bytes(sequences, names), alphabet, names=names), alphabet


# ------------------------------------------------------------------- Newick
def _strip_comments(s):
    out, depth, quoted = [], 0, False
    for ch in s:
        if ch == "'" and depth == 0:
            quoted = not quoted
            out.append(ch)
        elif quoted:
            out.append(ch)
        elif ch == "[":
            depth += 1
        elif ch == "]":
            depth -= 1
        elif depth == 0:
            out.append(ch)
    return "".join(out)


def parse_newick(newick_str):
    """Newick -> dict(parentIndex (R,) int32 DFS preorder with root -1,
    distanceToParent (R,) float64 (root 0), leaf_names, node_names)."""
    s = _strip_comments(newick_str.strip())
    while s.endswith(";"):
        s = s[:-1]
    s = s.strip()
    if not s:
        raise ValueError("Empty Newick string")
    n = len(s)
    pos = 0

    def label():
        nonlocal pos
        if pos >= n:
            return None
        if s[pos] == "'":
            pos += 1
            parts = []
            while pos < n:
                ch = s[pos]
                pos += 1
                if ch == "'":
                    if pos < n and s[pos] == "'":
                        parts.append("'")
                        pos += 1
                    else:
                        return "".join(parts)
                else:
                    parts.append(ch)
            raise ValueError("Unterminated quoted label")
        start = pos
        while pos < n and s[pos] not in "(),:;":
            pos += 1
        text = s[start:pos].strip()
        return text or None

    def length():
        nonlocal pos
        if pos < n and s[pos] == ":":
            pos += 1
            start = pos
            while pos < n and s[pos] not in "(),;":
                pos += 1
            text = s[start:pos].strip()
            return float(text) if text else 0.0
        return None

    def expect(ch):
        nonlocal pos
        if pos >= n:   # an unclosed group ends the string (IndexError, as in the reference)
            raise IndexError("string index out of range")
        got = s[pos]
        if got != ch:
            raise ValueError(f"Expected '{ch}' at position {pos}, got '{got}'")
        pos += 1

    # nodes in post-order: (name, dist, children); an explicit stack of the
    # open groups' child lists replaces the recursion
    nodes = []
    pending = []
    root = None

    def close(kids):
        name = label()
        d = length()
        nodes.append((name, 0.0 if d is None else d, kids))
        return len(nodes) - 1

    while root is None:
        while pos < n and s[pos] == "(":
            pos += 1
            pending.append([])
        idx = close([])
        while True:
            if not pending:
                root = idx
                break
            pending[-1].append(idx)
            if pos < n and s[pos] == ",":
                pos += 1
                break
            expect(")")
            idx = close(pending.pop())
    parent, dist_out, names, leaves = [], [], [], []
    todo = [(root, -1)]
    while todo:
        old, par = todo.pop()
        new = len(parent)
        name, d, kids = nodes[old]
        parent.append(par)
        dist_out.append(d if par >= 0 else 0.0)
        names.append(name)
        if not kids:
            leaves.append(name)
        for k in reversed(kids):
            todo.append((k, new))
    return {"parentIndex": np.array(parent, dtype=np.int32),
            "distanceToParent": np.array(dist_out, dtype=np.float64),
            "leaf_names": leaves, "node_names": names}


# --------------------------------------------------------------- alignments
def parse_fasta(text, alphabet=None):
    """FASTA -> dict(alignment (N, C) int32, leaf_names, alphabet)."""
    names, seqs, cur = [], [], None
    for line in text.splitlines():
        line = line.strip()
        if not line:
            continue
        if line.startswith(">"):
            if cur is not None:
                seqs.append("".join(cur))
            header = line[1:].strip()
            names.append(header.split()[0] if header else "")
            cur = []
        elif cur is not None:
            cur.append(line)
    if cur is not None:
        seqs.append("".join(cur))
    if not seqs:
        raise ValueError("No sequences found in FASTA input")
    aln, alphabet = _encode(seqs, alphabet, names, "No sequences found in FASTA input",
                            "Unequal sequence lengths in FASTA", "Empty sequences in FASTA input")
    return {"alignment": aln, "leaf_names": names, "alphabet": alphabet}


def parse_stockholm(text, alphabet=None):
    """Stockholm -> dict(alignment, leaf_names, alphabet); interleaved
    blocks are concatenated per name in first-seen order."""
    order, parts = [], {}
    for line in text.splitlines():
        line = line.strip()
        if not line or line.startswith("#") or line == "//":
            continue
        fields = line.split()
        if len(fields) < 2:
            continue
        name, seq = fields[0], fields[1]
        if name not in parts:
            order.append(name)
            parts[name] = []
        parts[name].append(seq)
    if not order:
        raise ValueError("No sequences found in Stockholm input")
    seqs = ["".join(parts[nm]) for nm in order]
    aln, alphabet = _encode(seqs, alphabet, order, "No sequences found in Stockholm input",
                            "Unequal sequence lengths in Stockholm", "Empty sequences in Stockholm input")
    return {"alignment": aln, "leaf_names": order, "alphabet": alphabet}


def parse_maf(text, alphabet=None):
    """MAF -> dict(alignment, leaf_names, alphabet): species = source name
    before the first '.', blocks concatenated, absent species gap-filled."""
    blocks, cur = [], None
    for line in text.splitlines():
        line = line.rstrip()
        if line.startswith("a"):
            cur = []
            blocks.append(cur)
        elif line.startswith("s") and cur is not None:
            f = line.split()
            cur.append((f[1].split(".")[0], f[-1]))
    if not blocks:
        raise ValueError("No alignment blocks found in MAF input")
    species = []
    for b in blocks:
        for sp, _ in b:
            if sp not in species:
                species.append(sp)
    if alphabet is None:
        seen = set()
        for b in blocks:
            for _, seq in b:
                seen.update(seq.upper())
        alphabet = detect_alphabet(seen - _GAP_CHARS)
    rows = {sp: [] for sp in species}
    for b in blocks:
        width = len(b[0][1]) if b else 0
        have = {sp: seq for sp, seq in b}
        for sp in species:
            rows[sp].append(have.get(sp, "-" * width))
    seqs = ["".join(rows[sp]) for sp in species]
    aln = tokenize(_as_bytes(seqs, species), alphabet, names=species) if seqs and len(seqs[0]) else \
        np.zeros((len(species), 0), np.int32)
    return {"alignment": aln, "leaf_names": species, "alphabet": alphabet}


def parse_strings(sequences, alphabet=None):
    """Equal-length strings -> dict(alignment, alphabet)."""
    aln, alphabet = _encode(list(sequences), alphabet, None, "Empty sequence list", "Unequal sequence lengths",
                            "Empty sequences")
    return {"alignment": aln, "alphabet": alphabet}


def parse_dict(sequences, alphabet=None):
    """name -> sequence dict -> dict(alignment, leaf_names, alphabet)."""
    if not sequences:
        raise ValueError("Empty sequence dictionary")
    names = list(sequences.keys())
    aln, alphabet = _encode([sequences[k] for k in names], alphabet, names, "Empty sequence dictionary",
                            "Unequal sequence lengths", "Empty sequences")
    return {"alignment": aln, "leaf_names": names, "alphabet": alphabet}


def combine_tree_alignment(tree_result, alignment_result):
    """Place each tree leaf's sequence (matched by name) at its node; internal
    rows get the ungapped-unobserved token A."""
    leaves = tree_result["leaf_names"]
    names = alignment_result["leaf_names"]
    data = np.asarray(alignment_result["alignment"])
    alphabet = alignment_result["alphabet"]
    row_of = {nm: i for i, nm in enumerate(names)}
    missing = [nm for nm in leaves if nm not in row_of]
    if missing:
        raise ValueError(f"Tree leaves not found in alignment: {missing}")
    parent = np.asarray(tree_result["parentIndex"])
    R = len(parent)
    full = np.full((R, data.shape[1]), len(alphabet), dtype=np.int32)
    nkids = np.bincount(parent[1:], minlength=R) if R > 1 else np.zeros(R, np.int64)
    leaf_nodes = np.flatnonzero(nkids == 0)
    full[leaf_nodes] = data[[row_of[nm] for nm in leaves]]
    return CombinedResult(alignment=full,
                          tree=Tree(parentIndex=tree_result["parentIndex"],
                                    distanceToParent=tree_result["distanceToParent"]),
                          alphabet=alphabet, leaf_names=leaves)
