"""Front-end: alignment and tree text formats to the hot path's inputs.

Same names, arguments, return values and errors as subby/formats.py
(``detect_alphabet`` :37-60, ``parse_newick`` :150-225, ``parse_fasta``
:228-315, ``parse_stockholm`` :318-410, ``parse_maf`` :413-507,
``parse_strings`` :510-564, ``parse_dict`` :567-625,
``combine_tree_alignment`` :1101-1169; the k-mer, codon and paired-column
transforms ``sliding_windows``, ``all_column_ktuples``, ``kmer_tokenize``,
``genetic_code``, ``codon_to_sense``, ``split_paired_columns``,
``merge_paired_columns`` :628-1098).  Differences are in how, not what:

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


# ---------------------------------------------------------------------------
# k-mer, codon and paired-column transforms (subby/formats.py:628-1098):
# derived alphabets for the large-A paths (A^k k-mers, 61 sense codons,
# A^2 column pairs), same names, token conventions and errors.
# ---------------------------------------------------------------------------

class KmerIndex:
    """Column tuples <-> positions of a k-mer alignment (subby/formats.py:628-656)."""

    def __init__(self, column_tuples):
        self.tuples = np.asarray(column_tuples, dtype=np.int64)
        self._pos = {tuple(int(x) for x in t): i for i, t in enumerate(self.tuples)}

    def tuple_to_idx(self, t):
        """Position of a column tuple in the k-mer alignment, -1 if absent."""
        return self._pos.get(tuple(int(x) for x in t), -1)

    def idx_to_tuple(self, idx):
        return tuple(self.tuples[idx])

    def __len__(self):
        return len(self.tuples)

    def __repr__(self):
        return f"KmerIndex({len(self)} tuples, k={self.tuples.shape[1] if len(self) > 0 else 0})"


def sliding_windows(C, k, stride=None, offset=0, edge="truncate"):
    """(M, k) int64 column indices of windows of k columns starting at
    offset, offset + stride, ... (stride defaults to k).  edge='truncate'
    keeps whole windows only; edge='pad' keeps the ragged last windows with
    -1 past the end (subby/formats.py:659-693)."""
    step = k if stride is None else stride
    if edge == "truncate":
        starts = np.arange(offset, C - k + 1, step)
    elif edge == "pad":
        starts = np.arange(offset, C, step)
    else:
        raise ValueError(f"Unknown edge mode: {edge!r}")
    cols = (starts[:, None] + np.arange(k)[None, :]).astype(np.int64)
    if edge == "pad":
        cols[cols >= C] = -1
    return cols.reshape(-1, k)


def all_column_ktuples(C, k, ordered=True):
    """Every k-tuple of distinct columns: permutations (ordered) or
    combinations, in itertools order, as (T, k) int64 (subby/formats.py:696-720)."""
    from itertools import combinations, permutations
    gen = permutations(range(C), k) if ordered else combinations(range(C), k)
    return np.array(list(gen), dtype=np.int64).reshape(-1, k)


def _kmer_labels(alphabet, k):
    if alphabet is None:
        return None
    from itertools import product
    return ["".join(p) for p in product(alphabet, repeat=k)]


def kmer_tokenize(alignment, A, k_or_tuples, gap_mode="any", alphabet=None):
    """k-mer tokens of an A-state alignment (subby/formats.py:723-842).

    ``k_or_tuples``: an int k (consecutive non-overlapping windows; C must be
    a multiple of k) or a (T, k) array of column tuples (-1 = a position
    outside the alignment, read as unobserved).  Output tokens: the base-A
    number of k observed states (first column most significant), A^k when
    any position is unobserved, A^k + 1 when a position is a gap (token < 0
    or > A) — with gap_mode='all' only all-gap k-mers are gaps and partly
    gapped ones get the illegal token A^k + 2.  Returns {'alignment' (R, T)
    int32, 'A_kmer': A^k, 'index': KmerIndex, 'alphabet' (labels, when an
    alphabet is given)}."""
    aln = np.asarray(alignment, dtype=np.int32)
    R, C = aln.shape
    if isinstance(k_or_tuples, (int, np.integer)):
        k = int(k_or_tuples)
        if C % k != 0:
            raise ValueError(f"Number of columns ({C}) not divisible by k ({k})")
        tuples = sliding_windows(C, k)
    else:
        tuples = np.asarray(k_or_tuples, dtype=np.int64)
        if tuples.ndim != 2:
            raise ValueError(f"column_tuples must be 2D (T, k), got shape {tuples.shape}")
        k = tuples.shape[1]
    A_k = A ** k
    out = {"alignment": np.zeros((R, 0), dtype=np.int32), "A_kmer": A_k, "index": KmerIndex(tuples)}
    if len(tuples):
        outside = tuples < 0
        b = aln[:, np.where(outside, 0, tuples)]                  # (R, T, k)
        b = np.where(outside[None], A, b)
        obs = (b >= 0) & (b < A)
        gap = (b < 0) | (b > A)
        weights = np.int64(A) ** np.arange(k - 1, -1, -1, dtype=np.int64)
        code = (np.where(obs, b, 0).astype(np.int64) * weights).sum(axis=2)
        tok = np.where(obs.all(axis=2), code, A_k)
        any_gap, all_gap = gap.any(axis=2), gap.all(axis=2)
        if gap_mode == "any":
            tok = np.where(any_gap, A_k + 1, tok)
        elif gap_mode == "all":
            tok = np.where(all_gap, A_k + 1, np.where(any_gap, A_k + 2, tok))
        else:
            raise ValueError(f"Unknown gap_mode: {gap_mode!r}")
        out["alignment"] = tok.astype(np.int32)
    labels = _kmer_labels(alphabet, k)
    if labels is not None:
        out["alphabet"] = labels
    return out


# The standard genetic code, third / second / first base varying fastest in
# T, C, A, G order (the textbook table read row by row); '*' = stop.
_CODE_TCAG = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG"


def genetic_code():
    """The standard genetic code over the 64 codons in ACGT lexicographic
    order (AAA, AAC, ..., TTT): codons, amino_acids, sense_mask, the 61
    sense_indices, codon_to_sense (stop -> -1), sense_codons,
    sense_amino_acids (subby/formats.py:877-919)."""
    from itertools import product
    tcag = "TCAG"
    codons = ["".join(p) for p in product("ACGT", repeat=3)]
    aa = [_CODE_TCAG[16 * tcag.index(c[0]) + 4 * tcag.index(c[1]) + tcag.index(c[2])] for c in codons]
    sense = np.array([a != "*" for a in aa], dtype=bool)
    idx = np.flatnonzero(sense).astype(np.int64)
    to_sense = np.full(64, -1, dtype=np.int64)
    to_sense[idx] = np.arange(len(idx), dtype=np.int64)
    return {"codons": codons, "amino_acids": aa, "sense_mask": sense, "sense_indices": idx,
            "codon_to_sense": to_sense, "sense_codons": [codons[i] for i in idx],
            "sense_amino_acids": [aa[i] for i in idx]}


def codon_to_sense(alignment, A=64):
    """64-codon tokens -> 61 sense-codon tokens: sense codons renumbered,
    stop codons and gaps (A + 1 or negative) -> 62, unobserved (A) and
    anything else -> 61 (subby/formats.py:922-965)."""
    aln = np.asarray(alignment, dtype=np.int32)
    table = genetic_code()["codon_to_sense"].copy()
    table[table < 0] = 62
    res = np.full_like(aln, 61)
    codon = (aln >= 0) & (aln < 64)
    res[codon] = table[aln[codon]]
    res[aln == A] = 61
    res[(aln == A + 1) | (aln < 0)] = 62
    return {"alignment": res, "A_sense": 61, "alphabet": genetic_code()["sense_codons"]}


def split_paired_columns(alignment, paired_columns, A=20):
    """Split an alignment into an A^2-state alignment of column pairs and an
    A-state alignment of the columns in no pair (subby/formats.py:972-1039);
    pairs and singles are k-mer tokens with gap_mode='any'."""
    aln = np.asarray(alignment, dtype=np.int32)
    N, C = aln.shape
    in_pair = {int(c) for pc in paired_columns for c in pc}
    singles = [c for c in range(C) if c not in in_pair]
    if len(paired_columns):
        pt = kmer_tokenize(aln, A, np.array(paired_columns, dtype=np.int64), gap_mode="any")
        p_aln, p_idx = pt["alignment"], pt["index"]
    else:
        p_aln, p_idx = np.zeros((N, 0), dtype=np.int32), KmerIndex(np.zeros((0, 2), dtype=np.int64))
    if singles:
        st = kmer_tokenize(aln, A, np.array(singles, dtype=np.int64).reshape(-1, 1), gap_mode="any")
        s_aln, s_idx = st["alignment"], st["index"]
    else:
        s_aln, s_idx = np.zeros((N, 0), dtype=np.int32), KmerIndex(np.zeros((0, 1), dtype=np.int64))
    return {"paired_alignment": p_aln, "singles_alignment": s_aln, "paired_columns": list(paired_columns),
            "single_columns": singles, "A_paired": A * A, "A_singles": A, "paired_index": p_idx,
            "singles_index": s_idx}


def merge_paired_columns(paired_posterior, singles_posterior, split_info):
    """(A, C) per-column posteriors from (A^2, P) pair posteriors (marginals
    over the partner column) and (A, S) single-column posteriors, in the
    original column order (subby/formats.py:1042-1098)."""
    pp = np.asarray(paired_posterior, dtype=np.float64)
    sp = np.asarray(singles_posterior, dtype=np.float64)
    pairs = split_info["paired_columns"]
    singles = split_info["single_columns"]
    A = split_info["A_singles"]
    cols = [c for pc in pairs for c in pc] + list(singles)
    out = np.zeros((A, max(cols) + 1 if cols else 0), dtype=np.float64)
    for p, (ci, cj) in enumerate(pairs):
        joint = pp[:A * A, p].reshape(A, A)
        out[:, ci] = joint.sum(axis=1)
        out[:, cj] = joint.sum(axis=0)
    for s, c in enumerate(singles):
        out[:, c] = sp[:, s]
    return out
