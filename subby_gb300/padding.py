"""Shape padding of subby.jax (subby/jax/_utils.py:12-27, 103-225), kept for
drop-in compatibility.

The reference pads alignments (gap columns) and trees (dummy leaves under
the root with zero branch length and gap rows) to a few bin sizes so that
JAX does not recompile for every shape.  This backend has no shape-keyed
compilation, so padding only costs work here, but padded inputs give the
reference's results: a gap column has logLike 0 and zero counts, and
``LogLike`` / ``RootProb`` / ``MixturePosterior`` drop trailing dummy leaves
(``strip_dummy_leaves``) before validating the tree, since each contributes
a factor 1 (its all-ones likelihood vector times a stochastic matrix) and
the kernels take binary trees only.
"""
from __future__ import annotations

import numpy as np

from .types import Tree

# sizes max(1, round(1.19^k)), k < 120, without repeats
GEOM_BINS: list = sorted({max(1, round(1.19 ** k)) for k in range(120)})


def _is_torch(x) -> bool:
    try:
        import torch
    except ImportError:  # pragma: no cover
        return False
    return isinstance(x, torch.Tensor)


def _cat(parts, axis):
    if _is_torch(parts[0]):
        import torch
        return torch.cat(parts, dim=axis)
    return np.concatenate(parts, axis=axis)


def _full_like(x, shape, value):
    if _is_torch(x):
        import torch
        return torch.full(shape, value, dtype=x.dtype, device=x.device)
    return np.full(shape, value, dtype=np.asarray(x).dtype)


def pad_to_geom_bin(n: int) -> int:
    """Smallest GEOM_BINS entry >= n; beyond the table the next power of two."""
    for b in GEOM_BINS:
        if b >= n:
            return b
    return int(2 ** np.ceil(np.log2(max(n, 1))))


def pad_alignment(alignment, bin_size: int = 128, bin_fn=None):
    """(alignment with gap (-1) columns appended up to bin_fn(C), or up to a
    multiple of bin_size, C)."""
    C = int(alignment.shape[1])
    Cp = bin_fn(C) if bin_fn is not None else -(-C // bin_size) * bin_size
    if Cp == C:
        return alignment, C
    return _cat([alignment, _full_like(alignment, (int(alignment.shape[0]), Cp - C), -1)], 1), C


def pad_tree(tree, n_nodes_padded: int):
    """The tree with dummy leaves (parent 0, branch length 0) appended up to
    n_nodes_padded nodes."""
    R = int(tree.parentIndex.shape[0])
    if n_nodes_padded <= R:
        return tree
    n = n_nodes_padded - R
    return Tree(parentIndex=_cat([tree.parentIndex, _full_like(tree.parentIndex, (n,), 0)], 0),
                distanceToParent=_cat([tree.distanceToParent, _full_like(tree.distanceToParent, (n,), 0)], 0))


def pad_tree_and_alignment(tree, alignment, node_bin_fn=None, col_bin_fn=None):
    """(padded tree, padded alignment, R, C): nodes and columns padded to
    node_bin_fn(R) / col_bin_fn(C) (default pad_to_geom_bin), new cells -1."""
    node_bin_fn = node_bin_fn or pad_to_geom_bin
    col_bin_fn = col_bin_fn or pad_to_geom_bin
    R, C = int(alignment.shape[0]), int(alignment.shape[1])
    Rp, Cp = node_bin_fn(R), col_bin_fn(C)
    aln = alignment
    if Rp > R:
        aln = _cat([aln, _full_like(aln, (Rp - R, C), -1)], 0)
    if Cp > C:
        aln = _cat([aln, _full_like(aln, (Rp, Cp - C), -1)], 1)
    return pad_tree(tree, Rp), aln, R, C


def unpad_columns(result, C_original: int):
    """The first C_original columns (last axis) of a result."""
    return result[..., :C_original]


def strip_dummy_leaves(alignment, tree, A):
    """Drop the trailing run of dummy leaves that makes the root non-binary:
    nodes with parent 0, branch length 0, no children and a row of tokens
    outside 0..A-1 (all-ones likelihood), while the root keeps more than two
    children.  Returns (alignment, tree) unchanged when there are none.
    ``A``: the alphabet size, or a function returning it (called only when
    the root has more than two children)."""
    parent = np.asarray(tree.parentIndex.detach().cpu() if _is_torch(tree.parentIndex) else tree.parentIndex,
                        dtype=np.int64)
    R = len(parent)
    kids_of_root = int(np.count_nonzero(parent[1:] == 0))
    if R < 4 or kids_of_root <= 2:
        return alignment, tree
    d = tree.distanceToParent
    dist = np.asarray(d.detach().cpu() if _is_torch(d) else d, dtype=np.float64)
    has_kids = np.zeros(R, dtype=bool)
    has_kids[parent[1:]] = True
    n = R
    while n > 1 and parent[n - 1] == 0 and dist[n - 1] == 0.0 and not has_kids[n - 1]:
        n -= 1
    n = max(n, R - (kids_of_root - 2))
    if n == R:
        return alignment, tree
    A = A() if callable(A) else A
    if not _is_torch(alignment):
        alignment = np.asarray(alignment)
    rows = alignment[n:R]
    neutral = (rows < 0) | (rows >= A)
    flat = neutral.all(dim=1).cpu().numpy() if _is_torch(neutral) else np.asarray(neutral).all(axis=1)
    # only the all-neutral rows after the last row with data may go
    k = n if flat.all() else n + int(np.flatnonzero(~flat)[-1]) + 1
    if k >= R:
        return alignment, tree
    return alignment[:k], Tree(parentIndex=tree.parentIndex[:k], distanceToParent=tree.distanceToParent[:k])
