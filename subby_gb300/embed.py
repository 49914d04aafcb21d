"""Alphabets the kernels do not take, run inside the next one they do.

The kernels are built for A = 2..8, 16, 20, 32 and 64.  A model over A
states with A in 9..15, 17..19, 21..31 or 33..63 — the 61 sense codons of
``codon_to_sense`` / ``gy94_model`` are the common case — runs as an A2-state
model (A2 the next kernel alphabet) whose extra A2 - A states are
unreachable:

* eigenvalues: the model's, then A2 - A zeros; eigenvectors (and their
  inverse) block-diagonal: the model's, then the identity; so M(t) and Q are
  block-diagonal and no probability moves between the blocks;
* pi: the model's, then ``EXTRA_PI`` (1e-20) per extra state (the kernels
  need a strictly positive pi);
* tokens: 0..A-1 unchanged, A (unobserved) -> A2, anything above A (gap or
  invalid: all-ones and gapped in the reference) -> A2 + 1, negatives
  unchanged; so the Steiner mask is the same;
* outputs: the first A states of counts, root / node / branch posteriors.

Every real-state output equals the A-state model's exactly except for the
extra states' share of the likelihood, pi_extra x (likelihood of the extra
block), which is 0 when a column has an observed token anywhere and
(A2 - A) x 1e-20 relative otherwise — below FP32 resolution.  The F81 fast
path (whose closed form needs all states exchangeable) is rejected.

Status: opt-in (``EmbeddedPlan(tree, model)``); ``get_plan`` and the
subby.jax-style functions still reject these alphabets.  The embedding is
exact in FP64 (tests/test_embed_host.py runs it through the oracle), but on a
GB300 a 61-state random reversible model (pi ~ Dirichlet(1), uniformly
random tokens on every node) embedded in the A = 64 tensor-core path gave
LogLike within 1e-5 and Counts with a column-wise error of 1.13e-4, above the
1e-4 bar.  In an FP32 restatement on the CPU the embedded and the direct
61-state computations agree to summation order and both carry ~1e-4 error
against FP64 on that input class (as does a plain 64-state model with
random tokens), so the deviation is the input's FP32 conditioning; the
posterior and irreversible paths of the embedding have not run on a GPU.
"""
from __future__ import annotations

import numpy as np

from .types import DiagModel, IrrevDiagModel

KERNEL_ALPHABETS = (2, 3, 4, 5, 6, 7, 8, 16, 20, 32, 64)
EXTRA_PI = 1e-20


def kernel_alphabet(A: int):
    """The smallest kernel alphabet >= A, or None above 64."""
    for a in KERNEL_ALPHABETS:
        if a >= A:
            return a
    return None


def embed_model(m, A2: int):
    """The A-state model m as an A2-state model with unreachable extra states."""
    pi = np.asarray(m.pi, dtype=np.float64)
    A = len(pi)
    pi2 = np.concatenate([pi, np.full(A2 - A, EXTRA_PI)])
    cx = isinstance(m, IrrevDiagModel)
    dt = np.complex128 if cx else np.float64
    mu2 = np.concatenate([np.asarray(m.eigenvalues, dtype=dt), np.zeros(A2 - A, dtype=dt)])

    def block(V):
        out = np.zeros((A2, A2), dtype=dt)
        out[:A, :A] = np.asarray(V, dtype=dt)
        out[A:, A:] = np.eye(A2 - A, dtype=dt)
        return out
    if cx:
        return IrrevDiagModel(mu2, block(m.eigenvectors), block(m.eigenvectors_inv), pi2)
    return DiagModel(mu2, block(m.eigenvectors), pi2)


def _is_torch(x) -> bool:
    try:
        import torch
    except ImportError:  # pragma: no cover
        return False
    return isinstance(x, torch.Tensor)


def embed_tokens(alignment, A: int, A2: int):
    """Tokens of the A-state alphabet as tokens of the A2-state one."""
    if _is_torch(alignment):
        import torch
        a = alignment.to(torch.int32)
        return torch.where(a > A, A2 + 1, torch.where(a == A, A2, a)).contiguous()
    a = np.asarray(alignment, dtype=np.int32)
    return np.where(a > A, A2 + 1, np.where(a == A, A2, a)).astype(np.int32)


def _first(x, A, axes):
    """x restricted to the first A states along ``axes`` (contiguous copy)."""
    idx = [slice(None)] * x.ndim
    for ax in axes:
        idx[ax] = slice(0, A)
    y = x[tuple(idx)]
    return y.contiguous() if _is_torch(y) else np.ascontiguousarray(y)


def _into(out, key, val):
    if out is None or key not in out:
        return val
    dst = out[key]
    if _is_torch(dst):
        dst.copy_(val)
    else:
        dst[...] = val
    return dst


class EmbeddedPlan:
    """A plan for an alphabet the kernels do not take; same methods and
    results as ``Plan`` (the A-state outputs), run by an inner ``Plan`` over
    the embedded A2-state model."""

    def __init__(self, tree, model, device=None, plan_cls=None):
        if plan_cls is None:
            from .api import Plan as plan_cls
        A = len(np.asarray(model.pi))
        A2 = kernel_alphabet(A)
        if A2 is None or A2 == A:
            raise ValueError(f"alphabet size {A} needs no embedding or cannot be embedded")
        self.A, self.A2 = A, A2
        self.inner = plan_cls(tree, embed_model(model, A2), device)
        self.R = self.inner.R
        self.device = device
        self.irreversible = isinstance(model, IrrevDiagModel)

    def _aln(self, alignment):
        return embed_tokens(alignment, self.A, self.A2)

    def run(self, alignment, loglike=True, counts=False, rootprob=False, f81=False, branch_mask="auto", bt64=None,
            out=None, stream=None, exact_irreversible=False):
        if f81:
            raise NotImplementedError(f"the F81 fast path needs a kernel alphabet (A={self.A} is embedded in "
                                      f"A={self.A2})")
        r = self.inner.run(self._aln(alignment), loglike=loglike, counts=counts, rootprob=rootprob,
                           branch_mask=branch_mask, bt64=bt64, stream=stream, exact_irreversible=exact_irreversible)
        res = {}
        if 'logLike' in r:
            res['logLike'] = _into(out, 'logLike', r['logLike'])
        if 'counts' in r:
            res['counts'] = _into(out, 'counts', _first(r['counts'], self.A, (0, 1)))
        if 'rootProb' in r:
            res['rootProb'] = _into(out, 'rootProb', _first(r['rootProb'], self.A, (0,)))
        return res

    def branch_counts(self, alignment, f81=False, branch_mask=None, out=None, stream=None, exact_irreversible=False):
        if f81:
            raise NotImplementedError("the F81 fast path needs a kernel alphabet")
        r = self.inner.branch_counts(self._aln(alignment), branch_mask=branch_mask, stream=stream,
                                     exact_irreversible=exact_irreversible)
        return _into({'b': out} if out is not None else None, 'b', _first(r, self.A, (1, 2)))

    def posteriors(self, alignment, node=None, want_node=True, want_branch=False, stream=None):
        r = self.inner.posteriors(self._aln(alignment), node=node, want_node=want_node, want_branch=want_branch,
                                  stream=stream)
        lead = 1 if node is None else 0
        res = {}
        if 'node' in r:
            res['node'] = _first(r['node'], self.A, (lead,))
        if 'branch' in r:
            res['branch'] = _first(r['branch'], self.A, (lead, lead + 1))
        return res

    def grad(self, alignment, g=None, want_loglike=True):
        ll, dldt, dldS = self.inner.grad(self._aln(alignment), g=g, want_loglike=want_loglike)
        return ll, dldt, np.ascontiguousarray(dldS[:self.A, :self.A])

    def device_bytes(self) -> int:
        return self.inner.device_bytes()

    def status(self):
        self.inner.status()

    def trim(self):
        self.inner.trim()

    def close(self):
        self.inner.close()
