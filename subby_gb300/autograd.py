"""torch.autograd wrappers around the hand-written adjoint kernel.

* ``loglike_with_grad`` — LogLike with d/d(branch lengths) from the adjoint
  (the Fisher-identity rule of subby/jax/vjp.py:62-133): the backward pass
  runs the outside pass again on the GPU and contracts
  D~_k mu_k e^{mu_k t} U~_k with the cotangent over columns.
* ``loglike_reversible`` — LogLike of a reversible model parameterised by
  log-exchangeabilities (upper triangle, row-major i<j) and pi, with
  gradients for branch lengths and log-exchangeabilities.  The adjoint kernel
  returns G = sum_c g_c V C_c V^T (C_c = unmasked eigenbasis counts), which
  is d(sum g logL)/dS~ for S~ = diag(sqrt pi) Q diag(1/sqrt pi); then
  dL/dQ_ij = sqrt(pi_i/pi_j) G_ij and the chain rule through Q(theta)
  (normalised to one substitution per unit time) runs in FP64 torch on the
  host (an A x A function).
"""
from __future__ import annotations

import numpy as np
import torch

from .api import Plan
from .models import diagonalize_rate_matrix
from .types import Tree


def _as_np(x, dtype):
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy().astype(dtype)
    return np.asarray(x, dtype=dtype)


class _LogLikeDist(torch.autograd.Function):
    @staticmethod
    def forward(ctx, distances, alignment, parent, model):
        tree = Tree(parent, _as_np(distances, np.float64))
        plan = Plan(tree, model)
        ll = plan.run(alignment, loglike=True)['logLike']
        ctx.plan = plan
        ctx.alignment = alignment
        return torch.as_tensor(ll, dtype=torch.float64, device=distances.device)

    @staticmethod
    def backward(ctx, g):
        _, dldt, _ = ctx.plan.grad(ctx.alignment, g=_as_np(g, np.float32), want_loglike=False)
        ctx.plan.close()
        return torch.as_tensor(dldt, dtype=g.dtype, device=g.device), None, None, None


def loglike_with_grad(alignment, tree, model):
    d = tree.distanceToParent
    if not isinstance(d, torch.Tensor):
        d = torch.as_tensor(np.asarray(d, dtype=np.float64))
    aln = _as_np(alignment, np.int32)
    return _LogLikeDist.apply(d, aln, _as_np(tree.parentIndex, np.int32), model)


def rate_matrix_torch(log_exch: torch.Tensor, pi: torch.Tensor) -> torch.Tensor:
    """Differentiable Q(theta): Q_ij = s_ij pi_j / Z, rows sum to zero,
    -sum_i pi_i Q_ii = 1 (same convention as models.reversible_rate_matrix)."""
    A = pi.shape[0]
    iu = torch.triu_indices(A, A, 1)
    s = torch.zeros((A, A), dtype=log_exch.dtype)
    s = s.index_put((iu[0], iu[1]), torch.exp(log_exch))
    s = s + s.T
    Q = s * pi[None, :]
    Q = Q / torch.sum(pi * Q.sum(1))
    return Q - torch.diag(Q.sum(1))


def exchangeability_grad(G, log_exch, pi):
    """d(sum g logL)/d(log s) from G = d(sum g logL)/dS~ (A x A, FP64).

    dL/dQ_ij = sqrt(pi_i/pi_j) G_ij for S~ = diag(sqrt pi) Q diag(1/sqrt pi);
    the chain through Q(log s) (with its normalisation) runs in FP64 torch.
    """
    pi = np.asarray(pi, dtype=np.float64)
    sp = np.sqrt(pi)
    dLdQ = torch.as_tensor(np.asarray(G, dtype=np.float64) * (sp[:, None] / sp[None, :]))
    with torch.enable_grad():
        le = torch.as_tensor(np.asarray(log_exch, dtype=np.float64)).clone().requires_grad_(True)
        Q = rate_matrix_torch(le, torch.as_tensor(pi))
        (dle,) = torch.autograd.grad(Q, le, grad_outputs=dLdQ)
    return dle.numpy()


class _LogLikeRev(torch.autograd.Function):
    @staticmethod
    def forward(ctx, distances, log_exch, alignment, parent, pi):
        pi_np = _as_np(pi, np.float64)
        le = log_exch.detach().double().cpu()
        Q = rate_matrix_torch(le, torch.as_tensor(pi_np)).numpy()
        model = diagonalize_rate_matrix(Q, pi_np)
        plan = Plan(Tree(parent, _as_np(distances, np.float64)), model)
        ctx.plan, ctx.alignment, ctx.pi = plan, alignment, pi_np
        ctx.save_for_backward(log_exch)
        ll = plan.run(alignment, loglike=True)['logLike']
        return torch.as_tensor(ll, dtype=torch.float64, device=distances.device)

    @staticmethod
    def backward(ctx, g):
        (log_exch,) = ctx.saved_tensors
        _, dldt, G = ctx.plan.grad(ctx.alignment, g=_as_np(g, np.float32), want_loglike=False)
        ctx.plan.close()
        dle = exchangeability_grad(G, log_exch.detach().double().cpu().numpy(), ctx.pi)
        return (torch.as_tensor(dldt, dtype=g.dtype, device=g.device),
                torch.as_tensor(dle, dtype=log_exch.dtype, device=log_exch.device), None, None, None)


def loglike_reversible(alignment, parentIndex, distances, log_exch, pi):
    """Per-column LogLike (float64 tensor) differentiable w.r.t. ``distances``
    and ``log_exch`` (both torch tensors)."""
    aln = _as_np(alignment, np.int32)
    return _LogLikeRev.apply(distances, log_exch, aln, _as_np(parentIndex, np.int32), pi)
