"""Batched models: ``*H`` model batches, per-column model lists, mixtures.

The reference accepts, besides one model (subby/jax/__init__.py:53-205):

* a model whose arrays carry leading batch dimensions ``*H`` (e.g. the K
  discrete-gamma rate categories of ``scale_model(base, rates)``): every
  output gains the leading ``*H``;
* a list of C models, one per alignment column: column c uses model c's
  M(t); the log-likelihood's root prior is the first model's pi for every
  column (subby/jax/__init__.py:267-277), RootProb multiplies by each
  column's own pi (:617-633), Counts and BranchCounts run column by column
  with the column's own model (:396-411, :497-512);
* ``MixturePosterior`` over K models (:653-678);
* a model grid: ``[[m_0, ..., m_{R-1}]]`` gives node n (the branch above
  it) its own model for every column, ``[[...], ...]`` (C rows) such a list
  per column (:74-152, :225-261).

Here a ``*H`` batch runs one resident plan per batch member, each over all
columns, with the results stacked on the device (no host round trip for
device inputs).  A per-column list is grouped by distinct model: each group
of columns is gathered into one sub-alignment and run by that model's plan,
and the results are scattered back — K distinct models cost K fused launches
instead of the reference's per-column loop.  The first-model root prior of
LogLike / RootProb is applied exactly from the group's own LogLike and root
posterior: with q = pi_g U / P_g, P_0 / P_g = sum_a q_a pi0_a / pi_g,a.
A model grid runs a per-branch plan (``subby_plan_create_rows``): M_n from
node n's model, the complex accumulation once per group of branches that
share a model, each branch in its own eigenbasis; a (C, R) grid groups the
columns by identical rows.
"""
from __future__ import annotations

import hashlib
from collections import OrderedDict

import numpy as np

from . import _lib
from .models import ensure_diag, unbatch, batch_shape


def _is_torch(x):
    try:
        import torch
    except ImportError:  # pragma: no cover
        return False
    return isinstance(x, torch.Tensor)


def kind(model) -> str:
    """'single', 'H' (leading batch dimensions), 'list' (one model per
    column) or 'grid' (list of lists)."""
    if isinstance(model, (list, tuple)) and not hasattr(model, '_fields'):
        if len(model) == 0:
            raise ValueError("empty model list")
        first = model[0]
        if isinstance(first, (list, tuple)) and not hasattr(first, '_fields'):
            return 'grid'
        return 'list'
    return 'H' if batch_shape(model) else 'single'


def _key(m) -> str:
    h = hashlib.sha1()
    for f in m._fields:
        a = np.ascontiguousarray(np.asarray(getattr(m, f)))
        h.update(f.encode() + str(a.dtype).encode() + str(a.shape).encode() + a.tobytes())
    return h.hexdigest()


def _stack(outs, H):
    if _is_torch(outs[0]):
        import torch
        return torch.stack(outs).reshape(tuple(H) + tuple(outs[0].shape))
    return np.stack(outs).reshape(tuple(H) + outs[0].shape)


def map_h(model, fn):
    """fn(single model) for every member of a ``*H`` batch, stacked (*H, ...)."""
    H, ms = unbatch(model)
    return _stack([fn(m) for m in ms], H)


def _groups(alignment, models):
    C = int(alignment.shape[1])
    if len(models) != C:
        raise ValueError(f"expected {C} per-column models, got {len(models)}")
    ms = [ensure_diag(m) for m in models]
    if any(batch_shape(m) for m in ms):
        raise NotImplementedError("per-column lists of batched models are not supported")
    groups = OrderedDict()
    for c, m in enumerate(ms):
        groups.setdefault(_key(m), (m, []))[1].append(c)
    return ms, list(groups.values())


def _take(x, idx):
    """Columns idx of x (column last), as a contiguous array / tensor."""
    if _is_torch(x):
        import torch
        return x.index_select(x.dim() - 1, torch.as_tensor(idx, device=x.device)).contiguous()
    return np.ascontiguousarray(np.asarray(x)[..., idx])


def _new(like_alignment, shape):
    if _is_torch(like_alignment) and like_alignment.is_cuda:
        import torch
        return torch.empty(shape, dtype=torch.float32, device=like_alignment.device)
    return np.empty(shape, dtype=np.float32)


def _put(out, idx, val):
    if _is_torch(out):
        import torch
        out.index_copy_(out.dim() - 1, torch.as_tensor(idx, device=out.device), val)
    else:
        out[..., idx] = val


def _ratio_to_root0(q, pi_g, pi_0):
    """sum_a q_a pi0_a / pi_g,a per column: P_0 / P_g."""
    w = np.asarray(pi_0, np.float64) / np.asarray(pi_g, np.float64)
    if _is_torch(q):
        import torch
        return (q.double() * torch.as_tensor(w, device=q.device)[:, None]).sum(0)
    return (np.asarray(q, np.float64) * w[:, None]).sum(0)


def loglike_list(alignment, tree, models, get_plan):
    ms, groups = _groups(alignment, models)
    pi0 = np.asarray(ms[0].pi, np.float64)
    out = _new(alignment, (int(alignment.shape[1]),))
    dev = alignment.device if (_is_torch(alignment) and alignment.is_cuda) else None
    for m, idx in groups:
        same = np.array_equal(np.asarray(m.pi, np.float64), pi0)
        r = get_plan(tree, m, dev).run(_take(alignment, idx), loglike=True, rootprob=not same)
        ll = r['logLike']
        if not same:
            f = _ratio_to_root0(r['rootProb'], m.pi, pi0)
            ll = (ll.double() + f.log()).float() if _is_torch(ll) else (ll + np.log(f)).astype(np.float32)
        _put(out, idx, ll)
    return out


def rootprob_list(alignment, tree, models, get_plan):
    ms, groups = _groups(alignment, models)
    pi0 = np.asarray(ms[0].pi, np.float64)
    A = len(pi0)
    out = _new(alignment, (A, int(alignment.shape[1])))
    dev = alignment.device if (_is_torch(alignment) and alignment.is_cuda) else None
    for m, idx in groups:
        q = get_plan(tree, m, dev).run(_take(alignment, idx), loglike=False, rootprob=True)['rootProb']
        if not np.array_equal(np.asarray(m.pi, np.float64), pi0):
            f = _ratio_to_root0(q, m.pi, pi0)
            q = (q.double() / f[None, :]).float() if _is_torch(q) else (q / f[None, :]).astype(np.float32)
        _put(out, idx, q)
    return out


def counts_list(alignment, tree, models, get_plan, f81=False, branch_mask="auto", exact_irreversible=False,
                per_branch=False):
    ms, groups = _groups(alignment, models)
    A = len(ms[0].pi)
    R = int(alignment.shape[0])
    C = int(alignment.shape[1])
    out = _new(alignment, ((R,) if per_branch else ()) + (A, A, C))
    dev = alignment.device if (_is_torch(alignment) and alignment.is_cuda) else None
    for m, idx in groups:
        bm = branch_mask if (branch_mask is None or isinstance(branch_mask, str)) else _take(branch_mask, idx)
        plan = get_plan(tree, m, dev)
        sub = _take(alignment, idx)
        if per_branch:
            res = plan.branch_counts(sub, f81=f81, branch_mask=bm, exact_irreversible=exact_irreversible)
        else:
            res = plan.run(sub, loglike=False, counts=True, f81=f81, branch_mask=bm,
                           exact_irreversible=exact_irreversible)['counts']
        _put(out, idx, res)
    return out


def mixture_posterior(log_likes, log_weights):
    """(K, C) softmax over components of log_likes + log_weights, on the GPU
    (``subby_mixture_posterior``)."""
    import ctypes as ct
    lib = _lib.load()
    lw = np.ascontiguousarray(np.asarray(log_weights, dtype=np.float64))
    K = int(lw.shape[0])
    if _is_torch(log_likes) and log_likes.is_cuda:
        import torch
        ll = log_likes.to(torch.float32).contiguous()
        if ll.dim() != 2 or ll.shape[0] != K:
            raise ValueError(f"log_likes must have shape (K={K}, C)")
        out = torch.empty_like(ll)
        st = torch.cuda.current_stream(ll.device).cuda_stream
        with torch.cuda.device(ll.device):
            _lib.check(lib.subby_mixture_posterior(ct.c_void_p(ll.data_ptr()), lw.ctypes.data_as(ct.c_void_p), K,
                                                   int(ll.shape[1]), ct.c_void_p(out.data_ptr()), _lib.DEVICE_PTRS,
                                                   ct.c_void_p(st)), "subby_mixture_posterior")
        return out
    ll = np.ascontiguousarray(np.asarray(log_likes, dtype=np.float32))
    if ll.ndim != 2 or ll.shape[0] != K:
        raise ValueError(f"log_likes must have shape (K={K}, C)")
    out = np.empty_like(ll)
    _lib.check(lib.subby_mixture_posterior(ll.ctypes.data_as(ct.c_void_p), lw.ctypes.data_as(ct.c_void_p), K,
                                           int(ll.shape[1]), out.ctypes.data_as(ct.c_void_p), 0, None),
               "subby_mixture_posterior")
    return out
