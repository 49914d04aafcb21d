"""Drop-in replacement for the entry points of ``subby.jax``.

``LogLike``, ``Counts``, ``BranchCounts``, ``RootProb``, ``MixturePosterior``,
``LogLikeCustomGrad`` and ``InsideOutside`` take the same arguments as
subby/jax/__init__.py:207, :338, :450, :543, :653, :294 and :681 and return
the same shapes (column last).  They run on the GPU through the C ABI of
``libsubby_gb300.so``; there is no CPU fallback.

Inputs may be numpy arrays (results come back as numpy float32, copies in
and out are part of the call) or CUDA ``torch`` tensors (results stay on the
device as torch tensors, work is enqueued on the current torch stream).

Models: ``DiagModel``, ``RateModel`` (diagonalised on the host),
``IrrevDiagModel`` (complex eigensystem; every entry point but the F81 fast
path, which is reversible-only in the reference too), ``*H`` batches,
per-column model lists and per-branch model grids
(subby/jax/__init__.py:53-205; ``subby_gb300/batch.py``).  Not supported
(``NotImplementedError``): InsideOutside over model grids (as in the
reference) and over per-column lists whose pi differ, per-branch
irreversible models.
"""
from __future__ import annotations

import ctypes as ct
import hashlib
import threading
from collections import OrderedDict

import numpy as np

from . import _lib, batch
from .models import ensure_diag
from .padding import strip_dummy_leaves
from .types import IrrevDiagModel, Tree

_PLAN_CACHE_SIZE = 32


def _is_torch(x) -> bool:
    try:
        import torch
    except ImportError:  # pragma: no cover
        return False
    return isinstance(x, torch.Tensor)


def _np(x, dtype):
    if _is_torch(x):
        x = x.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(x), dtype=dtype)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ct.c_void_p)


class Plan:
    """A (tree, model) pair prepared once and kept resident on the GPU.

    Creating a plan validates the tree (binary, preorder), builds the node
    schedule, computes M(t) in FP64 on the host and J(t) on the GPU.  The
    plan can then run any number of alignments with that tree and model.
    """

    def __init__(self, tree, model, device=None):
        lib = _lib.load()
        if isinstance(model, (list, tuple)) and not hasattr(model, '_fields'):
            self._init_rows(tree, model, device)
            return
        m = ensure_diag(model)
        self.parentIndex = _np(tree.parentIndex, np.int32)
        self.distances = _np(tree.distanceToParent, np.float64)
        self.irreversible = isinstance(m, IrrevDiagModel)
        if self.irreversible:
            self.eigenvalues = _np(m.eigenvalues, np.complex128)
            self.eigenvectors = _np(m.eigenvectors, np.complex128)
            self.eigenvectors_inv = _np(m.eigenvectors_inv, np.complex128)
        else:
            if np.iscomplexobj(m.eigenvalues) or np.iscomplexobj(m.eigenvectors):
                raise ValueError("complex eigensystems need an IrrevDiagModel (with eigenvectors_inv)")
            self.eigenvalues = _np(m.eigenvalues, np.float64)
            self.eigenvectors = _np(m.eigenvectors, np.float64)
        self.pi = _np(m.pi, np.float64)
        self.R = int(self.parentIndex.shape[0])
        self.A = int(self.pi.shape[0])
        if self.distances.shape != (self.R,):
            raise ValueError("distanceToParent must have shape (R,)")
        if self.eigenvalues.shape != (self.A,) or self.eigenvectors.shape != (self.A, self.A):
            raise ValueError("model arrays must have shapes (A,), (A, A), (A,)")
        self.device = device
        self._handle = ct.c_void_p()
        self._lock = threading.Lock()
        with _device_ctx(device):
            if self.irreversible:
                if self.eigenvectors_inv.shape != (self.A, self.A):
                    raise ValueError("eigenvectors_inv must have shape (A, A)")
                _lib.check(lib.subby_plan_create_irrev(
                    _ptr(self.parentIndex), _ptr(self.distances), _ptr(self.eigenvalues),
                    _ptr(self.eigenvectors), _ptr(self.eigenvectors_inv), _ptr(self.pi), self.R, self.A,
                    ct.byref(self._handle)), "subby_plan_create_irrev")
            else:
                _lib.check(lib.subby_plan_create(
                    _ptr(self.parentIndex), _ptr(self.distances), _ptr(self.eigenvalues),
                    _ptr(self.eigenvectors), _ptr(self.pi), self.R, self.A, ct.byref(self._handle)),
                    "subby_plan_create")

    def _init_rows(self, tree, models_row, device):
        """Per-branch models: one reversible model per node (node 0's pi is
        the root prior)."""
        lib = _lib.load()
        ms = [ensure_diag(m) for m in models_row]
        if any(isinstance(m, IrrevDiagModel) for m in ms):
            raise NotImplementedError("per-branch irreversible models are not supported")
        self.parentIndex = _np(tree.parentIndex, np.int32)
        self.distances = _np(tree.distanceToParent, np.float64)
        self.R = int(self.parentIndex.shape[0])
        if len(ms) != self.R:
            raise ValueError(f"expected {self.R} per-branch models, got {len(ms)}")
        self.irreversible = False
        self.eigenvalues = np.ascontiguousarray(np.stack([np.asarray(m.eigenvalues, np.float64) for m in ms]))
        self.eigenvectors = np.ascontiguousarray(np.stack([np.asarray(m.eigenvectors, np.float64) for m in ms]))
        self.pi = np.ascontiguousarray(np.stack([np.asarray(m.pi, np.float64) for m in ms]))
        self.A = int(self.pi.shape[1])
        self.device = device
        self._handle = ct.c_void_p()
        self._lock = threading.Lock()
        with _device_ctx(device):
            _lib.check(lib.subby_plan_create_rows(
                _ptr(self.parentIndex), _ptr(self.distances), _ptr(self.eigenvalues), _ptr(self.eigenvectors),
                _ptr(self.pi), self.R, self.A, ct.byref(self._handle)), "subby_plan_create_rows")
        self.pi = self.pi[0]

    # ------------------------------------------------------------------ run
    def run(self, alignment, loglike=True, counts=False, rootprob=False, f81=False,
            branch_mask="auto", bt64=None, out=None, stream=None, exact_irreversible=False):
        """Run the hot path; returns a dict with the requested outputs.

        ``branch_mask``: "auto" (Steiner mask, the reference default for
        Counts), None (unmasked) or an (R, C) bool array.  ``exact_irreversible``
        (irreversible models only): the expected counts of M(t) = e^{Qt}
        itself instead of the reference's formula, which for a non-reversible
        Q gives those of the transposed process.  ``bt64``: None =
        FP64 back-transform for A <= 8 and FP32 above; True/False forces it.
        ``out``: optional dict of preallocated output buffers (same keys).
        ``stream``: torch.cuda.Stream for the device-pointer path (default:
        the current stream).
        """
        lib = _lib.load()
        kind = _lib.COUNTS_F81 if f81 else _lib.COUNTS_EIGEN
        flags = _lib.IRREV_EXACT if exact_irreversible else 0
        if bt64 is True:
            flags |= _lib.BT_FP64
        elif bt64 is False:
            flags |= _lib.BT_FP32
        if isinstance(branch_mask, str):
            if branch_mask != "auto":
                raise ValueError('branch_mask must be "auto", None or an (R, C) array')
            mask_mode, mask = _lib.MASK_AUTO, None
        elif branch_mask is None:
            mask_mode, mask = _lib.MASK_NONE, None
        else:
            mask_mode, mask = _lib.MASK_GIVEN, branch_mask
        if not counts:
            mask_mode, mask = _lib.MASK_NONE, None
        A = self.A
        if _is_torch(alignment) and alignment.is_cuda:
            import torch
            aln = alignment
            if aln.dtype != torch.int32:
                aln = aln.to(torch.int32)
            aln = aln.contiguous()
            if aln.dim() != 2 or aln.shape[0] != self.R:
                raise ValueError(f"alignment must have shape (R={self.R}, C)")
            C = int(aln.shape[1])
            dev = aln.device
            res = {}
            out = out or {}
            if loglike:
                res['logLike'] = out.get('logLike', torch.empty(C, dtype=torch.float32, device=dev))
            if counts:
                res['counts'] = out.get('counts', torch.empty((A, A, C), dtype=torch.float32, device=dev))
            if rootprob:
                res['rootProb'] = out.get('rootProb', torch.empty((A, C), dtype=torch.float32, device=dev))
            dmask = None
            if mask_mode == _lib.MASK_GIVEN:
                dmask = torch.as_tensor(np.asarray(mask) if not _is_torch(mask) else mask)
                dmask = dmask.to(device=dev, dtype=torch.uint8).contiguous()
                if tuple(dmask.shape) != (self.R, C):
                    raise ValueError("branch_mask must have shape (R, C)")
            stream = (stream if stream is not None else torch.cuda.current_stream(dev)).cuda_stream

            def dp(t):
                return ct.c_void_p(t.data_ptr()) if t is not None else None
            with self._lock, _device_ctx(dev):
                _lib.check(lib.subby_plan_run(
                    self._handle, dp(aln), C, dp(res.get('logLike')), dp(res.get('counts')),
                    dp(res.get('rootProb')), kind, mask_mode, dp(dmask),
                    flags | _lib.DEVICE_PTRS, ct.c_void_p(stream)), "subby_plan_run")
            return res
        aln = _np(alignment, np.int32)
        if aln.ndim != 2 or aln.shape[0] != self.R:
            raise ValueError(f"alignment must have shape (R={self.R}, C)")
        C = int(aln.shape[1])
        out = out or {}
        res = {}
        if loglike:
            res['logLike'] = out.get('logLike', np.empty(C, dtype=np.float32))
        if counts:
            res['counts'] = out.get('counts', np.empty((A, A, C), dtype=np.float32))
        if rootprob:
            res['rootProb'] = out.get('rootProb', np.empty((A, C), dtype=np.float32))
        hmask = None
        if mask_mode == _lib.MASK_GIVEN:
            hmask = _np(mask, np.uint8)
            if hmask.shape != (self.R, C):
                raise ValueError("branch_mask must have shape (R, C)")

        def hp(a):
            return _ptr(a) if a is not None else None
        with self._lock, _device_ctx(self.device):
            _lib.check(lib.subby_plan_run(
                self._handle, _ptr(aln), C, hp(res.get('logLike')), hp(res.get('counts')),
                hp(res.get('rootProb')), kind, mask_mode, hp(hmask), flags, None),
                "subby_plan_run")
        return res

    def branch_counts(self, alignment, f81=False, branch_mask=None, out=None, stream=None,
                      exact_irreversible=False):
        """Per-branch counts (R, A, A, C): dwell times (diagonal) and
        substitution counts (off-diagonal) of every branch (branch 0, the
        root, is zeros).  ``branch_mask`` defaults to None (unmasked), as in
        subby.jax.BranchCounts; "auto" and an (R, C) array are accepted."""
        lib = _lib.load()
        kind = _lib.COUNTS_F81 if f81 else _lib.COUNTS_EIGEN
        xf = _lib.IRREV_EXACT if exact_irreversible else 0
        if isinstance(branch_mask, str):
            if branch_mask != "auto":
                raise ValueError('branch_mask must be "auto", None or an (R, C) array')
            mask_mode, mask = _lib.MASK_AUTO, None
        elif branch_mask is None:
            mask_mode, mask = _lib.MASK_NONE, None
        else:
            mask_mode, mask = _lib.MASK_GIVEN, branch_mask
        A, R = self.A, self.R
        if _is_torch(alignment) and alignment.is_cuda:
            import torch
            aln = alignment.to(torch.int32).contiguous()
            if aln.dim() != 2 or aln.shape[0] != R:
                raise ValueError(f"alignment must have shape (R={R}, C)")
            C = int(aln.shape[1])
            res = out if out is not None else torch.empty((R, A, A, C), dtype=torch.float32, device=aln.device)
            dmask = None
            if mask_mode == _lib.MASK_GIVEN:
                dmask = torch.as_tensor(np.asarray(mask) if not _is_torch(mask) else mask)
                dmask = dmask.to(device=aln.device, dtype=torch.uint8).contiguous()
            st = (stream if stream is not None else torch.cuda.current_stream(aln.device)).cuda_stream
            with self._lock, _device_ctx(aln.device):
                _lib.check(lib.subby_plan_branch_counts(
                    self._handle, ct.c_void_p(aln.data_ptr()), C, ct.c_void_p(res.data_ptr()), kind, mask_mode,
                    ct.c_void_p(dmask.data_ptr()) if dmask is not None else None, _lib.DEVICE_PTRS | xf,
                    ct.c_void_p(st)), "subby_plan_branch_counts")
            return res
        aln = _np(alignment, np.int32)
        if aln.ndim != 2 or aln.shape[0] != R:
            raise ValueError(f"alignment must have shape (R={R}, C)")
        C = int(aln.shape[1])
        res = out if out is not None else np.empty((R, A, A, C), dtype=np.float32)
        hmask = _np(mask, np.uint8) if mask_mode == _lib.MASK_GIVEN else None
        with self._lock, _device_ctx(self.device):
            _lib.check(lib.subby_plan_branch_counts(
                self._handle, _ptr(aln), C, _ptr(res), kind, mask_mode,
                _ptr(hmask) if hmask is not None else None, xf, None), "subby_plan_branch_counts")
        return res

    def posteriors(self, alignment, node=None, want_node=True, want_branch=False, stream=None):
        """Inside-outside posteriors: ``{'node': ..., 'branch': ...}`` with
        the node posteriors (R, A, C) (row 0: the root, = RootProb) and the
        branch joint posteriors (R, A, A, C) [n, i, j, c] = P(parent of n = i,
        n = j | column c) (branch 0 zeros); for ``node=n`` only that node's
        (A, C) / (A, A, C).  Numpy in, numpy out; a CUDA tensor in, tensors on
        its device out (enqueued on ``stream`` or the current stream)."""
        if not (want_node or want_branch):
            raise ValueError("request the node and/or the branch posteriors")
        lib = _lib.load()
        A, R = self.A, self.R
        nd = -1 if node is None else int(node)
        if nd < -1 or nd >= R:
            raise IndexError(f"node {node} out of range for R={R}")
        if want_branch and nd == 0:
            raise ValueError("node 0 (the root) has no branch")
        lead = (R,) if nd < 0 else ()
        res = {}
        if _is_torch(alignment) and alignment.is_cuda:
            import torch
            aln = alignment.to(torch.int32).contiguous()
            if aln.dim() != 2 or aln.shape[0] != R:
                raise ValueError(f"alignment must have shape (R={R}, C)")
            C = int(aln.shape[1])
            kw = dict(dtype=torch.float32, device=aln.device)
            if want_node:
                res['node'] = torch.empty(lead + (A, C), **kw)
            if want_branch:
                res['branch'] = torch.empty(lead + (A, A, C), **kw)
            dp = lambda k: ct.c_void_p(res[k].data_ptr()) if k in res else None  # noqa: E731
            st = (stream if stream is not None else torch.cuda.current_stream(aln.device)).cuda_stream
            with self._lock, _device_ctx(aln.device):
                _lib.check(lib.subby_plan_posteriors(
                    self._handle, ct.c_void_p(aln.data_ptr()), C, nd, dp('node'), dp('branch'), _lib.DEVICE_PTRS,
                    ct.c_void_p(st)), "subby_plan_posteriors")
            return res
        aln = _np(alignment, np.int32)
        if aln.ndim != 2 or aln.shape[0] != R:
            raise ValueError(f"alignment must have shape (R={R}, C)")
        C = int(aln.shape[1])
        if want_node:
            res['node'] = np.empty(lead + (A, C), dtype=np.float32)
        if want_branch:
            res['branch'] = np.empty(lead + (A, A, C), dtype=np.float32)
        hp = lambda k: _ptr(res[k]) if k in res else None  # noqa: E731
        with self._lock, _device_ctx(self.device):
            _lib.check(lib.subby_plan_posteriors(self._handle, _ptr(aln), C, nd, hp('node'), hp('branch'), 0, None),
                       "subby_plan_posteriors")
        return res

    def grad(self, alignment, g=None, want_loglike=True):
        """(logLike (C,), d(sum g logL)/dt (R,), d(sum g logL)/dS~ (A, A) FP64)."""
        lib = _lib.load()
        aln = _np(alignment, np.int32)
        if aln.ndim != 2 or aln.shape[0] != self.R:
            raise ValueError(f"alignment must have shape (R={self.R}, C)")
        C = int(aln.shape[1])
        gg = None if g is None else _np(g, np.float32)
        ll = np.empty(C, dtype=np.float32) if want_loglike else None
        dldt = np.zeros(self.R, dtype=np.float64)
        dldS = np.zeros((self.A, self.A), dtype=np.float64)
        with self._lock, _device_ctx(self.device):
            _lib.check(lib.subby_plan_grad(
                self._handle, _ptr(aln), C, _ptr(gg) if gg is not None else None,
                _ptr(ll) if ll is not None else None, _ptr(dldt), _ptr(dldS), 0, None),
                "subby_plan_grad")
        return ll, dldt, dldS

    def device_bytes(self) -> int:
        return int(_lib.load().subby_plan_device_bytes(self._handle))

    def set_root_prior(self, root_prior):
        """Use ``root_prior`` (A positive values) instead of the model's pi at
        the root: the root prior of subby.jax InsideOutside over a
        per-column model list, the first model's pi for every column
        (subby/jax/__init__.py:721-731)."""
        rp = np.ascontiguousarray(root_prior, dtype=np.float64)
        if rp.shape != (self.A,):
            raise ValueError(f"root prior must have shape ({self.A},)")
        with self._lock:
            _lib.check(_lib.load().subby_plan_set_root_prior(self._handle, _ptr(rp)), "subby_plan_set_root_prior")

    def status(self):
        """Raise SubbyError if a bounded device wait of this plan's kernels
        gave up since the last check (waits for the plan's enqueued work)."""
        with self._lock:
            _lib.check(_lib.load().subby_plan_status(self._handle), "subby_plan_status")

    def trim(self):
        """Release the workspace (kept tables); the next run allocates again."""
        with self._lock:
            _lib.check(_lib.load().subby_plan_trim(self._handle), "subby_plan_trim")

    def close(self):
        if getattr(self, "_handle", None) and self._handle.value:
            _lib.load().subby_plan_destroy(self._handle)
            self._handle = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


class _device_ctx:
    def __init__(self, dev):
        self.dev = dev
        self.ctx = None

    def __enter__(self):
        if self.dev is not None:
            import torch
            self.ctx = torch.cuda.device(self.dev)
            self.ctx.__enter__()

    def __exit__(self, *a):
        if self.ctx is not None:
            self.ctx.__exit__(*a)


# ---------------------------------------------------------------------------
# plan cache and the subby.jax-compatible functions
# ---------------------------------------------------------------------------

_cache: "OrderedDict[str, Plan]" = OrderedDict()
_cache_lock = threading.Lock()


def _key(tree, model, device):
    h = hashlib.sha1()
    parts = [tree.parentIndex, tree.distanceToParent, model.eigenvalues, model.eigenvectors, model.pi]
    if isinstance(model, IrrevDiagModel):
        parts.append(model.eigenvectors_inv)
    for a in parts:
        arr = np.ascontiguousarray(_np(a, np.complex128 if np.iscomplexobj(a) else np.float64))
        h.update(arr.tobytes())
        h.update(str(arr.shape).encode())
    h.update(str(device).encode())
    return h.hexdigest()


def get_plan(tree, model, device=None) -> Plan:
    """Cached Plan for (tree, model)."""
    _reject_batched(model)
    m = ensure_diag(model)
    k = _key(tree, m, device)
    with _cache_lock:
        p = _cache.get(k)
        if p is not None:
            _cache.move_to_end(k)
            return p
    p = Plan(tree, m, device)
    with _cache_lock:
        _cache[k] = p
        while len(_cache) > _PLAN_CACHE_SIZE:
            _cache.popitem(last=False)[1].close()
    return p


def clear_plan_cache():
    with _cache_lock:
        while _cache:
            _cache.popitem()[1].close()


def _reject_batched(model):
    if isinstance(model, (list, tuple)) and not hasattr(model, '_fields'):
        raise NotImplementedError("per-column model lists and model grids are not supported")


def _device_of(x):
    if _is_torch(x) and x.is_cuda:
        return x.device
    return None


def _rows_plan(tree, models_row, device):
    """Cached plan for per-branch models (the (1, R) model grid)."""
    ms = [ensure_diag(m) for m in models_row]
    h = hashlib.sha1()
    for m in ms:
        h.update(batch._key(m).encode())
    k = _key(tree, ms[0], device) + "/rows/" + h.hexdigest()
    with _cache_lock:
        p = _cache.get(k)
        if p is not None:
            _cache.move_to_end(k)
            return p
    p = Plan(tree, ms, device)
    with _cache_lock:
        _cache[k] = p
        while len(_cache) > _PLAN_CACHE_SIZE:
            _cache.popitem(last=False)[1].close()
    return p


def _grid(alignment, tree, grid, fn, out_shape):
    """Model grid: (1, R) per-branch models for every column, or (C, R) per
    column (columns grouped by identical rows).  fn(plan, sub_alignment,
    column indices) -> result for those columns."""
    dev = _device_of(alignment)
    C = int(alignment.shape[1])
    if len(grid) == 1:
        return fn(_rows_plan(tree, grid[0], dev), alignment, None)
    if len(grid) != C:
        raise ValueError(f"model grid has {len(grid)} columns but the alignment has {C}")
    groups = OrderedDict()
    for c, row in enumerate(grid):
        key = "/".join(batch._key(ensure_diag(m)) for m in row)
        groups.setdefault(key, (row, []))[1].append(c)
    out = batch._new(alignment, out_shape)
    for row, idx in groups.values():
        bm_idx = idx
        batch._put(out, idx, fn(_rows_plan(tree, row, dev), batch._take(alignment, idx), bm_idx))
    return out


def _unpad(alignment, tree, model, k):
    """subby.jax's padded trees (dummy leaves under the root) for LogLike
    and RootProb: the trailing dummy leaves are dropped (each contributes a
    factor 1), so the kernels see the binary tree."""
    if k == 'grid':
        return alignment, tree
    m0 = model[0] if k == 'list' else model
    return strip_dummy_leaves(alignment, tree, lambda: int(np.asarray(ensure_diag(m0).pi).shape[-1]))


def _slice_mask(branch_mask, idx):
    if idx is None or branch_mask is None or isinstance(branch_mask, str):
        return branch_mask
    return batch._take(branch_mask, idx)


def LogLike(alignment, tree: Tree, model, maxChunkSize: int = 128):
    """Per-column log-likelihoods (C,); subby/jax/__init__.py:207.  A ``*H``
    batched model gives (*H, C); a list of C models one model per column."""
    del maxChunkSize  # columns are tiled on the device
    k = batch.kind(model)
    alignment, tree = _unpad(alignment, tree, model, k)
    if k == 'grid':
        return _grid(alignment, tree, model, lambda p, a, idx: p.run(a, loglike=True)['logLike'],
                     (int(alignment.shape[1]),))
    if k == 'list':
        return batch.loglike_list(alignment, tree, model, get_plan)
    dev = _device_of(alignment)
    one = lambda m: get_plan(tree, m, dev).run(alignment, loglike=True)['logLike']  # noqa: E731
    return batch.map_h(model, one) if k == 'H' else one(model)


def Counts(alignment, tree: Tree, model, maxChunkSize: int = 128, f81_fast_flag: bool = False,
           branch_mask="auto", exact_irreversible: bool = False):
    """(A, A, C) dwell times (diagonal) and substitution counts; subby/jax/__init__.py:338.
    ``*H`` batches and per-column model lists as for ``LogLike``.
    ``exact_irreversible`` (not in the reference): see ``Plan.run``."""
    del maxChunkSize
    k = batch.kind(model)
    if k == 'grid':
        A = len(ensure_diag(model[0][0]).pi)
        return _grid(alignment, tree, model, lambda p, a, idx: p.run(
            a, loglike=False, counts=True, f81=f81_fast_flag, branch_mask=_slice_mask(branch_mask, idx))['counts'],
            (A, A, int(alignment.shape[1])))
    if k == 'list':
        return batch.counts_list(alignment, tree, model, get_plan, f81=f81_fast_flag, branch_mask=branch_mask,
                                 exact_irreversible=exact_irreversible)
    dev = _device_of(alignment)
    one = lambda m: get_plan(tree, m, dev).run(  # noqa: E731
        alignment, loglike=False, counts=True, f81=f81_fast_flag, branch_mask=branch_mask,
        exact_irreversible=exact_irreversible)['counts']
    return batch.map_h(model, one) if k == 'H' else one(model)


def BranchCounts(alignment, tree: Tree, model, maxChunkSize: int = 128, f81_fast_flag: bool = False,
                 branch_mask=None, exact_irreversible: bool = False):
    """(R, A, A, C) per-branch dwell times and substitution counts, branch 0
    zeros; subby/jax/__init__.py:450 (unmasked there; ``branch_mask`` as in
    the oracle's BranchCounts, subby/oracle/oracle.py:1517)."""
    del maxChunkSize
    k = batch.kind(model)
    if k == 'grid':
        A = len(ensure_diag(model[0][0]).pi)
        return _grid(alignment, tree, model, lambda p, a, idx: p.branch_counts(
            a, f81=f81_fast_flag, branch_mask=_slice_mask(branch_mask, idx)),
            (int(alignment.shape[0]), A, A, int(alignment.shape[1])))
    if k == 'list':
        return batch.counts_list(alignment, tree, model, get_plan, f81=f81_fast_flag, branch_mask=branch_mask,
                                 exact_irreversible=exact_irreversible, per_branch=True)
    dev = _device_of(alignment)
    one = lambda m: get_plan(tree, m, dev).branch_counts(  # noqa: E731
        alignment, f81=f81_fast_flag, branch_mask=branch_mask, exact_irreversible=exact_irreversible)
    return batch.map_h(model, one) if k == 'H' else one(model)


def RootProb(alignment, tree: Tree, model, maxChunkSize: int = 128):
    """(A, C) posterior root distribution; subby/jax/__init__.py:543."""
    del maxChunkSize
    k = batch.kind(model)
    alignment, tree = _unpad(alignment, tree, model, k)
    if k == 'grid':
        A = len(ensure_diag(model[0][0]).pi)
        return _grid(alignment, tree, model, lambda p, a, idx: p.run(a, loglike=False, rootprob=True)['rootProb'],
                     (A, int(alignment.shape[1])))
    if k == 'list':
        return batch.rootprob_list(alignment, tree, model, get_plan)
    dev = _device_of(alignment)
    one = lambda m: get_plan(tree, m, dev).run(alignment, loglike=False, rootprob=True)['rootProb']  # noqa: E731
    return batch.map_h(model, one) if k == 'H' else one(model)


def MixturePosterior(alignment, tree: Tree, models, log_weights, maxChunkSize: int = 128):
    """(K, C) posterior over the K mixture components per column;
    subby/jax/__init__.py:653-678 (log-likelihoods of batched components
    are summed over their ``*H`` dimensions, as there)."""
    del maxChunkSize
    lls = []
    for m in models:
        ll = LogLike(alignment, tree, m)
        while ll.ndim > 1:
            ll = ll.sum(0)
        lls.append(ll)
    if _is_torch(lls[0]):
        import torch
        stacked = torch.stack(lls)
    else:
        stacked = np.stack(lls)
    return batch.mixture_posterior(stacked, log_weights)


def LogLikeCustomGrad(alignment, tree: Tree, model, maxChunkSize: int = 128, method: str = 'eigen'):
    """LogLike whose gradient w.r.t. ``tree.distanceToParent`` comes from the
    hand-written adjoint kernel (subby/jax/__init__.py:294, vjp.py:35-136).

    ``tree.distanceToParent`` may be a torch tensor with ``requires_grad``;
    the result is then a torch tensor connected to it.  Only ``method='eigen'``
    exists here (the Padé variant of the reference computes the same value).
    """
    del maxChunkSize
    if method not in ('eigen', 'pade'):
        raise ValueError("method must be 'eigen' or 'pade'")
    from .autograd import loglike_with_grad
    return loglike_with_grad(alignment, tree, model)


class InsideOutside:
    """Inside-outside queries on one alignment; subby/jax/__init__.py:681-1040.

    The reference runs both passes once and keeps U and D for the queries;
    here the (tree, model) plan stays resident and each query runs its fused
    kernels (walk + accumulation or posterior kernel) over the alignment, so
    nothing of size R x C x A is held between queries.  ``*H`` batched models
    give outputs with leading ``*H``; per-column model lists are grouped by
    model (posteriors need one root prior: lists whose pis differ raise
    ``NotImplementedError``); model grids raise ``NotImplementedError``, as in
    the reference.
    """

    def __init__(self, alignment, tree: Tree, model, maxChunkSize: int = 128):
        del maxChunkSize
        self._kind = batch.kind(model)
        if self._kind == 'grid':
            raise NotImplementedError("InsideOutside does not support model grids")
        self._alignment = alignment
        self._tree = tree
        self._model = model
        self._logLike = None

    def _one(self, m):
        return get_plan(self._tree, m, _device_of(self._alignment))

    def _each(self, fn):
        """fn(plan, alignment) for a single model, stacked over *H."""
        if self._kind == 'H':
            return batch.map_h(self._model, lambda m: fn(self._one(m), self._alignment))
        return fn(self._one(self._model), self._alignment)

    @property
    def log_likelihood(self):
        """Per-column log-likelihoods (*H, C)."""
        if self._logLike is None:
            self._logLike = LogLike(self._alignment, self._tree, self._model)
        return self._logLike

    def counts(self, f81_fast_flag: bool = False, branch_mask="auto"):
        """(*H, A, A, C) dwell times and substitution counts (as ``Counts``)."""
        return Counts(self._alignment, self._tree, self._model, f81_fast_flag=f81_fast_flag, branch_mask=branch_mask)

    def branch_counts(self, f81_fast_flag: bool = False):
        """(*H, R, A, A, C) per-branch counts, unmasked (as ``BranchCounts``)."""
        return BranchCounts(self._alignment, self._tree, self._model, f81_fast_flag=f81_fast_flag)

    def _posteriors(self, node, want_node, want_branch, key):
        if self._kind != 'list':
            return self._each(lambda p, a: p.posteriors(a, node=node, want_node=want_node,
                                                        want_branch=want_branch)[key])
        ms, groups = batch._groups(self._alignment, self._model)
        # the inside and outside passes of every column take the first
        # model's pi at the root (subby/jax/__init__.py:721-731: rootProb =
        # stacked.pi[0]); the root's own posterior row takes the column's own
        # pi (its outside vector is set from the stacked pis, :763-774)
        pi0 = np.asarray(ms[0].pi, np.float64)
        R, A, C = int(self._alignment.shape[0]), len(pi0), int(self._alignment.shape[1])
        lead = (R,) if node is None else ()
        shape = lead + ((A,) if key == 'node' else (A, A)) + (C,)
        out = batch._new(self._alignment, shape)
        for m, idx in groups:
            same = np.array_equal(np.asarray(m.pi, np.float64), pi0)
            # a group whose own pi differs runs on a plan of its own with the
            # shared root prior (cached plans keep their model's pi)
            plan = self._one(m) if same else Plan(self._tree, ensure_diag(m), _device_of(self._alignment))
            try:
                if not same:
                    plan.set_root_prior(pi0)
                r = plan.posteriors(batch._take(self._alignment, idx), node=node, want_node=want_node,
                                    want_branch=want_branch)[key]
            finally:
                if not same:
                    plan.close()
            if not same and key == 'node' and (node is None or int(node) == 0):
                # root row: pi0 o U_0 normalised -> pi_g o U_0 normalised
                # (U_0 does not depend on the root prior)
                w = np.asarray(m.pi, np.float64) / pi0
                if _is_torch(r):
                    import torch
                    w = torch.as_tensor(w, dtype=r.dtype, device=r.device)
                row = r[0] if node is None else r
                row = row * w[:, None]
                row = row / row.sum(0, keepdims=True) if not _is_torch(row) else row / row.sum(0, keepdim=True)
                if node is None:
                    r[0] = row
                else:
                    r = row
            batch._put(out, idx, r)
        return out

    def node_posterior(self, node=None):
        """Posterior state distribution: (*H, A, C) for ``node``, (*H, R, A, C)
        for every node when ``node`` is None."""
        return self._posteriors(node, True, False, 'node')

    def branch_posterior(self, node=None):
        """Joint posterior of (parent state, child state): (*H, A, A, C) for
        ``node`` > 0, (*H, R, A, A, C) with branch 0 zeros when ``node`` is
        None."""
        if node is not None and int(node) == 0:
            raise ValueError("node 0 (the root) has no branch")
        return self._posteriors(node, False, True, 'branch')
