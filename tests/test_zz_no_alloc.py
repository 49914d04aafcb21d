"""The allocation-free entry point (subby_counts_noalloc) against the regular
entry point and the FP64 oracle.

Who calls it: code that must not allocate device memory — a host framework
whose caching allocator owns the whole device heap, a plugin or callback run
where allocation is forbidden, a service that fixes its device footprint at
start-up.  subby_counts_noalloc keeps its tables in a fixed file-scope device
array instead of allocating.  These tests call it through the C ABI, several
times in a row with different trees and models, and check each result
against subby_plan_run on the same inputs and against the oracle, within the
parity tolerances (LogLike 1e-5 relative, Counts 1e-4 column-wise).  They sit
in a file of their own that pytest collects last, and pass run alone in a
fresh process as well as after the other tests.
"""
import ctypes as ct

import numpy as np
import pytest

import oracle
from tests._tol import assert_cols, assert_loglike, COUNTS_RTOL

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import _lib, synth, models  # noqa: E402


def _p(a):
    return a.ctypes.data_as(ct.c_void_p)


def _args(tree, model):
    par = np.ascontiguousarray(tree.parentIndex, np.int32)
    dst = np.ascontiguousarray(tree.distanceToParent, np.float64)
    ev, V, pi = (np.ascontiguousarray(x, np.float64) for x in (model.eigenvalues, model.eigenvectors, model.pi))
    return par, dst, ev, V, pi


def _call(aln, tree, model, f81=False, mask_mode=_lib.MASK_AUTO, mask=None, want_ll=True):
    """One subby_counts_noalloc call on the current stream; returns (rc, counts, logLike)."""
    lib = _lib.load()
    R, C = aln.shape
    par, dst, ev, V, pi = _args(tree, model)
    d_aln = torch.as_tensor(aln).cuda().contiguous()
    d_mask = None if mask is None else torch.as_tensor(np.ascontiguousarray(mask, np.uint8)).cuda()
    d_cnt = torch.full((4, 4, C), float("nan"), dtype=torch.float32, device="cuda")
    d_ll = torch.full((C,), float("nan"), dtype=torch.float32, device="cuda") if want_ll else None
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.subby_counts_noalloc(ct.c_void_p(d_aln.data_ptr()), _p(par), _p(dst), _p(ev), _p(V), _p(pi),
                                  R, C, _lib.COUNTS_F81 if f81 else _lib.COUNTS_EIGEN, mask_mode,
                                  None if d_mask is None else ct.c_void_p(d_mask.data_ptr()),
                                  ct.c_void_p(d_cnt.data_ptr()),
                                  None if d_ll is None else ct.c_void_p(d_ll.data_ptr()), ct.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, d_cnt.cpu().numpy(), (None if d_ll is None else d_ll.cpu().numpy())


def _noalloc(*a, **k):
    rc, c, ll = _call(*a, **k)
    assert rc == 0, _lib.load().subby_strerror(rc)
    return c, ll


def _regular(aln, tree, model, f81=False, branch_mask="auto"):
    plan = sg.Plan(tree, model)
    r = plan.run(aln, loglike=True, counts=True, f81=f81, branch_mask=branch_mask)
    plan.close()
    return r['counts'], r['logLike']


def _oracle(aln, tree, model, f81=False, branch_mask="auto"):
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    md = {k: np.asarray(v, np.float64) for k, v in model._asdict().items()}
    return oracle.Counts(aln, ot, md, f81_fast=f81, branch_mask=branch_mask), oracle.LogLike(aln, ot, md)


def _second_case():
    rng = np.random.default_rng(33)
    tree = synth.random_tree(40, 0.1, rng)
    model = models.hky85_diag(3.0, [0.2, 0.3, 0.3, 0.2])
    return synth.simulated_alignment(tree, model, 777, 0.1, rng), tree, model


def test_noalloc_warmup_call_then_real_call():
    """C = 0 is the warm-up: it resolves the array's address and loads the
    kernels, computes nothing and needs no buffers; the next call runs."""
    aln, tree, model = _second_case()
    lib = _lib.load()
    par, dst, ev, V, pi = _args(tree, model)
    rc = lib.subby_counts_noalloc(None, _p(par), _p(dst), _p(ev), _p(V), _p(pi), len(par), 0,
                                  _lib.COUNTS_EIGEN, _lib.MASK_AUTO, None, None, None, None)
    assert rc == 0
    assert lib.subby_last_error() == b""
    got_c, got_l = _noalloc(aln, tree, model)
    ref_c, ref_l = _oracle(aln, tree, model)
    assert_cols(got_c, ref_c, COUNTS_RTOL, "noalloc counts after warm-up")
    assert_loglike(got_l, ref_l)


def test_noalloc_matches_regular_entry_point_twice_in_a_row():
    w1 = synth.plain_large(seed=2, C=3000)
    aln2, tree2, model2 = _second_case()
    for aln, tree, model in ((w1['alignment'], w1['tree'], w1['model']), (aln2, tree2, model2)):
        got_c, got_l = _noalloc(aln, tree, model)
        ref_c, ref_l = _regular(aln, tree, model)
        assert_cols(got_c, ref_c, COUNTS_RTOL, "noalloc counts")
        assert_loglike(got_l, ref_l)


def test_noalloc_matches_oracle_twice_in_a_row():
    w1 = synth.plain_large(seed=5, C=512)
    aln2, tree2, model2 = _second_case()
    for aln, tree, model in ((w1['alignment'], w1['tree'], w1['model']), (aln2[:, :300], tree2, model2)):
        got_c, got_l = _noalloc(aln, tree, model)
        ref_c, ref_l = _oracle(aln, tree, model)
        assert_cols(got_c, ref_c, COUNTS_RTOL, "noalloc counts vs oracle")
        assert_loglike(got_l, ref_l)


@pytest.mark.parametrize("f81", [False, True])
@pytest.mark.parametrize("mask_mode", [_lib.MASK_NONE, _lib.MASK_GIVEN])
def test_noalloc_mask_modes(f81, mask_mode):
    """Unmasked and caller-given masks, eigen and F81, against the regular
    entry point and the oracle; the call without a logLike buffer too."""
    rng = np.random.default_rng(7 + mask_mode + 2 * f81)
    tree = synth.random_tree(24, 0.1, rng)
    model = models.f81_model(rng.dirichlet(np.ones(4))) if f81 else models.hky85_diag(2.0, rng.dirichlet(np.ones(4)))
    aln = synth.simulated_alignment(tree, model, 400, 0.1, rng)
    if mask_mode == _lib.MASK_GIVEN:
        mask = rng.random(aln.shape) < 0.7
        bm = mask
    else:
        mask, bm = None, None
    got_c, got_l = _noalloc(aln, tree, model, f81=f81, mask_mode=mask_mode, mask=mask)
    ref_c, _ = _regular(aln, tree, model, f81=f81, branch_mask=bm)
    or_c, or_l = _oracle(aln, tree, model, f81=f81, branch_mask=bm)
    assert_cols(got_c, ref_c, COUNTS_RTOL, "noalloc vs regular")
    assert_cols(got_c, or_c, COUNTS_RTOL, "noalloc vs oracle")
    assert_loglike(got_l, or_l)
    got_c2, none = _noalloc(aln, tree, model, f81=f81, mask_mode=mask_mode, mask=mask, want_ll=False)
    assert none is None
    np.testing.assert_array_equal(got_c2, got_c)


def test_noalloc_single_node_tree():
    """R = 1: the root is the only leaf, no branches: zero counts and the
    root's own likelihood."""
    tree = sg.Tree(np.array([-1], np.int32), np.array([0.0]))
    model = models.hky85_diag(2.0, [0.1, 0.2, 0.3, 0.4])
    aln = np.array([[0, 1, 2, 3, 4, 5, -1]], np.int32)
    got_c, got_l = _noalloc(aln, tree, model, mask_mode=_lib.MASK_NONE)
    np.testing.assert_array_equal(got_c, np.zeros_like(got_c))
    _, or_l = _oracle(aln, tree, model, branch_mask=None)
    assert_loglike(got_l, or_l)


def test_noalloc_rejections_name_their_reason():
    lib = _lib.load()
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    m = models.jukes_cantor_model(4)
    ev, V, pi = (np.ascontiguousarray(x, np.float64) for x in m)

    def call(tree, kind=_lib.COUNTS_EIGEN):
        par = np.ascontiguousarray(tree.parentIndex, np.int32)
        dst = np.ascontiguousarray(tree.distanceToParent, np.float64)
        return lib.subby_counts_noalloc(ct.c_void_p(dummy.data_ptr()), _p(par), _p(dst), _p(ev), _p(V), _p(pi),
                                        len(par), 1, kind, _lib.MASK_NONE, None, ct.c_void_p(dummy.data_ptr()),
                                        None, None)
    # more than 1023 nodes: rejected before any GPU work
    assert call(synth.random_tree(600, 0.1, np.random.default_rng(1))) == _lib.ERR_UNSUPPORTED
    assert b"1023" in lib.subby_last_error()
    # ~500 nodes in eigen mode: the tables exceed the kernel's on-chip budget
    assert call(synth.random_tree(250, 0.1, np.random.default_rng(2))) == _lib.ERR_UNSUPPORTED
    assert b"budget" in lib.subby_last_error() or b"array" in lib.subby_last_error()
    # an invalid tree
    bad = sg.Tree(np.array([-1, 0, 0, 0], np.int32), np.array([0.0, 0.1, 0.1, 0.1]))
    assert call(bad) == _lib.ERR_TREE
    assert b"children" in lib.subby_last_error()
    # a later successful call clears the reason
    aln, tree, model = _second_case()
    _noalloc(aln[:, :64], tree, model)
    assert lib.subby_last_error() == b""


def test_noalloc_refuses_a_capturing_stream():
    """The table upload reads a host staging buffer that the next call
    rewrites, so a call on a stream under capture is refused before it
    enqueues anything."""
    aln, tree, model = _second_case()
    lib = _lib.load()
    par, dst, ev, V, pi = _args(tree, model)
    d_aln = torch.as_tensor(aln).cuda().contiguous()
    d_cnt = torch.zeros((4, 4, aln.shape[1]), dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        g.capture_begin()
        try:
            rc = lib.subby_counts_noalloc(ct.c_void_p(d_aln.data_ptr()), _p(par), _p(dst), _p(ev), _p(V), _p(pi),
                                          len(par), aln.shape[1], _lib.COUNTS_EIGEN, _lib.MASK_AUTO, None,
                                          ct.c_void_p(d_cnt.data_ptr()), None, ct.c_void_p(s.cuda_stream))
            d_cnt.add_(1.0)  # the capture holds one node of its own
        finally:
            g.capture_end()
    torch.cuda.synchronize()
    assert rc == _lib.ERR_UNSUPPORTED
    assert b"capturing" in lib.subby_last_error()
    # the stream is usable afterwards
    got_c, got_l = _noalloc(aln, tree, model)
    ref_c, ref_l = _oracle(aln, tree, model)
    assert_cols(got_c, ref_c, COUNTS_RTOL, "noalloc counts after a refused capture")
