"""The allocation-free entry point (subby_counts_noalloc) against the regular one.

Callers that cannot allocate device memory (a caching allocator owning the
device heap, a plugin that must not allocate) use subby_counts_noalloc: its
tables live in a fixed file-scope device array.  This test calls it through
the C ABI twice in a row, with two different trees and models, and checks each
result against subby_plan_run on the same inputs within the parity
tolerances.  It sits in a file of its own that pytest collects last.
"""
import ctypes as ct

import numpy as np
import pytest

from tests._tol import assert_cols, assert_loglike, COUNTS_RTOL

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import _lib, synth, models  # noqa: E402


def _p(a):
    return a.ctypes.data_as(ct.c_void_p)


def _noalloc(aln, tree, model, f81=False, mask_mode=_lib.MASK_AUTO):
    lib = _lib.load()
    R, C = aln.shape
    par = np.ascontiguousarray(tree.parentIndex, np.int32)
    dst = np.ascontiguousarray(tree.distanceToParent, np.float64)
    ev, V, pi = (np.ascontiguousarray(x, np.float64) for x in (model.eigenvalues, model.eigenvectors, model.pi))
    d_aln = torch.as_tensor(aln).cuda().contiguous()
    d_cnt = torch.empty((4, 4, C), dtype=torch.float32, device="cuda")
    d_ll = torch.empty(C, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.subby_counts_noalloc(ct.c_void_p(d_aln.data_ptr()), _p(par), _p(dst), _p(ev), _p(V), _p(pi),
                                  R, C, _lib.COUNTS_F81 if f81 else _lib.COUNTS_EIGEN, mask_mode, None,
                                  ct.c_void_p(d_cnt.data_ptr()), ct.c_void_p(d_ll.data_ptr()),
                                  ct.c_void_p(stream))
    assert rc == 0, lib.subby_strerror(rc)
    torch.cuda.synchronize()
    return d_cnt.cpu().numpy(), d_ll.cpu().numpy()


def _regular(aln, tree, model, f81=False):
    plan = sg.Plan(tree, model)
    r = plan.run(aln, loglike=True, counts=True, f81=f81, branch_mask="auto")
    plan.close()
    return r['counts'], r['logLike']


def test_noalloc_matches_regular_entry_point_twice_in_a_row():
    w1 = synth.plain_large(seed=2, C=3000)
    rng = np.random.default_rng(33)
    tree2 = synth.random_tree(40, 0.1, rng)
    model2 = models.hky85_diag(3.0, [0.2, 0.3, 0.3, 0.2])
    aln2 = synth.simulated_alignment(tree2, model2, 777, 0.1, rng)
    for aln, tree, model in ((w1['alignment'], w1['tree'], w1['model']), (aln2, tree2, model2)):
        got_c, got_l = _noalloc(aln, tree, model)
        ref_c, ref_l = _regular(aln, tree, model)
        assert_cols(got_c, ref_c, COUNTS_RTOL, "noalloc counts")
        assert_loglike(got_l, ref_l)


def test_noalloc_f81_and_size_limit():
    w = synth.plain_large(seed=2, C=1000, f81=True)
    got_c, _ = _noalloc(w['alignment'], w['tree'], w['model'], f81=True)
    ref_c, _ = _regular(w['alignment'], w['tree'], w['model'], f81=True)
    assert_cols(got_c, ref_c, COUNTS_RTOL, "noalloc f81 counts")
    # more than 1023 nodes is rejected before any GPU work
    big = synth.random_tree(600, 0.1, np.random.default_rng(1))
    lib = _lib.load()
    R = len(big.parentIndex)
    par = np.ascontiguousarray(big.parentIndex, np.int32)
    dst = np.ascontiguousarray(big.distanceToParent)
    m = models.jukes_cantor_model(4)
    ev, V, pi = (np.ascontiguousarray(x, np.float64) for x in m)
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = lib.subby_counts_noalloc(ct.c_void_p(dummy.data_ptr()), _p(par), _p(dst), _p(ev), _p(V), _p(pi),
                                  R, 1, 0, 0, None, ct.c_void_p(dummy.data_ptr()), None, None)
    assert rc == _lib.ERR_UNSUPPORTED
