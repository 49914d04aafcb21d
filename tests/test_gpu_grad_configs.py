"""Gradients and large-alphabet Counts at the workload shapes, against FP64.

* The A=20 differentiation workload (R=399 nodes, 200 leaves, branch lengths
  Exp(mean 0.08), 15% gaps): d(sum logL)/d(branch lengths) and
  d(sum logL)/d(log-exchangeabilities) from the adjoint kernel on a seeded
  256-column subsample of the 10^5 simulated columns, against central finite
  differences with h = 1e-4 of the FP64 oracle (the gradient rule of
  subby/jax/vjp.py:62-133; the exchangeability gradient, which the reference
  leaves to jax.grad, by the Fisher identity).  At full size the gradient is
  checked by linearity: the gradient over all columns equals the sum of the
  gradients over two column halves.
* Exchangeability and distance gradients at A = 16 and A = 64 (the walk +
  per-branch X_n path; tensor cores at A = 64) against the same FP64 finite
  differences (a seeded subset of the 2016 exchangeabilities at A = 64).
* The A=64 precision workload (R=127, random reversible model with ~5%
  near-degenerate eigenvalue pairs, 65536 simulated columns): Counts, LogLike
  and RootProb of a full-size run, on the split-BF16 tensor-core walk and the
  FP32 CUDA-core walk, compared with the oracle on a seeded subsample of 256
  columns, masked and unmasked.

Tolerances: gradients max |d| / max |ref| <= 1e-3 against differences with
h = 1e-4 (whose own truncation error is 3e-4 on the shortest branches) and
<= 2e-4 against h = 1e-6; 1e-4 for the linearity identity;
LogLike 1e-5 relative, Counts / RootProb 1e-4 column-wise (tests/_tol.py).
"""
import multiprocessing as mp

import numpy as np
import pytest

import oracle
from tests._tol import assert_cols, assert_loglike, COUNTS_RTOL, ROOTPROB_RTOL

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import subby_gb300 as sg  # noqa: E402
from subby_gb300 import synth, models, autograd, _lib  # noqa: E402

FD_RTOL = 1e-3      # vs differences with h = 1e-4 (their own truncation error reaches 3e-4)
TIGHT_RTOL = 2e-4   # vs differences with h = 1e-6 (truncation ~3e-8)


def _close(got, ref, what, rtol=FD_RTOL):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    scale = max(np.max(np.abs(ref)), 1e-12)
    err = np.max(np.abs(got - ref)) / scale
    assert err <= rtol, f"{what}: max |d| / max |ref| = {err:.2e} > {rtol:.0e}"


@pytest.fixture(scope="module")
def pool():
    # spawn: workers start clean, with no CUDA state inherited
    p = mp.get_context("spawn").Pool(max(1, min(16, mp.cpu_count())))
    yield p
    p.close()
    p.join()


@pytest.fixture(scope="module")
def grad20():
    return synth.grad20(seed=4, C=100000)


def test_c4_gradients_vs_central_differences(grad20, pool):
    w = grad20
    idx = np.sort(np.random.default_rng(404).choice(w['alignment'].shape[1], 256, replace=False))
    sub = np.ascontiguousarray(w['alignment'][:, idx])
    tree = w['tree']
    assert len(tree.parentIndex) == 399 and w['model'].pi.shape == (20,)
    plan = sg.Plan(tree, w['model'])
    ll, dldt, G = plan.grad(sub)
    plan.close()
    dle = autograd.exchangeability_grad(G, w['log_exch'], w['pi'])
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    assert_loglike(ll, oracle.LogLike(sub, ot, w['model']._asdict()))
    for h, rtol in ((1e-4, FD_RTOL), (1e-6, TIGHT_RTOL)):
        fd_t = oracle.loglike_fd_grad(sub, ot, w['log_exch'], w['pi'], h=h, wrt="distances", pool=pool)
        _close(dldt, fd_t, f"c4 d(sum logL)/dt vs FD h={h}", rtol)
        fd_s = oracle.loglike_fd_grad(sub, ot, w['log_exch'], w['pi'], h=h, wrt="exchangeabilities", pool=pool)
        assert fd_s.shape == (190,)
        _close(dle, fd_s, f"c4 d(sum logL)/dlog s vs FD h={h}", rtol)
    # the Fisher-identity distance gradient of the oracle agrees as well
    _close(dldt, oracle.loglike_distance_grad(sub, ot, w['model']._asdict()), "c4 d/dt vs oracle", rtol=2e-4)


def test_c4_gradient_is_linear_over_column_halves(grad20):
    """Full size (10^5 columns): grad(all) = grad(first half) + grad(second half)."""
    w = grad20
    aln = w['alignment']
    half = aln.shape[1] // 2
    plan = sg.Plan(w['tree'], w['model'])
    _, t_all, G_all = plan.grad(aln)
    _, t_a, G_a = plan.grad(np.ascontiguousarray(aln[:, :half]))
    _, t_b, G_b = plan.grad(np.ascontiguousarray(aln[:, half:]))
    plan.close()
    _close(t_all, t_a + t_b, "d/dt linearity", rtol=1e-4)
    _close(G_all, G_a + G_b, "d/dS linearity", rtol=1e-4)
    assert np.all(np.isfinite(t_all)) and t_all[0] == 0.0


@pytest.mark.parametrize("A,leaves,C,nsub", [(16, 9, 200, None), (64, 6, 160, 128)])
def test_large_alphabet_gradients_vs_central_differences(A, leaves, C, nsub, pool):
    rng = np.random.default_rng(500 + A)
    model, log_exch, pi = models.random_reversible(A, rng, 0.5, 2.0)
    tree = synth.random_tree(leaves, 0.1, rng)
    aln = synth.simulated_alignment(tree, model, C, 0.1, rng)
    plan = sg.Plan(tree, model)
    _, dldt, G = plan.grad(aln)
    plan.close()
    dle = autograd.exchangeability_grad(G, log_exch, pi)
    ot = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    idx = None if nsub is None else np.sort(rng.choice(len(log_exch), nsub, replace=False))
    sel = slice(None) if idx is None else idx
    for h, rtol in ((1e-4, FD_RTOL), (1e-6, TIGHT_RTOL)):
        fd_s = oracle.loglike_fd_grad(aln, ot, log_exch, pi, h=h, wrt="exchangeabilities", idx=idx, pool=pool)
        _close(dle[sel], fd_s[sel], f"A={A} d/dlog s vs FD h={h}", rtol)
        fd_t = oracle.loglike_fd_grad(aln, ot, log_exch, pi, h=h, wrt="distances", pool=pool)
        _close(dldt, fd_t, f"A={A} d/dt vs FD h={h}", rtol)


@pytest.fixture(scope="module")
def precision64():
    w = synth.precision64(seed=3, C=65536)
    idx = np.sort(np.random.default_rng(303).choice(65536, 256, replace=False))
    sub = np.ascontiguousarray(w['alignment'][:, idx])
    ot = oracle.Tree(w['tree'].parentIndex, w['tree'].distanceToParent)
    md = w['model']._asdict()
    ref = {"auto": oracle.Counts(sub, ot, md, branch_mask="auto"),
           None: oracle.Counts(sub, ot, md, branch_mask=None),
           "ll": oracle.LogLike(sub, ot, md), "rp": oracle.RootProb(sub, ot, md)}
    return w, idx, ref


@pytest.mark.parametrize("sel", [0, 2], ids=["split_bf16_tensor_core", "fp32_cuda_core"])
@pytest.mark.parametrize("mask", ["auto", None], ids=["masked", "unmasked"])
def test_c3_full_size_run_vs_oracle_subsample(precision64, sel, mask):
    w, idx, ref = precision64
    d_aln = torch.as_tensor(w['alignment']).cuda()
    lib = _lib.load()
    plan = sg.Plan(w['tree'], w['model'])
    try:
        lib.subby_debug_set_kernel(sel)
        r = plan.run(d_aln, loglike=True, counts=True, rootprob=True, branch_mask=mask)
        torch.cuda.synchronize()
    finally:
        lib.subby_debug_set_kernel(0)
        plan.close()
    ii = torch.as_tensor(idx).cuda()
    assert_loglike(r['logLike'][ii].cpu().numpy(), ref["ll"])
    assert_cols(r['counts'][:, :, ii].cpu().numpy(), ref[mask], COUNTS_RTOL, f"c3 counts mask={mask}")
    assert_cols(r['rootProb'][:, ii].cpu().numpy(), ref["rp"], ROOTPROB_RTOL, "c3 rootProb")


def test_c4_gradient_device_memory_is_bounded_in_the_column_count(grad20):
    """The adjoint's per-branch staging runs in column chunks of about 4 GiB
    at most, so once C passes the chunk size the plan's device memory grows
    only by the uploaded tokens: doubling 2 x 10^5 columns to 4 x 10^5 adds
    the extra alignment and nothing else (and doubles the gradient).  The
    absolute figure at 2 x 10^5 columns is the 4 GiB staging chunk, the
    tokens and the walk's node slots (every internal node of the 399-node
    tree stored, per column of the 304 resident 128-column tiles)."""
    w = grad20
    a2 = np.ascontiguousarray(np.concatenate([w['alignment']] * 2, axis=1))
    a4 = np.ascontiguousarray(np.concatenate([a2, a2], axis=1))
    plan = sg.Plan(w['tree'], w['model'])
    _, t2, G2 = plan.grad(a2)
    b2 = plan.device_bytes()
    _, t4, G4 = plan.grad(a4)
    b4 = plan.device_bytes()
    plan.close()
    assert b2 < (7 << 30), b2
    assert b4 - b2 <= 1.5 * a2.nbytes + (64 << 20), (b2, b4, a2.nbytes)
    _close(t4, 2 * t2, "d/dt of the doubled alignment", rtol=1e-4)
    _close(G4, 2 * G2, "d/dS of the doubled alignment", rtol=1e-4)
