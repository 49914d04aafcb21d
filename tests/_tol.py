"""Tolerances of the parity tests (FP32 GPU path vs the FP64 oracle).

* LogLike: relative error <= 1e-5, measured as |d| / max(1, |ref|) so that
  columns whose log-likelihood is exactly 0 (all-gap) are judged absolutely.
* Counts and root posteriors: per-column norm-wise relative error
  max_ij |d_ijc| / max(max_ij |ref_ijc|, 1e-3) <= 1e-4 (entries can be ~0,
  so per-entry relative error is ill-defined).
* Node and branch posteriors: the same norm-wise measure per (node, column)
  over the states (node) or state pairs (branch), <= 1e-4.
"""
import numpy as np

LOGLIKE_RTOL = 1e-5
COUNTS_RTOL = 1e-4
ROOTPROB_RTOL = 1e-4
POSTERIOR_RTOL = 1e-4


def loglike_err(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    both_inf = np.isinf(got) & np.isinf(ref) & (np.sign(got) == np.sign(ref))
    d = np.where(both_inf, 0.0, np.abs(got - ref))
    return float(np.max(d / np.maximum(1.0, np.abs(np.where(both_inf, 1.0, ref))), initial=0.0))


def colwise_err(got, ref, floor=1e-3):
    """Max over columns of ||got_c - ref_c||_inf / max(||ref_c||_inf, floor); column is last axis."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    C = ref.shape[-1]
    g = got.reshape(-1, C)
    r = ref.reshape(-1, C)
    num = np.max(np.abs(g - r), axis=0, initial=0.0)
    den = np.maximum(np.max(np.abs(r), axis=0, initial=0.0), floor)
    return float(np.max(num / den, initial=0.0))


def assert_loglike(got, ref, tol=LOGLIKE_RTOL, what="logLike"):
    e = loglike_err(got, ref)
    assert e <= tol, f"{what}: relative error {e:.3e} > {tol:.1e}"


def assert_cols(got, ref, tol, what):
    assert np.all(np.isfinite(got)), f"{what}: non-finite values"
    e = colwise_err(got, ref)
    assert e <= tol, f"{what}: column-wise relative error {e:.3e} > {tol:.1e}"
