"""Host side of the batched-model API (no GPU): model-kind detection,
rate categories and scale_model against the reference oracle's fixtures,
and the first-model root-prior identity used for per-column model lists."""
import os

import numpy as np
import pytest

import oracle
from subby_gb300 import batch, models


def test_kind():
    m = models.hky85_diag(2.0, [0.25] * 4)
    assert batch.kind(m) == 'single'
    assert batch.kind(models.scale_model(m, np.array([0.5, 1.0]))) == 'H'
    assert batch.kind([m, m]) == 'list'
    assert batch.kind([[m, m]]) == 'grid'
    with pytest.raises(ValueError):
        batch.kind([])


def test_gamma_and_scale_model_match_fixtures():
    with np.load(os.path.join(os.path.dirname(__file__), "golden", "mixture", "gamma_categories.npz")) as z:
        for a, r in zip(z['alpha'], z['rates']):
            got, w = models.gamma_rate_categories(float(a), 4)
            np.testing.assert_allclose(got, r, rtol=1e-13)
            np.testing.assert_allclose(w, 0.25)
    m = models.hky85_diag(2.0, [0.1, 0.2, 0.3, 0.4])
    b = models.scale_model(m, np.array([0.5, 2.0]))
    assert b.eigenvalues.shape == (2, 4) and b.eigenvectors.shape == (2, 4, 4)
    H, ms = models.unbatch(b)
    assert H == (2,)
    np.testing.assert_allclose(ms[1].eigenvalues, 2.0 * np.asarray(m.eigenvalues))


def test_root_prior_identity():
    """LogLike with root prior pi0 = LogLike with pi_g + log sum_a q_a pi0_a/pi_g,a
    (q the RootProb under pi_g) — the identity batch.loglike_list applies."""
    rng = np.random.default_rng(1)
    tree = oracle.Tree([-1, 0, 0, 1, 1], [0, 0.2, 0.3, 0.1, 0.4])
    aln = rng.integers(0, 6, size=(5, 30)).astype(np.int32)
    mg = oracle.hky85_diag(2.0, [0.1, 0.2, 0.3, 0.4])
    pi0 = np.array([0.4, 0.3, 0.2, 0.1])
    M = oracle.compute_sub_matrices(mg, tree.distanceToParent)
    ll0 = oracle.upward_pass(aln, tree, M, pi0)[2]
    llg = oracle.LogLike(aln, tree, mg)
    q = oracle.RootProb(aln, tree, mg)
    np.testing.assert_allclose(ll0, llg + np.log(batch._ratio_to_root0(q, mg['pi'], pi0)), atol=1e-12)
    np.testing.assert_allclose(oracle.LogLike_per_column(aln, tree, [mg] * 30), llg, atol=1e-12)


def test_column_groups_by_model():
    a = models.hky85_diag(2.0, [0.25] * 4)
    b = models.hky85_diag(3.0, [0.1, 0.2, 0.3, 0.4])
    aln = np.zeros((5, 6), dtype=np.int32)
    ms, groups = batch._groups(aln, [a, b, a, a, b, a])
    assert [idx for _, idx in groups] == [[0, 2, 3, 5], [1, 4]]
    with pytest.raises(ValueError):
        batch._groups(aln, [a, b])
    with pytest.raises(NotImplementedError):
        batch._groups(aln[:, :2], [models.scale_model(a, np.array([1.0, 2.0])), a])


def test_take_and_put_numpy():
    x = np.arange(20, dtype=np.float32).reshape(4, 5)
    sub = batch._take(x, [1, 3])
    np.testing.assert_array_equal(sub, x[:, [1, 3]])
    out = np.zeros((4, 5), np.float32)
    batch._put(out, [1, 3], sub)
    np.testing.assert_array_equal(out[:, [1, 3]], sub)


def test_request_models():
    from subby_gb300 import io
    m, alpha = io._parse_model({"name": "jukes-cantor", "alphabetSize": 4, "alphabet": list("ACGT")})
    assert alpha == list("ACGT") and np.allclose(m.pi, 0.25)
    m, _ = io._parse_model({"name": "HKY_85", "kappa": 2, "pi": [0.1, 0.2, 0.3, 0.4]})
    assert type(m).__name__ == "DiagModel"
    Q = np.array([[-1.0, 0.5, 0.5], [0.5, -1.0, 0.5], [0.5, 0.5, -1.0]])
    m, _ = io._parse_model({"subRate": Q.tolist(), "rootProb": [1 / 3] * 3})
    assert type(m).__name__ == "DiagModel"            # detailed balance holds
    m, _ = io._parse_model({"subRate": Q.tolist(), "rootProb": [1 / 3] * 3, "reversible": False})
    assert type(m).__name__ == "IrrevDiagModel"
    with pytest.raises(ValueError):
        io._parse_model({"name": "gtr"})
    with pytest.raises(ValueError):
        io._parse_alignment(["AC", "GT"], None)
    assert io._parse_alignment([["A", "-"], ["G", "T"]], list("ACGT")).tolist() == [[0, 5], [2, 3]]
