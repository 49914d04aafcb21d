"""Generate tests/golden/models/constructors.npz from the REFERENCE model constructors.

    python tests/golden/make_models_golden.py [--reference /root/reference]

Runs subby/oracle/oracle.py's hky85_diag, jukes_cantor_model, f81_model,
diagonalize_rate_matrix, diagonalize_irreversible, check_detailed_balance,
model_from_rate_matrix and gy94_model on seeded inputs and stores their outputs
(eigenvalues, eigenvectors, eigenvectors_inv, pi) and the inputs; and
ExpectedCounts on a few models (models/expected_counts.npz).
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    from subby.oracle import oracle as ro   # noqa: E402  (reference)
    rng = np.random.default_rng(404)
    out = {}

    def put(name, m, **inputs):
        for k in ("eigenvalues", "eigenvectors", "eigenvectors_inv", "pi"):
            if k in m:
                out[f"{name}/{k}"] = np.asarray(m[k])
        for k, v in inputs.items():
            out[f"{name}/in_{k}"] = np.asarray(v)

    for i, (kappa, pi) in enumerate([(2.0, [0.25] * 4), (4.0, [0.295, 0.205, 0.205, 0.295]),
                                     (0.7, rng.dirichlet(np.ones(4)))]):
        put(f"hky{i}", ro.hky85_diag(kappa, np.asarray(pi)), kappa=kappa, pi=pi)
    for A in (2, 4, 20, 64):
        put(f"jc{A}", ro.jukes_cantor_model(A), A=A)
    for A in (4, 20):
        pi = rng.dirichlet(np.ones(A))
        put(f"f81_{A}", ro.f81_model(pi), pi=pi)
    for A in (4, 20):
        pi = rng.dirichlet(2 * np.ones(A))
        S = rng.lognormal(size=(A, A))
        S = S + S.T
        Q = S * pi[None, :]
        np.fill_diagonal(Q, 0.0)
        np.fill_diagonal(Q, -Q.sum(1))
        put(f"rev{A}", ro.diagonalize_rate_matrix(Q, pi), Q=Q, pi=pi)
        put(f"auto_rev{A}", ro.model_from_rate_matrix(Q, pi), Q=Q, pi=pi)
        N = rng.uniform(0.1, 1.0, size=(A, A))
        np.fill_diagonal(N, 0.0)
        np.fill_diagonal(N, -N.sum(1))
        w, v = np.linalg.eig(N.T)
        st = np.real(v[:, np.argmin(np.abs(w))])
        st = st / st.sum()
        put(f"irrev{A}", ro.diagonalize_irreversible(N, st), Q=N, pi=st)
        if A == 4:
            irrev4 = ro.diagonalize_irreversible(N, st)
        put(f"auto_irrev{A}", ro.model_from_rate_matrix(N, st), Q=N, pi=st)
        out[f"balance/rev{A}"] = np.asarray(ro.check_detailed_balance(Q, pi))
        out[f"balance/irrev{A}"] = np.asarray(ro.check_detailed_balance(N, st))
    os.makedirs(os.path.join(HERE, "models"), exist_ok=True)
    for i, (omega, kappa, pi) in enumerate([(0.3, 2.0, None), (1.7, 0.5, rng.dirichlet(np.ones(61)))]):
        put(f"gy94_{i}", ro.gy94_model(omega, kappa, pi), omega=omega, kappa=kappa,
            pi=np.full(61, 1.0 / 61) if pi is None else pi)
    np.savez_compressed(os.path.join(HERE, "models", "constructors.npz"), **out)
    print(f"wrote models/constructors.npz ({len(out)} arrays)")

    # ExpectedCounts (single-branch CTMC integrals), oracle.py:1909-2105
    ec = {}
    pi6 = rng.dirichlet(np.ones(6))
    S6 = rng.lognormal(size=(6, 6))
    Q6 = (S6 + S6.T) * pi6[None, :]
    np.fill_diagonal(Q6, 0.0)
    np.fill_diagonal(Q6, -Q6.sum(1))
    N5 = rng.uniform(0.1, 1.0, size=(5, 5))
    np.fill_diagonal(N5, 0.0)
    np.fill_diagonal(N5, -N5.sum(1))
    cases = [("hky", ro.hky85_diag(2.0, np.array([0.1, 0.2, 0.3, 0.4])), 0.3),
             ("jc", ro.jukes_cantor_model(4), 1.0),
             ("rev6", ro.diagonalize_rate_matrix(Q6, pi6), 0.7),
             ("irrev4", irrev4, 0.5),
             ("irrev5", ro.diagonalize_irreversible(N5, np.full(5, 0.2)), 0.2)]
    for name, m, t in cases:
        for k in ("eigenvalues", "eigenvectors", "eigenvectors_inv", "pi"):
            if k in m:
                ec[f"{name}/{k}"] = np.asarray(m[k])
        ec[f"{name}/t"] = np.asarray(t)
        ec[f"{name}/expected"] = ro.ExpectedCounts(m, t)
    np.savez_compressed(os.path.join(HERE, "models", "expected_counts.npz"), **ec)
    print(f"wrote models/expected_counts.npz ({len(ec)} arrays)")


if __name__ == "__main__":
    main()
