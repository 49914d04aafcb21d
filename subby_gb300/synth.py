"""Seeded synthetic workloads (trees, models, simulated alignments).

No public dataset is involved: every workload is generated here from a fixed
seed.  The recipes follow the five workload definitions of this backend:

* ``plain_small``   A=4 HKY85 (kappa=2, pi~Dir(1^4)), 16 leaves (R=31),
                    Exp(mean 0.1) branches, C=1024, leaves uniform over 4
                    states with 5% unobserved cells split evenly between
                    tokens A and A+1, internal rows token A.
* ``plain_large``   A=4 HKY85 and F81, 128 leaves (R=255), Exp(mean 0.05),
                    C=2^20 simulated down the tree, 10% gaps.
* ``precision64``   A=64 random reversible (s~LogNormal(0,1), pi~Dir(1^64))
                    with ~5% of the eigenvalue pairs within 1e-7 (an
                    exchangeable block, see models.near_degenerate_reversible),
                    64 leaves (R=127), Exp(mean 0.1), C=65536 simulated.
* ``grad20``        A=20 random reversible (s~LogNormal(0,0.5),
                    pi~Dir(2^20)), 200 leaves (R=399), Exp(mean 0.08),
                    C=100000 simulated, 15% gaps.
* ``serving``       job stream, see ``serving_jobs``.

Tree recipe: start from one leaf, repeatedly split a uniformly chosen leaf
into two children until L leaves exist, then number the nodes in DFS
preorder with children in creation order, so ``parentIndex[n] < n``.
"""
from __future__ import annotations

import numpy as np

from .types import Tree, DiagModel
from . import models as _models


def random_tree(n_leaves: int, mean_branch: float, rng: np.random.Generator) -> Tree:
    if n_leaves < 1:
        raise ValueError("n_leaves must be >= 1")
    children = {0: []}
    leaves = [0]
    nxt = 1
    while len(leaves) < n_leaves:
        k = int(rng.integers(len(leaves)))
        v = leaves[k]
        a, b = nxt, nxt + 1
        nxt += 2
        children[v] = [a, b]
        children[a] = []
        children[b] = []
        leaves[k] = a
        leaves.append(b)
    # DFS preorder renumbering
    order = []
    stack = [0]
    while stack:
        v = stack.pop()
        order.append(v)
        stack.extend(reversed(children[v]))
    new = {v: i for i, v in enumerate(order)}
    R = len(order)
    parent = np.full(R, -1, dtype=np.int32)
    for v, ch in children.items():
        for c in ch:
            parent[new[c]] = new[v]
    dist = rng.exponential(mean_branch, size=R)
    dist[0] = 0.0
    return Tree(parent, dist.astype(np.float64))


def sub_matrices64(model: DiagModel, distances) -> np.ndarray:
    if hasattr(model, 'eigenvectors_inv'):
        # irreversible: M = Re V diag(e^{mu t}) V^-1
        V = np.asarray(model.eigenvectors, dtype=np.complex128)
        Vi = np.asarray(model.eigenvectors_inv, dtype=np.complex128)
        E = np.exp(np.asarray(model.eigenvalues, np.complex128)[None, :] * np.asarray(distances)[:, None])
        M = np.maximum(np.einsum('ik,rk,kj->rij', V, E, Vi).real, 0.0)
        return M / M.sum(axis=-1, keepdims=True)
    V = np.asarray(model.eigenvectors, dtype=np.float64)
    mu = np.asarray(model.eigenvalues, dtype=np.float64)
    sp = np.sqrt(np.asarray(model.pi, dtype=np.float64))
    E = np.exp(mu[None, :] * np.asarray(distances)[:, None])
    S = np.einsum('ik,rk,jk->rij', V, E, V)
    M = S / sp[None, :, None] * sp[None, None, :]
    M = np.maximum(M, 0.0)
    return M / M.sum(axis=-1, keepdims=True)


def simulate_states(tree: Tree, model: DiagModel, C: int, rng: np.random.Generator) -> np.ndarray:
    """States at every node, (R, C) int32: root ~ pi, child ~ row of M(t).

    Inverse-CDF sampling with FP64 transition rows (rounded to FP32
    thresholds): child = #{k < A-1 : u >= cumM[parent_state, k]}.
    """
    pi = np.asarray(model.pi, dtype=np.float64)
    A = len(pi)
    R = len(tree.parentIndex)
    M = sub_matrices64(model, tree.distanceToParent)
    cumM = np.cumsum(M, axis=-1).astype(np.float32)
    cumM[..., -1] = 1.0
    st_dtype = np.int8 if A <= 127 else np.int16
    states = np.empty((R, C), dtype=st_dtype)
    cpi = np.cumsum(pi).astype(np.float32)
    cpi[-1] = 1.0
    u = rng.random(C, dtype=np.float32)
    states[0] = np.searchsorted(cpi, u, side='right').clip(0, A - 1)
    for n in range(1, R):
        p = tree.parentIndex[n]
        u = rng.random(C, dtype=np.float32)
        sp = states[p]
        out = np.zeros(C, dtype=st_dtype)
        cn = cumM[n]
        for k in range(A - 1):
            out += (u >= cn[:, k][sp])
        states[n] = out
    return states.astype(np.int32)


def leaf_mask(tree: Tree) -> np.ndarray:
    R = len(tree.parentIndex)
    cnt = np.zeros(R, dtype=np.int64)
    np.add.at(cnt, np.asarray(tree.parentIndex[1:]), 1)
    return cnt == 0


def simulated_alignment(tree: Tree, model: DiagModel, C: int, gap_rate: float,
                        rng: np.random.Generator, unobserved_split: bool = False) -> np.ndarray:
    """Leaves keep simulated states, internal rows get token A, a fraction
    ``gap_rate`` of leaf cells become A+1 (or, with ``unobserved_split``,
    A or A+1 with equal probability)."""
    A = len(model.pi)
    aln = simulate_states(tree, model, C, rng)
    leaf = leaf_mask(tree)
    aln[~leaf] = A
    g = rng.random(aln.shape, dtype=np.float32) < gap_rate
    g &= leaf[:, None]
    if unobserved_split:
        half = rng.random(aln.shape, dtype=np.float32) < 0.5
        aln[g & half] = A
        aln[g & ~half] = A + 1
    else:
        aln[g] = A + 1
    return aln


# ---------------------------------------------------------------------------
# Named workloads
# ---------------------------------------------------------------------------

def plain_small(seed: int = 1, C: int = 1024):
    rng = np.random.default_rng(seed)
    pi = rng.dirichlet(np.ones(4))
    model = _models.hky85_diag(2.0, pi)
    tree = random_tree(16, 0.1, rng)
    leaf = leaf_mask(tree)
    R = len(tree.parentIndex)
    aln = rng.integers(0, 4, size=(R, C)).astype(np.int32)
    aln[~leaf] = 4
    g = (rng.random((R, C)) < 0.05) & leaf[:, None]
    half = rng.random((R, C)) < 0.5
    aln[g & half] = 4
    aln[g & ~half] = 5
    return dict(name="plain_small", alignment=aln, tree=tree, model=model, A=4, seed=seed)


def plain_large(seed: int = 2, C: int = 1 << 20, f81: bool = False):
    rng = np.random.default_rng(seed)
    pi = rng.dirichlet(np.ones(4))
    tree = random_tree(128, 0.05, rng)
    model = _models.f81_model(pi) if f81 else _models.hky85_diag(2.0, pi)
    arng = np.random.default_rng(seed * 1000 + (7 if f81 else 3))
    aln = simulated_alignment(tree, model, C, 0.10, arng)
    return dict(name="plain_large_f81" if f81 else "plain_large", alignment=aln, tree=tree,
                model=model, A=4, seed=seed)


def precision64(seed: int = 3, C: int = 65536, A: int = 64, n_leaves: int = 64):
    rng = np.random.default_rng(seed)
    model, log_exch, pi, pairs = _models.near_degenerate_reversible(A, rng)
    tree = random_tree(n_leaves, 0.1, rng)
    aln = simulated_alignment(tree, model, C, 0.0, rng)
    return dict(name="precision64", alignment=aln, tree=tree, model=model, A=A, seed=seed,
                forced_pairs=pairs, log_exch=log_exch, pi=pi)


def grad20(seed: int = 4, C: int = 100000, n_leaves: int = 200):
    rng = np.random.default_rng(seed)
    model, log_exch, pi = _models.random_reversible(20, rng, 0.5, 2.0)
    tree = random_tree(n_leaves, 0.08, rng)
    aln = simulated_alignment(tree, model, C, 0.15, rng)
    return dict(name="grad20", alignment=aln, tree=tree, model=model, A=20, seed=seed,
                log_exch=log_exch, pi=pi)


def serving_jobs(n_jobs: int = 10000, rate: float = 200.0, seed: int = 5,
                 max_columns: int = 200000, min_columns: int = 100,
                 min_leaves: int = 8, max_leaves: int = 512):
    """Job descriptors of the serving stream (lazy: tokens made on demand).

    Poisson arrivals at ``rate`` jobs/s; leaves and C log-uniform integers;
    A uniform over {4 (HKY85), 16 (random reversible), 64 (F81 fast path or
    random reversible, 50/50)}.  Each job carries its own seed.
    """
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n_jobs))
    jobs = []
    for i in range(n_jobs):
        leaves = int(np.exp(rng.uniform(np.log(min_leaves), np.log(max_leaves + 1))))
        C = int(np.exp(rng.uniform(np.log(min_columns), np.log(max_columns + 1))))
        A = int(rng.choice([4, 16, 64]))
        kind = "hky85" if A == 4 else ("reversible" if A == 16 else
                                      ("f81" if rng.random() < 0.5 else "reversible"))
        jobs.append(dict(id=i, arrival=float(t[i]), leaves=max(2, min(leaves, max_leaves)),
                         C=max(min_columns, min(C, max_columns)), A=A, kind=kind,
                         seed=int(rng.integers(1 << 31))))
    return jobs


def materialize_job(job):
    """Tree, model and simulated tokens of one serving job."""
    rng = np.random.default_rng(job['seed'])
    A = job['A']
    if job['kind'] == 'hky85':
        model = _models.hky85_diag(2.0, rng.dirichlet(np.ones(4)))
    elif job['kind'] == 'f81':
        model = _models.f81_model(rng.dirichlet(np.ones(A)))
    else:
        model, _, _ = _models.random_reversible(A, rng, 1.0, 1.0)
    tree = random_tree(job['leaves'], 0.1, rng)
    aln = simulated_alignment(tree, model, job['C'], 0.05, rng)
    return aln, tree, model
