"""CPU emulation of the tree program run by k_tree.cu (no GPU needed).

The host compiles the tree into steps over STORED nodes (a per-column slot
holds their child contribution CC = M U) while DERIVED nodes (children are
leaves or stored) are recomputed on demand.  This test re-implements the
classification rule and the kernel's inside/outside step logic (power-of-two
rescaling, derived nodes processed inline, Steiner mask bits, D written over
dead CC slots) in FP64 numpy and checks LogLike, Counts (masked and
unmasked, eigen and F81) and RootProb against the oracle, so the algorithm
the CUDA kernel transcribes is validated independently of the GPU.
"""
import numpy as np
import pytest

import oracle
from tests import _golden
from tests._tol import assert_cols, assert_loglike
from subby_gb300 import synth


def children(parent):
    R = len(parent)
    left = np.full(R, -1)
    right = np.full(R, -1)
    for n in range(1, R):
        p = parent[n]
        if left[p] < 0:
            left[p] = n
        else:
            right[p] = n
    return left, right


def postorder(left, right):
    out, st = [], [(0, 0)]
    while st:
        v, s = st.pop()
        if left[v] < 0:
            continue
        if s == 0:
            st += [(v, 1), (left[v], 0)]
        elif s == 1:
            st += [(v, 2), (right[v], 0)]
        else:
            out.append(v)
    return out


def compile_program(parent):
    left, right = children(parent)
    order = postorder(left, right)
    kind = {n: -1 for n in range(len(parent))}   # -1 leaf, -2 derived, -3 root, >=0 slot
    ns = 0
    for v in order:
        if v == 0:
            kind[v] = -3
            continue
        ok = all(kind[c] == -1 or kind[c] >= 0 for c in (left[v], right[v]))
        if ok:
            kind[v] = -2
        else:
            kind[v] = ns
            ns += 1
    steps = [v for v in order if v == 0 or kind[v] >= 0]
    return steps, kind, left, right, ns


def frexp2(v):
    m = np.max(v)
    if not m > 0:
        return v, 0
    e = int(np.floor(np.log2(m)))
    return v * 2.0 ** (-e), e


def run_column(tokens, parent, dist, model, mask_mode, f81):
    """One column through the emulated program; returns (logL, counts, rootprob)."""
    A = len(model['pi'])
    pi = np.asarray(model['pi'])
    V = np.asarray(model['eigenvectors'])
    mu = np.asarray(model['eigenvalues'])
    M = oracle.compute_sub_matrices(model, dist)
    J = oracle.compute_J(mu, dist)
    sp = np.sqrt(pi)
    steps, kind, left, right, ns = compile_program(parent)
    code = lambda n: tokens[n] if 0 <= tokens[n] < A else A          # noqa: E731
    ungapped = lambda n: int(0 <= tokens[n] <= A)                     # noqa: E731
    L = lambda n: (np.eye(A)[code(n)] if code(n) < A else np.ones(A))  # noqa: E731
    slots = [None] * ns

    def basic(n):
        if kind[n] == -1:
            return dict(cc=M[n] @ L(n), e=0, h=ungapped(n), init=ungapped(n), leaf=True)
        s = slots[kind[n]]
        return dict(cc=s['v'], e=s['e'], h=s['h'], init=s['init'], leaf=False)

    def derive(n):
        kl, kr = basic(left[n]), basic(right[n])
        u, e = frexp2(kl['cc'] * kr['cc'] * L(n))
        return dict(cc=M[n] @ u, e=kl['e'] + kr['e'] + e, h=kl['h'] | kr['h'],
                    init=kl['h'] & kr['h'], leaf=False, u=u, kids=(kl, kr))

    def child(n):
        return derive(n) if kind[n] == -2 else basic(n)

    root_u, eroot, iroot = None, 0, 0
    if len(parent) == 1:
        root_u = L(0)
    for p in steps:
        cl, cr = child(left[p]), child(right[p])
        u, e = frexp2(cl['cc'] * cr['cc'] * L(p))
        eU = cl['e'] + cr['e'] + e
        if p == 0:
            root_u, eroot, iroot = u, eU, cl['h'] & cr['h']
        else:
            slots[kind[p]] = dict(v=M[p] @ u, e=eU, h=cl['h'] | cr['h'], init=cl['h'] & cr['h'])
    P = float(pi @ root_u)
    logL = eroot * np.log(2.0) + np.log(P)
    rp = pi * root_u / P
    if not steps:
        return logL, np.zeros((A, A)), rp
    C = np.zeros((A, A))
    f81acc = np.zeros((A, A))
    mu81 = 1.0 / (1.0 - np.sum(pi ** 2))

    def branch(n, D, U, eDU, act):
        s = (2.0 ** (eDU - eroot) / P) if act else 0.0
        if f81:
            t = dist[n]
            ee = np.exp(-mu81 * t)
            a, b, g = t * ee, (1 - ee) / mu81 - t * ee, t * (1 + ee) - 2 * (1 - ee) / mu81
            Ds = D * s
            piU, Dsum = pi @ U, Ds.sum()
            f81acc[:] += a * np.outer(Ds, U) + b * (np.outer(Ds, np.full(A, piU)) + np.outer(pi, Dsum * U)) \
                + g * np.outer(pi, np.full(A, Dsum * piU))
            return
        Ut = (U * sp) @ V
        Dt = (D / sp) @ V
        C[:] += np.outer(Dt * s, Ut) * J[n]

    def active(n, stn, stp):
        if mask_mode == 'auto':
            return stn & stp
        return 1

    for p in reversed(steps):
        cl, cr = child(left[p]), child(right[p])
        if p == 0:
            O, eO, stp = pi * L(0), 0, iroot
        else:
            s = slots[kind[p]]
            D, eD, stp, actp = s['v'], s['eD'], s['st'], s['act']
            U, e = frexp2(cl['cc'] * cr['cc'] * L(p))
            branch(p, D, U, eD + cl['e'] + cr['e'] + e, actp)
            O, e2 = frexp2((D @ M[p]) * L(p))
            eO = eD + e2
        for me, sib, n in ((cl, cr, left[p]), (cr, cl, right[p])):
            Dc = O * sib['cc']
            eDc = eO + sib['e']
            stc = me['init'] | (stp & me['h'])
            actc = active(n, stc, stp)
            if kind[n] == -1:
                branch(n, Dc, L(n), eDc, actc)
            elif kind[n] >= 0:
                slots[kind[n]] = dict(v=Dc, eD=eDc, st=stc, act=actc)
            else:
                branch(n, Dc, me['u'], eDc + me['e'], actc)
                Oc, e3 = frexp2((Dc @ M[n]) * L(n))
                eOc = eDc + e3
                for g, gs, gn in ((me['kids'][0], me['kids'][1], left[n]),
                                  (me['kids'][1], me['kids'][0], right[n])):
                    Dg = Oc * gs['cc']
                    eDg = eOc + gs['e']
                    stg = g['init'] | (stc & g['h'])
                    actg = active(gn, stg, stc)
                    if kind[gn] == -1:
                        branch(gn, Dg, L(gn), eDg, actg)
                    else:
                        slots[kind[gn]] = dict(v=Dg, eD=eDg, st=stg, act=actg)
    if f81:
        off = ~np.eye(A, dtype=bool)
        return logL, np.where(off, mu81 * pi[None, :] * f81acc, f81acc), rp
    S = (V * mu) @ V.T
    VCV = V @ C @ V.T
    return logL, np.where(np.eye(A, dtype=bool), VCV, S * VCV), rp


def emulate(aln, parent, dist, model, mask_mode='none', f81=False):
    out = [run_column(aln[:, c], parent, dist, model, mask_mode, f81) for c in range(aln.shape[1])]
    return (np.array([o[0] for o in out]), np.stack([o[1] for o in out], axis=-1),
            np.stack([o[2] for o in out], axis=-1))


def _check(aln, parent, dist, model, f81=False):
    t = oracle.Tree(parent, dist)
    for mm in ('none', 'auto'):
        ll, cnt, rp = emulate(aln, parent, dist, model, mm, f81)
        assert_loglike(ll, oracle.LogLike(aln, t, model), tol=1e-12)
        ref = oracle.Counts(aln, t, model, f81_fast=f81, branch_mask=None if mm == 'none' else 'auto')
        assert_cols(cnt, ref, 1e-10, f"counts mask={mm} f81={f81}")
        assert_cols(rp, oracle.RootProb(aln, t, model), 1e-12, "rootprob")


@pytest.mark.parametrize("name", [n for n in _golden.names()
                                  if int(_golden.load(n)['A']) <= 8 and "eigenvectors_inv" not in _golden.load(n)])
def test_program_matches_oracle_on_golden(name):
    g = _golden.load(name)
    model = {k: g[k] for k in ('eigenvalues', 'eigenvectors', 'pi')}
    _check(g['alignment'][:, :24], g['parentIndex'], g['distanceToParent'], model,
           f81='counts_f81' in g)


def test_program_on_random_trees():
    rng = np.random.default_rng(21)
    from subby_gb300 import models
    m = models.hky85_diag(2.0, [0.3, 0.2, 0.3, 0.2])
    md = m._asdict()
    for leaves in (1, 2, 3, 5, 9, 40):
        tr = synth.random_tree(leaves, 0.1, rng)
        aln = synth.simulated_alignment(tr, m, 6, 0.2, rng)
        _check(aln, tr.parentIndex, tr.distanceToParent, md)
    # BFS-numbered balanced tree
    R = 15
    parent = np.array([-1] + [(i - 1) // 2 for i in range(1, R)])
    aln = rng.integers(-1, 6, size=(R, 5))
    _check(aln, parent, rng.uniform(0.01, 0.5, R) * (np.arange(R) > 0), md)


def test_stored_fraction_on_the_large_workload_tree():
    tr = synth.random_tree(128, 0.05, np.random.default_rng(2))
    steps, kind, left, right, ns = compile_program(tr.parentIndex)
    assert ns < 70 and len(steps) == ns + 1
