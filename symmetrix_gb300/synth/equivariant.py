"""Real Clebsch-Gordan tensors and equivariant polynomial bases for synthetic MACE models.

The MACE JSON format stores two equivariant objects that the extractor takes from
e3nn / mace-torch (libsymmetrix's symmetrix/source/symmetrix/extract_mace_data.py):

* the layer-1 tensor-product coupling table (Phi1_clebsch_gordan, Phi1_lme,
  Phi1_lelm1lm2; extract_mace_data.py:345-392), and
* the symmetric-contraction U tensors folded with per-channel weights into
  multivariate polynomials over the 16 A-basis components (M0_*/M1_*;
  extract_mace_data.py:239-304 and :423-474).

Neither e3nn nor mace-torch is available here, so both are derived from the
mathematics in the evaluator's own Y_lm basis: a real CG tensor C^L_{l1 l2} is
the one-dimensional invariant subspace of D_L (x) D_l1 (x) D_l2 (null space over
random rotations), and the degree-nu equivariant polynomial maps R^16 -> V_L are
spanned by the coupling trees ((x_l1 x_l2)_l12 x_l3)_L, orthonormalised in order.
Because everything is derived in the evaluator's basis, energies from a
synthetic model are invariant under O(3) to round-off.
"""
import itertools
from functools import lru_cache

import numpy as np

from .sh import random_rotations, wigner_real


@lru_cache(maxsize=None)
def _wigner_set(l_max=6, n_rot=3, seed=7):
    rng = np.random.default_rng(seed)
    rots = random_rotations(rng, n_rot)
    return [[wigner_real(R, l, np.random.default_rng(100 + l)) for l in range(l_max + 1)] for R in rots]


@lru_cache(maxsize=None)
def real_cg(l1, l2, L):
    """C[M, m1, m2] with C(D1 u, D2 v) = D_L C(u, v); ||C||_F^2 = 2L+1; zero if not a triangle."""
    if not (abs(l1 - l2) <= L <= l1 + l2):
        return np.zeros((2 * L + 1, 2 * l1 + 1, 2 * l2 + 1))
    n = (2 * L + 1) * (2 * l1 + 1) * (2 * l2 + 1)
    rows = []
    for D in _wigner_set(max(l1, l2, L)):
        K = np.kron(np.kron(D[L], D[l1]), D[l2])
        rows.append(K - np.eye(n))
    A = np.concatenate(rows, axis=0)
    _, s, vt = np.linalg.svd(A)
    v = vt[-1]
    if s[-1] > 1e-8 or (len(s) > 1 and s[-2] < 1e-6):
        raise RuntimeError(f"CG null space for ({l1},{l2},{L}) is not one-dimensional")
    v = v / np.linalg.norm(v) * np.sqrt(2 * L + 1)
    first = v[np.argmax(np.abs(v) > 1e-9)]
    v = v * np.sign(first)
    C = v.reshape(2 * L + 1, 2 * l1 + 1, 2 * l2 + 1)
    C[np.abs(C) < 1e-13] = 0.0
    return C


def _block(l):
    return range(l * l, (l + 1) * (l + 1))


def _add(poly, M, key, val):
    if val == 0.0:
        return
    key = tuple(sorted(int(k) for k in key))
    M = int(M)
    poly.setdefault((M, key), 0.0)
    poly[(M, key)] += float(val)


def _candidates(L, degree, l_in_max):
    """Coupling-tree polynomial maps of the given degree, as {(M, monomial): coeff} dicts."""
    out = []
    par_ok = lambda ls: (sum(ls) + L) % 2 == 0
    if degree == 1:
        if L <= l_in_max:
            poly = {}
            for M in range(2 * L + 1):
                _add(poly, M, (L * L + M,), 1.0)
            out.append(poly)
    elif degree == 2:
        for l1 in range(l_in_max + 1):
            for l2 in range(l1, l_in_max + 1):
                if not par_ok((l1, l2)) or not (abs(l1 - l2) <= L <= l1 + l2):
                    continue
                C = real_cg(l1, l2, L)
                poly = {}
                for M, m1, m2 in zip(*np.nonzero(C)):
                    _add(poly, M, (l1 * l1 + m1, l2 * l2 + m2), C[M, m1, m2])
                out.append(poly)
    elif degree == 3:
        for l1 in range(l_in_max + 1):
            for l2 in range(l1, l_in_max + 1):
                for l3 in range(l_in_max + 1):
                    if not par_ok((l1, l2, l3)):
                        continue
                    for l12 in range(abs(l1 - l2), l1 + l2 + 1):
                        if not (abs(l12 - l3) <= L <= l12 + l3):
                            continue
                        C1 = real_cg(l1, l2, l12)
                        C2 = real_cg(l12, l3, L)
                        T = np.einsum("amn,Mac->Mmnc", C1, C2)
                        poly = {}
                        for M, m1, m2, m3 in zip(*np.nonzero(np.abs(T) > 1e-14)):
                            _add(poly, M, (l1 * l1 + m1, l2 * l2 + m2, l3 * l3 + m3), T[M, m1, m2, m3])
                        out.append(poly)
    else:
        raise ValueError("degree must be 1, 2 or 3")
    return out


@lru_cache(maxsize=None)
def equivariant_polynomial_basis(L, degree, l_in_max=3):
    """Orthonormal basis of degree-`degree` polynomial maps x in R^16 -> V_L (parity-respecting).

    Returns (monomials, U) with monomials a tuple of sorted index tuples and
    U[eta, M, t] the coefficient of monomial t in component M of basis map eta.
    """
    cands = _candidates(L, degree, l_in_max)
    if not cands:
        return (), np.zeros((0, 2 * L + 1, 0))
    keys = sorted({k[1] for p in cands for k in p})
    idx = {k: i for i, k in enumerate(keys)}
    A = np.zeros((len(cands), (2 * L + 1) * len(keys)))
    for c, p in enumerate(cands):
        for (M, key), val in p.items():
            A[c, M * len(keys) + idx[key]] = val
    # Ordered modified Gram-Schmidt (twice): unlike an SVD, the basis it returns
    # depends only on the candidate order, so every platform builds the same model.
    basis = []
    # candidates that vanish identically (antisymmetric couplings of equal irreps) have
    # round-off norms; the threshold is absolute on the scale of the largest candidate
    tol = 1e-7 * np.linalg.norm(A, axis=1).max()
    for v in A:
        w = v.copy()
        for _ in range(2):
            for b in basis:
                w -= (b @ w) * b
        nw = np.linalg.norm(w)
        if nw > tol:
            basis.append(w / nw)
    U = np.array(basis).reshape(len(basis), 2 * L + 1, len(keys))
    U[np.abs(U) < 1e-12] = 0.0
    used = np.nonzero(np.any(np.abs(U) > 0, axis=(0, 1)))[0]
    keys = [keys[i] for i in used]
    U = U[:, :, used]
    return tuple(keys), U


def tp_instructions(l_max, L_max):
    """Layer-1 tensor-product instructions (l1 from Y, l2 from H1, l_out), sorted by l_out.

    Mirrors how the extractor reads them off the e3nn convolution tensor product
    (extract_mace_data.py:337-339): only outputs with natural parity (-1)^l and
    l <= l_max are kept, and the instruction list is ordered by output irrep.
    """
    ins = []
    for l2 in range(L_max + 1):
        for l1 in range(l_max + 1):
            for l in range(abs(l1 - l2), min(l1 + l2, l_max) + 1):
                if (l1 + l2 + l) % 2 == 0:
                    ins.append((l1, l2, l))
    ins.sort(key=lambda t: t[2])  # stable: keeps creation order within each l
    return ins


def phi1_tables(l_max, L_max):
    """Phi1_l, Phi1_l1, Phi1_l2, Phi1_lme, Phi1_clebsch_gordan, Phi1_lelm1lm2 in the JSON layout.

    Index conventions follow compute_lme / compute_lelm1lm2 of
    extract_mace_data.py:343-360: Phi1 rows are ordered [l][m][e] and Phi1r rows
    [instruction][m1][m2].
    """
    ins = tp_instructions(l_max, L_max)
    Phi1_l = [t[2] for t in ins]
    Phi1_l1 = [t[0] for t in ins]
    Phi1_l2 = [t[1] for t in ins]
    num_e = [sum(1 for l in Phi1_l if l == ll) for ll in range(l_max + 1)]
    off_l = [sum((2 * ll + 1) * num_e[ll] for ll in range(l)) for l in range(l_max + 1)]
    first_e = [sum(1 for l in Phi1_l if l < ll) for ll in range(l_max + 1)]
    off_p = np.cumsum([0] + [(2 * a + 1) * (2 * b + 1) for a, b, _ in ins]).tolist()
    lme, cg, p_idx = [], [], []
    # enumerate in the extractor's order: (l1, m1), (l2, m2), then instruction, then m
    for l1 in range(l_max + 1):
        for m1 in range(2 * l1 + 1):
            for l2 in range(L_max + 1):
                for m2 in range(2 * l2 + 1):
                    for le, (a, b, l) in enumerate(ins):
                        if a != l1 or b != l2:
                            continue
                        C = real_cg(l1, l2, l)
                        e = le - first_e[l]
                        for m in range(2 * l + 1):
                            v = C[m, m1, m2]
                            if abs(v) > 1e-12:
                                lme.append(off_l[l] + m * num_e[l] + e)
                                cg.append(float(v))
                                p_idx.append(off_p[le] + m1 * (2 * l2 + 1) + m2)
    return dict(Phi1_l=Phi1_l, Phi1_l1=Phi1_l1, Phi1_l2=Phi1_l2, Phi1_lme=lme,
                Phi1_clebsch_gordan=cg, Phi1_lelm1lm2=p_idx), num_e
