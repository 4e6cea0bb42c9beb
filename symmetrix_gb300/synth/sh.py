"""Real spherical harmonics (l <= 3) in the convention the MACE evaluator uses.

libsymmetrix evaluates Y_lm by shuffling each edge vector (x, y, z) -> (z, x, y),
calling sphericart's orthonormal real harmonics and scaling by 2*sqrt(pi)
(libsymmetrix/source/mace.cpp:118-148).  The result is e3nn's "component"
normalisation with y as the polar axis: Y_00 = 1 and sum_m Y_lm^2 = 2l+1.

The real harmonics here are the standard orthonormal ones without the
Condon-Shortley phase (Y_1,-1 ~ y, Y_1,0 ~ z, Y_1,1 ~ x), the same convention as
libsymmetrix/source/spherical_harmonic.cpp:38-43 (real_sph_harm_xyz), written as
homogeneous Cartesian polynomials P_lm so that Y_lm(v) = P_lm(v) / |v|^l.

This module is used by the synthetic-model generator to derive Wigner matrices,
Clebsch-Gordan tables and equivariant polynomial bases that are consistent with
the evaluator's Y_lm; it is not on the GPU path.
"""
import numpy as np

_PI = np.pi
_C = {
    "c0": 0.5 / np.sqrt(_PI),
    "c1": np.sqrt(3.0 / (4.0 * _PI)),
    "c2a": 0.5 * np.sqrt(15.0 / _PI),
    "c2b": 0.25 * np.sqrt(5.0 / _PI),
    "c2c": 0.25 * np.sqrt(15.0 / _PI),
    "c3a": 0.25 * np.sqrt(35.0 / (2.0 * _PI)),
    "c3b": 0.5 * np.sqrt(105.0 / _PI),
    "c3c": 0.25 * np.sqrt(21.0 / (2.0 * _PI)),
    "c3d": 0.25 * np.sqrt(7.0 / _PI),
    "c3e": 0.25 * np.sqrt(105.0 / _PI),
}


def real_sh_unit(u, l_max=3):
    """Orthonormal real harmonics of unit vectors u[..., 3] (axes as given), [..., (l_max+1)^2]."""
    X, Y, Z = u[..., 0], u[..., 1], u[..., 2]
    c = _C
    out = [np.full_like(X, c["c0"])]
    if l_max >= 1:
        out += [c["c1"] * Y, c["c1"] * Z, c["c1"] * X]
    if l_max >= 2:
        r2 = X * X + Y * Y + Z * Z
        out += [c["c2a"] * X * Y, c["c2a"] * Y * Z, c["c2b"] * (3 * Z * Z - r2),
                c["c2a"] * X * Z, c["c2c"] * (X * X - Y * Y)]
    if l_max >= 3:
        r2 = X * X + Y * Y + Z * Z
        out += [c["c3a"] * Y * (3 * X * X - Y * Y), c["c3b"] * X * Y * Z,
                c["c3c"] * Y * (5 * Z * Z - r2), c["c3d"] * Z * (5 * Z * Z - 3 * r2),
                c["c3c"] * X * (5 * Z * Z - r2), c["c3e"] * Z * (X * X - Y * Y),
                c["c3a"] * X * (X * X - 3 * Y * Y)]
    return np.stack(out, axis=-1)


def real_sh_unit_general(u, l_max):
    """Same convention as real_sh_unit for any l_max, from the associated-Legendre recurrence.

    P_l^m without the Condon-Shortley phase; Y_l0 = N P_l^0,
    Y_l,+m = sqrt(2) N P_l^m cos(m phi), Y_l,-m = sqrt(2) N P_l^m sin(m phi).
    """
    from math import factorial
    X, Y, Z = u[..., 0], u[..., 1], u[..., 2]
    phi = np.arctan2(Y, X)
    st = np.sqrt(np.maximum(0.0, 1.0 - Z * Z))
    out = np.zeros(u.shape[:-1] + ((l_max + 1) ** 2,))
    P = {}
    for m in range(l_max + 1):
        dfact = 1.0
        for k in range(1, 2 * m, 2):
            dfact *= k
        P[(m, m)] = dfact * st ** m
        if m + 1 <= l_max:
            P[(m + 1, m)] = Z * (2 * m + 1) * P[(m, m)]
        for l in range(m + 2, l_max + 1):
            P[(l, m)] = ((2 * l - 1) * Z * P[(l - 1, m)] - (l + m - 1) * P[(l - 2, m)]) / (l - m)
    for l in range(l_max + 1):
        for m in range(0, l + 1):
            N = np.sqrt((2 * l + 1) / (4 * _PI) * factorial(l - m) / factorial(l + m))
            if m == 0:
                out[..., l * l + l] = N * P[(l, 0)]
            else:
                out[..., l * l + l + m] = np.sqrt(2.0) * N * P[(l, m)] * np.cos(m * phi)
                out[..., l * l + l - m] = np.sqrt(2.0) * N * P[(l, m)] * np.sin(m * phi)
    return out


def sh_e3nn(v, l_max=3):
    """Y_lm of edge vectors v[..., 3] exactly as the evaluator forms them (shuffle, x 2 sqrt(pi))."""
    v = np.asarray(v, dtype=np.float64)
    r = np.linalg.norm(v, axis=-1, keepdims=True)
    u = v / r
    shuffled = np.stack([u[..., 2], u[..., 0], u[..., 1]], axis=-1)
    if l_max <= 3:
        return 2.0 * np.sqrt(_PI) * real_sh_unit(shuffled, l_max)
    return 2.0 * np.sqrt(_PI) * real_sh_unit_general(shuffled, l_max)


def sh_e3nn_grad(v, l_max=3, h=1e-6):
    """Central-difference gradient dY/dv, [..., 3, (l_max+1)^2] (test helper)."""
    v = np.asarray(v, dtype=np.float64)
    g = []
    for a in range(3):
        e = np.zeros(3)
        e[a] = h
        g.append((sh_e3nn(v + e, l_max) - sh_e3nn(v - e, l_max)) / (2 * h))
    return np.stack(g, axis=-2)


def random_rotations(rng, n, improper=False):
    """n random orthogonal 3x3 matrices (det +1, or -1 for half when improper)."""
    out = []
    for i in range(n):
        q, r = np.linalg.qr(rng.normal(size=(3, 3)))
        q = q * np.sign(np.diag(r))
        if np.linalg.det(q) < 0:
            q[:, 0] = -q[:, 0]
        if improper and i % 2 == 1:
            q = -q
        out.append(q)
    return out


def wigner_real(R, l, rng=None):
    """Real Wigner matrix D_l(R) with Y_l(R v) = D_l(R) Y_l(v) for the evaluator's Y_lm."""
    if rng is None:
        rng = np.random.default_rng(1234)
    pts = rng.normal(size=(4 * (2 * l + 1) + 8, 3))
    sl = slice(l * l, (l + 1) * (l + 1))
    Y0 = sh_e3nn(pts, l)[:, sl]
    Y1 = sh_e3nn(pts @ R.T, l)[:, sl]
    DT, *_ = np.linalg.lstsq(Y0, Y1, rcond=None)
    return DT.T
