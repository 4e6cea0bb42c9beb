"""Seeded synthetic MACE models written in libsymmetrix's JSON model format.

The JSON keys, shapes and index conventions are those that MACE::load_from_json
reads (libsymmetrix/source/mace.cpp:905-1030) and that the extractor writes
(symmetrix/source/symmetrix/extract_mace_data.py:19-519):

* radial functions: 8 Bessel functions x polynomial envelope (p=5) -> random
  SiLU MLP -> one output per (l, channel) for layer 0 and per (instruction,
  channel) for layer 1, tabulated on `num_knots` knots over [1e-12, r_cut] as
  cubic splines with ("not-a-knot", "clamped") end conditions, values and
  first derivatives stored per unordered species pair (extract_mace_data.py:
  142-178);
* linears: N(0, 1/fan_in) weights, with the interaction linears divided by the
  average neighbour count as in extract_mace_data.py:227-237, :479-504;
* symmetric contractions: random per-(species, eta, channel) weights on an
  orthonormal basis of equivariant polynomials (see equivariant.py), folded
  into per-monomial coefficients exactly like extract_mace_data.py:287-304;
* the layer-1 coupling table from real Clebsch-Gordan tensors.

Everything is float64 and reproducible from `seed`.
"""
import json

import numpy as np

from .equivariant import equivariant_polynomial_basis, phi1_tables

CHEMICAL_SYMBOLS = [
    "X", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar",
    "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn"]


def atomic_number(sym):
    return CHEMICAL_SYMBOLS.index(sym)


# Covalent radii (A) by atomic number, Z = 0..30 (Cordero et al., Dalton Trans. 2008, as
# tabulated by ASE; index 0 is ASE's placeholder 0.2).  The ZBL block indexes them by Z
# (zbl.cpp:25-26), as the extractor writes them (extract_mace_data.py:135-136).
COVALENT_RADII = [0.2, 0.31, 0.28, 1.28, 0.96, 0.84, 0.76, 0.71, 0.66, 0.57, 0.58, 1.66, 1.41, 1.21, 1.11,
                  1.07, 1.05, 1.02, 1.06, 2.03, 1.76, 1.70, 1.60, 1.53, 1.39, 1.39, 1.32, 1.26, 1.24, 1.32, 1.22]


def bessel_envelope(r, r_cut, num_bessel=8, p=5):
    """MACE radial embedding: sqrt(2/rc) sin(n pi r/rc)/r times the polynomial envelope."""
    n = np.arange(1, num_bessel + 1)
    b = np.sqrt(2.0 / r_cut) * np.sin(n[None, :] * np.pi * r[:, None] / r_cut) / r[:, None]
    x = r / r_cut
    env = (1.0 - (p + 1.0) * (p + 2.0) / 2.0 * x ** p + p * (p + 2.0) * x ** (p + 1)
           - p * (p + 1.0) / 2.0 * x ** (p + 2))
    env = np.where(r < r_cut, env, 0.0)
    return b * env[:, None]


def _silu(x):
    return x / (1.0 + np.exp(-x))


def _radial_mlp(rng, n_in, hidden, n_out):
    dims = [n_in] + list(hidden) + [n_out]
    return [rng.normal(size=(dims[i], dims[i + 1])) / np.sqrt(dims[i]) for i in range(len(dims) - 1)]


def _apply_mlp(ws, x):
    for w in ws[:-1]:
        x = 1.679 * _silu(x @ w)  # SiLU with the second-moment normalisation e3nn applies
    return x @ ws[-1]


def _spline_tables(r_knots, values):
    """Nodal values and derivatives of ("not-a-knot", "clamped") cubic splines, [n_spl][knot]."""
    from scipy.interpolate import CubicSpline
    spl = CubicSpline(r_knots, values, bc_type=("not-a-knot", "clamped"), axis=0)
    d = spl.derivative()(r_knots)
    return values.T.copy(), d.T.copy()


def make_model(num_channels=32, species=("H", "C", "O"), r_cut=5.0, L_max=1, correlation=3,
               num_bessel=8, envelope_p=5, num_knots=200, avg_num_neighbors=None, seed=0,
               radial_hidden=(64, 64), l_max=3, a0_gain=7.0, a1_gain=12.0, energy_scale=0.35, zbl=False,
               core=(0.8, 1.3), density_scaled=False):
    """Return a dict in libsymmetrix's MACE JSON layout for a random two-layer MACE.

    density_scaled: density-normalised interaction blocks (A0_scaled / A1_scaled,
    libsymmetrix/source/mace.cpp:273-346, :681-757): A is divided by 1 + sum_j s(r_ij)
    with one spline s per unordered species pair and layer, s(r) = w tanh(b(r).v)^2 on
    the Bessel-envelope basis b (non-negative, zero at r_cut, as MACE's density
    blocks); drawn from a separate stream so the other weights equal the unscaled
    model's of the same seed."""
    if l_max != 3:
        raise ValueError("the evaluator supports l_max = 3 only")
    if correlation > 3:
        raise ValueError("polynomial degree above 3 is not supported by the model format")
    rng = np.random.default_rng(seed)
    C = int(num_channels)
    Z = sorted(atomic_number(s) if isinstance(s, str) else int(s) for s in species)
    S = len(Z)
    num_lm = (l_max + 1) ** 2
    num_LM = (L_max + 1) ** 2
    if avg_num_neighbors is None:
        avg_num_neighbors = 0.1 * 4.0 / 3.0 * np.pi * r_cut ** 3
    out = {
        "num_elements": S, "num_channels": C, "r_cut": float(r_cut), "l_max": l_max, "L_max": L_max,
        "atomic_numbers": Z,
        "atomic_energies": rng.normal(size=S).tolist(),
        "has_zbl": bool(zbl),
        "A0_scaled": False, "A1_scaled": False,
    }
    if zbl:
        # MACE's ZBLBasis defaults (p = 6, Ziegler-Biersack-Littmark universal screening)
        out.update({"zbl_a_exp": 0.300, "zbl_a_prefactor": 0.4543,
                    "zbl_c": [0.1818, 0.5099, 0.2802, 0.02817], "zbl_covalent_radii": COVALENT_RADII,
                    "zbl_p": 6})
    phi, num_e = phi1_tables(l_max, L_max)
    n_instr = len(phi["Phi1_l"])

    # ----- radial splines (extract_mace_data.py:142-178) -----
    r_knots, h = np.linspace(1e-12, r_cut, num_knots, retstep=True)
    emb = bessel_envelope(r_knots, r_cut, num_bessel, envelope_p)
    mlp0 = _radial_mlp(rng, num_bessel, radial_hidden, (l_max + 1) * C)
    mlp1 = _radial_mlp(rng, num_bessel, radial_hidden, n_instr * C)
    # A random potential has no repulsive core and grows without bound as pairs close in;
    # the radials are switched off smoothly (C2) inside `core` so that short range is left
    # to the ZBL term and the energy stays bounded below.
    if core:
        xs = np.clip((r_knots - core[0]) / (core[1] - core[0]), 0.0, 1.0)
        damp = (xs ** 3 * (10.0 - 15.0 * xs + 6.0 * xs ** 2))[:, None]
    else:
        damp = 1.0
    base0 = _apply_mlp(mlp0, emb) * damp
    base1 = _apply_mlp(mlp1, emb) * damp
    v0, d0, v1, d1 = [], [], [], []
    for a in range(S):
        for b in range(a, S):
            s0 = 1.0 + 0.25 * rng.normal(size=base0.shape[1])
            s1 = 1.0 + 0.25 * rng.normal(size=base1.shape[1])
            vv, dd = _spline_tables(r_knots, base0 * s0[None, :])
            v0.append(vv.tolist()); d0.append(dd.tolist())
            vv, dd = _spline_tables(r_knots, base1 * s1[None, :])
            v1.append(vv.tolist()); d1.append(dd.tolist())
    out["radial_spline_h"] = float(h)
    out["radial_spline_values_0"] = v0
    out["radial_spline_derivs_0"] = d0
    out["radial_spline_values_1"] = v1
    out["radial_spline_derivs_1"] = d1

    # ----- layer 0 linears (extract_mace_data.py:180-237) -----
    out["H0_weights"] = rng.normal(size=(S, C)).flatten().tolist()
    # 1/sqrt(avg neighbours): random-sign radial sums grow like sqrt(n), keeping A0 = O(1)
    # (a0_gain, a1_gain bring the A-basis to O(1) so that the degree-3 terms matter)
    out["A0_weights"] = [[(a0_gain * rng.normal(size=(C, C)) / np.sqrt(C) / np.sqrt(avg_num_neighbors)).flatten().tolist()
                          for l in range(l_max + 1)] for s in range(S)]

    # ----- symmetric contractions (extract_mace_data.py:239-304, :423-474) -----
    def contraction(L, scale):
        """{species: {M: {k: coeffs}}}, {M: monomials} for output irrep L."""
        bases = [equivariant_polynomial_basis(L, d, l_max) for d in range(1, correlation + 1)]
        weights = [rng.normal(size=(S, U.shape[0], C)) * scale[d] / np.sqrt(max(U.shape[0], 1))
                   for d, (_, U) in enumerate(bases)]
        coeffs, monos = {}, {}
        for M in range(2 * L + 1):
            keys, cols = [], []
            for d, (mono, U) in enumerate(bases):
                for t, key in enumerate(mono):
                    if np.any(U[:, M, t] != 0.0):
                        keys.append(list(key)); cols.append((d, t))
            monos[M] = keys
            for s in range(S):
                c = np.zeros((C, len(keys)))
                for j, (d, t) in enumerate(cols):
                    c[:, j] = weights[d][s].T @ bases[d][1][:, M, t]
                coeffs.setdefault(s, {})[M] = c
        return coeffs, monos

    m0_w, m0_m = {}, {}
    for L in range(L_max + 1):
        coeffs, monos = contraction(L, scale=(1.0, 0.5, 0.25))
        for M in range(2 * L + 1):
            LM = L * L + M
            m0_m[str(LM)] = monos[M]
            for s in range(S):
                m0_w.setdefault(str(s), {})[str(LM)] = {
                    str(k): coeffs[s][M][k].tolist() for k in range(C)}
    out["M0_weights"] = m0_w
    out["M0_monomials"] = m0_m

    # ----- H1 (extract_mace_data.py:306-318) -----
    out["H1_weights"] = np.concatenate(
        [(rng.normal(size=(C, C)) / np.sqrt(C)).flatten() for _ in range(L_max + 1)]).tolist()

    # ----- Phi1 coupling table (extract_mace_data.py:320-392) -----
    out.update(phi)

    # ----- A1 (extract_mace_data.py:394-421) -----
    out["A1_weights"] = [(a1_gain * rng.normal(size=(num_e[l] * C, C)) / np.sqrt(num_e[l] * C)
                          / np.sqrt(avg_num_neighbors)).flatten().tolist() for l in range(l_max + 1)]

    # ----- M1 (extract_mace_data.py:423-474) -----
    coeffs, monos = contraction(0, scale=(1.0, 0.5, 0.25))
    out["M1_weights"] = {str(s): {str(k): coeffs[s][0][k].tolist() for k in range(C)} for s in range(S)}
    out["M1_monomials"] = monos[0]

    # ----- H2 and readouts (extract_mace_data.py:476-519) -----
    out["H2_weights_for_H1"] = [(rng.normal(size=(C, C)) / np.sqrt(C)).flatten().tolist() for _ in range(S)]
    out["H2_weights_for_M1"] = (rng.normal(size=(C, C)) / np.sqrt(C)).flatten().tolist()
    # energy_scale plays the role of MACE's scale_shift.scale, which the extractor
    # multiplies into both readouts (extract_mace_data.py:514, :520)
    out["readout_1_weights"] = (energy_scale * rng.normal(size=C) / np.sqrt(C)).tolist()
    out["readout_2_weights_1"] = (rng.normal(size=(16, C)) / np.sqrt(C)).flatten().tolist()
    out["readout_2_weights_2"] = (energy_scale * rng.normal(size=16) / 4.0).tolist()
    out["readout_2_scale_factor"] = 1.679

    if density_scaled:
        drng = np.random.default_rng(seed + 7919)
        for layer in ("A0", "A1"):
            vals, ders = [], []
            for a in range(S):
                for b in range(a, S):
                    v = drng.normal(size=num_bessel) * 2.0
                    w = 0.05 * (1.0 + drng.random())
                    dens = w * np.tanh(emb @ v) ** 2
                    vv, dd = _spline_tables(r_knots, dens[:, None])
                    vals.append(vv[0].tolist())
                    ders.append(dd[0].tolist())
            out[f"{layer}_scaled"] = True
            out[f"{layer}_spline_h"] = float(h)
            out[f"{layer}_spline_values"] = vals
            out[f"{layer}_spline_derivs"] = ders
    return out


def write_model(model, path):
    with open(path, "w") as f:
        json.dump(model, f)
    return path


# Model shapes of the workloads this engine is measured on.
CONFIGS = {
    # 3 species, 32x0e+32x1o, 64-atom 10 A box (CPU-runnable FP64 case)
    "small": dict(num_channels=32, species=("H", "C", "O"), r_cut=5.0, L_max=1, num_knots=200),
    # 4 species, 128x0e+128x1o, 4096-atom box at 0.10 atoms/A^3
    "fp32_4096": dict(num_channels=128, species=("H", "C", "N", "O"), r_cut=5.0, L_max=1, num_knots=200),
    # 10 species, 128x0e+128x1o+128x2e, r_cut 6
    "bf16_32768": dict(num_channels=128, species=("H", "C", "N", "O", "F", "Na", "Mg", "Al", "Si", "S"),
                       r_cut=6.0, L_max=2, num_knots=200),
    # 10 species, 128x0e+128x1o, the 1,048,576-atom box
    "large_1m": dict(num_channels=128, species=("H", "C", "N", "O", "F", "Na", "Mg", "Al", "Si", "S"), r_cut=5.0,
                     L_max=1, num_knots=200),
    # 7 species, 64x0e+64x1o molecules
    "molecules": dict(num_channels=64, species=("H", "C", "N", "O", "F", "S", "Cl"), r_cut=5.0, L_max=1,
                      num_knots=200),
}
