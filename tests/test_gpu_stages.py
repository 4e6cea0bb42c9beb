"""Per-stage calls and writable stage buffers on the GPU, checked the way the reference
checks its stages (symmetrix/test/test_mace.py:73-84, 260-424): the adjoint of a stage,
seeded with ones, against the central finite difference of the sum of its forward
outputs.

The engine computes in float32, so the steps differ from the reference's h = 1e-4:
the stages that are linear in the perturbed input (H1 in M0, A1 in Phi1, Phi1 in H1)
are differenced with h = 0.5, exact up to the float32 rounding of the outputs, and
checked to 1e-4 of the gradient's scale; Phi1 as a function of the edge vectors (with
its radials and spherical harmonics) with h = 1e-3, to 2e-3 of the scale.  Stage
buffers after a full evaluation also match the oracle's, and a stage run on the
evaluation's own buffers reproduces them.
"""
import numpy as np
import pytest

from helpers import edge_args
from oracle.pyoracle import Evaluator
from symmetrix_gb300.synth.structures import neighbor_list, random_box

pytestmark = pytest.mark.gpu


def numerical_gradient(f, x, h, idx):
    """Central differences of f at the entries idx of x (the reference's numerical_gradient,
    symmetrix/test/test_mace.py:73-84, on a subset of the entries)."""
    x = np.array(x, dtype=np.float64)
    g = np.zeros(len(idx))
    for q, i in enumerate(idx):
        x0 = x[i]
        x[i] = x0 + h
        fp = f(x)
        x[i] = x0 - h
        fm = f(x)
        x[i] = x0
        g[q] = (fp - fm) / (2 * h)
    f(x)
    return g


@pytest.fixture(scope="module")
def setup(engine_lib, small_model_path):
    from symmetrix_gb300 import MACE
    pos, L, species = random_box(12, 0.05, 1.0, 3, seed=31)
    nl = neighbor_list(pos, 4.5, L)  # edges below 4.5 A: a 1e-3 A step never crosses r_cut
    m = MACE(small_model_path, keep_stages=True)
    m.compute_node_energies_forces(*edge_args(species, nl))
    return m, species, nl


def _close(a, b, rel):
    scale = max(np.abs(b).max(), 1e-12)
    err = np.abs(np.asarray(a) - np.asarray(b)).max()
    print(f"max|d|={err:.3e} scale={scale:.3e}")
    return err <= rel * scale


def test_stage_buffers_after_evaluation_match_oracle(setup, small_model_path):
    m, species, nl = setup
    ref = Evaluator(small_model_path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    for name in ("M0", "H1", "Phi1", "A1", "A1_adj", "Phi1_adj", "H1_adj", "M0_adj"):
        assert _close(m.stage(name), ref.get(name), 1e-4), name
    # a stage run on the evaluation's own inputs reproduces its output
    H1 = m.H1
    m.compute_H1(len(species))
    assert _close(m.H1, H1, 1e-6)


def test_H1(setup):
    """test_mace.py:260-299: d sum(H1) / dM0 through reverse_H1."""
    m, species, nl = setup
    n = len(species)
    rng = np.random.default_rng(1)
    M0 = rng.normal(size=m.M0.size)

    def f(x):
        m.M0 = x
        m.compute_H1(n)
        return m.H1.sum()

    f(M0)
    m.H1_adj = np.ones(m.H1.size)
    m.reverse_H1(n)
    g = m.M0_adj
    idx = rng.choice(M0.size, 48, replace=False)
    assert _close(g[idx], numerical_gradient(f, M0, 0.5, idx), 1e-4)


def test_A1(setup):
    """test_mace.py:388-424: d sum(A1) / dPhi1 through reverse_A1."""
    m, species, nl = setup
    n = len(species)
    rng = np.random.default_rng(2)
    Phi1 = rng.normal(size=m.Phi1.size)

    def f(x):
        m.Phi1 = x
        m.compute_A1(n)
        return m.A1.sum()

    f(Phi1)
    m.A1_adj = np.ones(m.A1.size)
    m.reverse_A1(n)
    g = m.Phi1_adj
    idx = rng.choice(Phi1.size, 48, replace=False)
    assert _close(g[idx], numerical_gradient(f, Phi1, 0.5, idx), 1e-4)


def test_Phi1(setup):
    """test_mace.py:329-385: d sum(Phi1) / dxyz (node_forces) and d sum(Phi1) / dH1 (H1_adj)
    through reverse_Phi1."""
    m, species, nl = setup
    n = len(species)
    nt, nn, ni, ne = species, nl["num_neigh"], nl["neigh_indices"], species[nl["neigh_indices"]]
    xyz = nl["xyz"].reshape(-1).copy()
    rng = np.random.default_rng(3)
    H1 = rng.normal(size=m.H1.size)
    m.H1 = H1

    def f(xyz_flat):
        r = np.sqrt(np.sum(xyz_flat.reshape(-1, 3) ** 2, axis=1))
        m.compute_R1(n, nt, nn, ne, r)
        m.compute_Y(xyz_flat)
        m.compute_Phi1(n, nn, ni)
        return m.Phi1.sum()

    r = nl["r"].copy()
    f(xyz)
    m.Phi1_adj = np.ones(m.Phi1.size)
    m.reverse_Phi1(n, nn, ni, xyz, r, True, True)
    forces = m.node_forces.copy()
    idx = rng.choice(xyz.size, 60, replace=False)
    assert _close(forces[idx], -numerical_gradient(f, xyz, 1e-3, idx), 2e-3)

    # H1_adj: linear in H1
    def fh(x):
        m.H1 = x
        m.compute_Phi1(n, nn, ni)
        return m.Phi1.sum()

    m.compute_R1(n, nt, nn, ne, r)
    m.compute_Y(xyz)
    fh(H1)
    m.Phi1_adj = np.ones(m.Phi1.size)
    m.H1_adj = np.zeros(m.H1.size)
    m.reverse_Phi1(n, nn, ni, xyz, r, True, False)
    g = m.H1_adj
    idx = rng.choice(H1.size, 48, replace=False)
    assert _close(g[idx], numerical_gradient(fh, H1, 0.5, idx), 1e-4)
    # node_forces accumulate without zero_dxyz
    m.reverse_Phi1(n, nn, ni, xyz, r, False, True)
    assert _close(m.node_forces, 2 * forces, 1e-6)


def test_stage_errors(setup):
    m, species, nl = setup
    with pytest.raises(ValueError):
        m.H1 = np.zeros(3)  # wrong length
    with pytest.raises(ValueError):
        m.compute_H1(len(species) + 1)  # not the buffers' node count
