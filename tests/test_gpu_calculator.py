"""ASE calculator shim on the GPU engine against the float64 oracle.

A triclinic periodic cell goes through the host neighbour list and the evaluator
call; an orthorhombic box through the engine's GPU neighbour build.  Energies,
atomic forces and stress are compared with the oracle on the same neighbour list
(FP32 plain form tolerances: 2e-5 eV per atom, 1e-5 eV/A).
"""
import numpy as np
import pytest

from helpers import atomic_forces, virial
from oracle.pyoracle import Evaluator
from symmetrix_gb300.calculator import Symmetrix
from symmetrix_gb300.neighbors import neighbor_list_cell
from test_calculator import FakeAtoms

pytestmark = pytest.mark.gpu


def _oracle(path, z_model, numbers, pos, cell, pbc, r_cut):
    sp = np.array([z_model.index(int(a)) for a in numbers], dtype=np.int32)
    nl = neighbor_list_cell(pos, cell, pbc, r_cut)
    ev = Evaluator(path, "port")
    ev.compute_node_energies_forces(len(pos), sp, nl["num_neigh"], nl["neigh_indices"], sp[nl["neigh_indices"]],
                                    nl["xyz"].reshape(-1), nl["r"])
    f = np.asarray(ev.node_forces)
    F = atomic_forces(len(pos), nl["i"], nl["neigh_indices"], f)
    return float(np.sum(ev.node_energies)), F, virial(nl["xyz"], f)


@pytest.mark.parametrize("kind", ["triclinic", "orthorhombic"])
def test_calculator_matches_oracle(engine_lib, small_model_path, kind):
    calc = Symmetrix(small_model_path, dtype="float64")
    rng = np.random.default_rng(11)
    if kind == "triclinic":
        cell = np.array([[10.5, 0.0, 0.0], [2.1, 10.2, 0.0], [-1.4, 1.7, 10.8]])
    else:
        cell = np.diag([10.6, 11.2, 10.9])
    # jittered lattice: no pair closer than ~1.5 A
    g = (np.stack(np.meshgrid(*[np.arange(4)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) / 4
    frac = g + 0.04 * rng.standard_normal(g.shape)
    pos = frac @ cell
    numbers = rng.choice(calc.evaluator.atomic_numbers, len(pos))
    atoms = FakeAtoms(numbers, pos, cell, True)
    E = calc.get_potential_energy(atoms)
    F = calc.get_forces(atoms)
    S = calc.get_stress(atoms)
    Er, Fr, Wr = _oracle(small_model_path, calc.evaluator.atomic_numbers, numbers, pos, cell, [True] * 3,
                         calc.cutoff)
    V = abs(np.linalg.det(cell))
    Sr = -Wr.T / V
    Sr = np.array([Sr[0, 0], Sr[1, 1], Sr[2, 2], 0.5 * (Sr[1, 2] + Sr[2, 1]), 0.5 * (Sr[0, 2] + Sr[2, 0]),
                   0.5 * (Sr[0, 1] + Sr[1, 0])])
    print(f"{kind}: dE/atom {abs(E - Er) / len(pos):.2e}  max|dF| {np.abs(F - Fr).max():.2e}  "
          f"max|dS| {np.abs(S - Sr).max():.2e}")
    assert abs(E - Er) / len(pos) < 2e-5
    assert np.abs(F - Fr).max() < 1e-5
    assert np.abs(S - Sr).max() * V < 1e-4
