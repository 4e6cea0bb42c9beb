"""ASE calculator shim and host neighbour list (CPU).

The calculator logic (species mapping, edge forces -> atomic forces, virial and
stress, the choice between the GPU neighbour build and the host list) runs here
against a float64 pair-potential evaluator with the engine's interface, and is
checked by finite differences of its own energy, as the reference's
test_symmetrix_calc.py does for forces and stress.
"""
import numpy as np
import pytest

from symmetrix_gb300.calculator import Symmetrix, evaluate_structure, voigt6
from symmetrix_gb300.neighbors import neighbor_list_cell
from symmetrix_gb300.synth.structures import neighbor_list, random_box


class PairEvaluator:
    """E_i = 1/2 sum_j phi(r_ij), phi(r) = (r_c - r)^3 / r; node_forces[e] = -dE/dxyz_e."""

    def __init__(self, atomic_numbers=(1, 6, 8), r_cut=3.0):
        self.atomic_numbers = list(atomic_numbers)
        self.r_cut = r_cut
        self.calls = {"edges": 0, "atoms": 0}

    def _phi(self, r, ti, tj):
        w = 1.0 + 0.1 * (ti + tj)
        return w * (self.r_cut - r) ** 3 / r, w * (-3 * (self.r_cut - r) ** 2 / r - (self.r_cut - r) ** 3 / r ** 2)

    def compute_node_energies_forces(self, n, node_types, num_neigh, neigh_indices, neigh_types, xyz, r):
        self.calls["edges"] += 1
        xyz = np.asarray(xyz).reshape(-1, 3)
        i = np.repeat(np.arange(n), num_neigh)
        p, dp = self._phi(np.asarray(r), np.asarray(node_types)[i], np.asarray(neigh_types))
        self.node_energies = np.bincount(i, weights=0.5 * p, minlength=n)
        # E depends on xyz_e through both edge directions; the per-edge derivative of
        # the 1/2-weighted term is the edge's own contribution
        self.node_forces = (-(0.5 * dp / np.asarray(r))[:, None] * xyz).reshape(-1)

    def compute_atoms(self, pos, species, box):
        self.calls["atoms"] += 1
        cell = np.diag(box) if box is not None else np.eye(3)
        pbc = [box is not None] * 3
        nl = neighbor_list_cell(pos, cell, pbc, self.r_cut)
        n = len(pos)
        self.compute_node_energies_forces(n, species, nl["num_neigh"], nl["neigh_indices"], species[nl["neigh_indices"]],
                                          nl["xyz"], nl["r"])
        f = self.node_forces.reshape(-1, 3)
        F = np.zeros((n, 3))
        np.add.at(F, nl["neigh_indices"], f)
        np.add.at(F, nl["i"], -f)
        return float(self.node_energies.sum()), self.node_energies, F, nl["xyz"].T @ f


class FakeAtoms:
    def __init__(self, numbers, positions, cell, pbc):
        self.numbers, self.positions = np.asarray(numbers), np.asarray(positions, float)
        self.cell, self.pbc = np.asarray(cell, float), np.broadcast_to(pbc, 3).copy()

    def get_atomic_numbers(self):
        return self.numbers

    def get_positions(self):
        return self.positions

    def get_cell(self):
        return self.cell

    def get_pbc(self):
        return self.pbc

    def copy(self):
        return FakeAtoms(self.numbers, self.positions.copy(), self.cell.copy(), self.pbc.copy())


def triclinic(n=40, seed=4):
    rng = np.random.default_rng(seed)
    cell = np.array([[7.0, 0.0, 0.0], [1.3, 6.5, 0.0], [-0.8, 0.9, 7.4]])
    frac = rng.random((n, 3))
    return rng.choice([1, 6, 8], n), frac @ cell, cell


def test_cell_list_matches_cubic_list():
    pos, L, _ = random_box(120, 0.1, 0.9, 3, seed=3)
    pos = pos - L * np.floor(pos / L)
    a = neighbor_list(pos, 4.0, L)
    b = neighbor_list_cell(pos, np.eye(3) * L, [True] * 3, 4.0)
    assert np.array_equal(a["num_neigh"], b["num_neigh"])
    assert np.allclose(np.sort(a["r"]), np.sort(b["r"]))


def test_cell_list_triclinic_against_brute_force():
    _, pos, cell = triclinic()
    nl = neighbor_list_cell(pos, cell, [True, True, False], 3.0)
    cnt = np.zeros(len(pos), int)
    rng = range(-2, 3)
    for i in range(len(pos)):
        for j in range(len(pos)):
            for a in rng:
                for b in rng:
                    d = pos[j] + a * cell[0] + b * cell[1] - pos[i]
                    r = np.linalg.norm(d)
                    if 1e-8 < r < 3.0:
                        cnt[i] += 1
    assert np.array_equal(cnt, nl["num_neigh"])
    assert np.allclose(np.linalg.norm(nl["xyz"], axis=1), nl["r"])
    assert (np.diff(nl["i"]) >= 0).all()


def test_voigt_order():
    s = np.arange(9.0).reshape(3, 3)
    assert np.allclose(voigt6(s), [0, 4, 8, 6, 4, 2])


@pytest.mark.parametrize("pbc", [[True, True, True], [True, True, False], [False, False, False]])
def test_calculator_forces_and_stress_by_finite_differences(pbc):
    z, pos, cell = triclinic()
    calc = Symmetrix.__new__(Symmetrix)  # the engine-free parts: attach the pair evaluator
    Symmetrix.__mro__[1].__init__(calc)
    calc.evaluator, calc.cutoff = PairEvaluator(), 3.0
    atoms = FakeAtoms(z, pos, cell, pbc)
    E0 = calc.get_potential_energy(atoms)
    F = calc.get_forces(atoms)
    assert np.isclose(E0, calc.results["energies"].sum())
    h = 1e-5
    for a, k in [(0, 0), (5, 1), (17, 2)]:
        p, m = atoms.copy(), atoms.copy()
        p.positions[a, k] += h
        m.positions[a, k] -= h
        fd = -(calc.get_potential_energy(p) - calc.get_potential_energy(m)) / (2 * h)
        assert abs(fd - F[a, k]) < 1e-6 * max(1.0, abs(fd))
    if all(pbc):
        S = calc.get_stress(atoms)
        V = abs(np.linalg.det(cell))
        for (a, b), v in zip([(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)], range(6)):
            eps = np.zeros((3, 3))
            eps[a, b] = eps[b, a] = h
            p, m = atoms.copy(), atoms.copy()
            p.positions, p.cell = atoms.positions @ (np.eye(3) + eps), atoms.cell @ (np.eye(3) + eps)
            m.positions, m.cell = atoms.positions @ (np.eye(3) - eps), atoms.cell @ (np.eye(3) - eps)
            fd = (calc.get_potential_energy(p) - calc.get_potential_energy(m)) / (2 * h) / V
            if a != b:
                fd /= 2.0
            assert abs(fd - S[v]) < 1e-6 * max(1.0, abs(fd)), (a, b)


def test_orthorhombic_and_general_paths_agree():
    pos, L, sp = random_box(60, 0.08, 0.9, 3, seed=5)
    z = np.array([1, 6, 8])[sp]
    ev = PairEvaluator()
    fast = evaluate_structure(ev, z, pos - L * np.floor(pos / L), np.eye(3) * L, [True] * 3)
    assert ev.calls["atoms"] == 1
    ev2 = PairEvaluator()
    cell = np.eye(3) * L
    cell[1, 0] = 1e-3  # not orthorhombic: host list
    slow = evaluate_structure(ev2, z, pos - L * np.floor(pos / L), cell, [True] * 3)
    assert ev2.calls["edges"] == 1
    assert abs(fast["energy"] - slow["energy"]) < 1e-2 * abs(fast["energy"]) + 1e-6
    with pytest.raises(ValueError):
        evaluate_structure(ev, np.full(len(z), 26), pos, np.eye(3) * L, [True] * 3)


def test_module_offers_the_reference_binding_names():
    """Code written against the reference's `symmetrix` module finds the names its
    calculator uses (symmetrix_calc.py:43-49) on this package, without a GPU."""
    import symmetrix_gb300 as symmetrix
    assert hasattr(symmetrix, "MACEKokkos") and issubclass(symmetrix.MACEKokkosFloat, symmetrix.MACE)
    if not symmetrix._kokkos_is_initialized():
        symmetrix._init_kokkos()
    assert symmetrix._kokkos_is_initialized()
