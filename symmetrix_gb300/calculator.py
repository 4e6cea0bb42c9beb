"""ASE calculator over the GB300 engine, shaped like the reference's `Symmetrix`
(symmetrix/source/symmetrix/symmetrix_calc.py:23-102).

`Symmetrix(model_file, dtype="float64", use_kokkos=True, **kwargs)` with
implemented_properties energy, free_energy, energies, forces, stress.  The results
follow the reference: energy = sum of node energies, forces F_j += f_e, F_i -= f_e
from the per-edge forces, stress = -(f^T xyz) / V in Voigt order.

dtype maps onto the engine's forms: "float32" and "float64" -> the FP32 plain form
(the engine has no float64 GPU form; its forces are within 1e-5 eV/A of the float64
evaluator), "bfloat16" -> the BF16-mixed form.  use_kokkos is accepted and ignored
(there is one GPU engine).  A model file that is not libsymmetrix JSON raises
RuntimeError, as the reference's evaluator does; the reference's fallback converts
a PyTorch MACE model first, which needs mace-torch and is left to the caller.

ASE is imported when present; without it a minimal stand-in base provides the same
calculate()/results protocol and the get_potential_energy / get_forces / get_stress
accessors, so the calculator also works on any object with ASE's Atoms accessors.
"""
import numpy as np

from .mace import MACE
from .neighbors import neighbor_list_cell

try:  # pragma: no cover - ASE is optional
    from ase.calculators.calculator import Calculator, all_changes
    HAVE_ASE = True
except ImportError:
    HAVE_ASE = False
    all_changes = ["positions", "numbers", "cell", "pbc"]

    class Calculator:
        """The part of ase.calculators.calculator.Calculator this shim relies on."""

        implemented_properties = []

        def __init__(self, **kwargs):
            self.atoms = None
            self.results = {}
            self.parameters = dict(kwargs)

        def calculate(self, atoms=None, properties=("energy",), system_changes=all_changes):
            if atoms is not None:
                self.atoms = atoms.copy() if hasattr(atoms, "copy") else atoms
            self.results = {}

        def get_property(self, name, atoms=None):
            self.calculate(atoms, [name])
            return self.results[name]

        def get_potential_energy(self, atoms=None, force_consistent=False):
            return self.get_property("free_energy" if force_consistent else "energy", atoms)

        def get_potential_energies(self, atoms=None):
            return self.get_property("energies", atoms)

        def get_forces(self, atoms=None):
            return self.get_property("forces", atoms)

        def get_stress(self, atoms=None):
            return self.get_property("stress", atoms)

_FORMS = {"float64": "float32", "float32": "float32", "bfloat16": "bfloat16"}


def voigt6(s):
    """3x3 -> (xx, yy, zz, yz, xz, xy), symmetrised like ase.stress.full_3x3_to_voigt_6_stress."""
    s = np.asarray(s)
    return np.array([s[0, 0], s[1, 1], s[2, 2], 0.5 * (s[1, 2] + s[2, 1]), 0.5 * (s[0, 2] + s[2, 0]),
                     0.5 * (s[0, 1] + s[1, 0])])


def evaluate_structure(evaluator, numbers, positions, cell, pbc):
    """Energy, node energies, forces (n, 3), virial W_ab = sum_e xyz_a f_b and stress (Voigt)
    of one structure.  Orthorhombic fully periodic cells and non-periodic systems use the
    engine's GPU neighbour build; other cells a host neighbour list."""
    z = list(evaluator.atomic_numbers)
    try:
        species = np.array([z.index(int(a)) for a in numbers], dtype=np.int32)
    except ValueError:
        raise ValueError("structure contains an element the model does not describe") from None
    pos = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
    n = len(pos)
    cell = np.asarray(cell, dtype=np.float64).reshape(3, 3)
    pbc = [bool(p) for p in np.broadcast_to(pbc, 3)]
    ortho = np.allclose(cell - np.diag(np.diag(cell)), 0.0)
    if not any(pbc) or (all(pbc) and ortho and (np.diag(cell) > 2.0 * evaluator.r_cut).all()):
        box = np.diag(cell).copy() if all(pbc) else None
        energy, node_e, forces, W = evaluator.compute_atoms(pos, species, box)
    else:
        nl = neighbor_list_cell(pos, cell, pbc, evaluator.r_cut)
        evaluator.compute_node_energies_forces(n, species, nl["num_neigh"], nl["neigh_indices"],
                                               species[nl["neigh_indices"]], nl["xyz"].reshape(-1), nl["r"])
        node_e = np.array(evaluator.node_energies[:n])
        f = np.asarray(evaluator.node_forces).reshape(-1, 3)[:len(nl["r"])]
        forces = np.zeros((n, 3))
        np.add.at(forces, nl["neigh_indices"], f)
        np.add.at(forces, nl["i"], -f)
        W = nl["xyz"].T @ f
        energy = float(node_e.sum())
    out = {"energy": energy, "energies": node_e, "forces": forces, "virial": W}
    if all(pbc):
        out["stress"] = voigt6(-W.T / abs(np.linalg.det(cell)))
    return out


class Symmetrix(Calculator):
    """ASE calculator evaluating a libsymmetrix JSON MACE model on the GB300 engine."""

    implemented_properties = ["energy", "free_energy", "energies", "forces", "stress"]

    def __init__(self, model_file, dtype="float64", use_kokkos=True, device=0, **kwargs):
        Calculator.__init__(self, **kwargs)
        if dtype not in _FORMS:
            raise ValueError(f"Unsupported dtype '{dtype}'. Supported dtypes are 'float64', 'float32' and "
                             f"'bfloat16'.")
        self.dtype = dtype
        self.use_kokkos = use_kokkos
        self.evaluator = MACE(str(model_file), device=device, precision=_FORMS[dtype])
        self.cutoff = self.evaluator.r_cut

    def calculate(self, atoms=None, properties=("energy",), system_changes=all_changes):
        Calculator.calculate(self, atoms, properties, system_changes)
        a = self.atoms
        r = evaluate_structure(self.evaluator, a.get_atomic_numbers(), a.get_positions(), a.get_cell(),
                               a.get_pbc())
        self.results["energy"] = self.results["free_energy"] = r["energy"]
        self.results["energies"] = np.asarray(r["energies"])
        self.results["forces"] = r["forces"]
        if "stress" in r:
            self.results["stress"] = r["stress"]
