"""Batching form: many independent non-periodic molecules in one pass
(smx_compute_molecules) and in one MD (smx_md_create_molecules).

* Each molecule's energy and forces equal a separate non-periodic evaluation of that
  molecule alone (same edges in the same order: bitwise-equal energies, forces to
  float32 rounding), and the oracle for a few of them.
* Molecules placed on top of each other stay independent (edges only within a
  molecule).
* Batch MD: total energy conserved over 32 steps of 0.25 fs.
"""
import numpy as np
import pytest

from helpers import atomic_forces
from oracle.pyoracle import Evaluator
from symmetrix_gb300.synth.structures import maxwell_boltzmann, neighbor_list, random_molecule, species_masses

pytestmark = pytest.mark.gpu


def molecules(n, seed, spread=True):
    rng = np.random.default_rng(seed)
    mols = []
    for m in range(n):
        k = int(rng.integers(8, 41))
        pos, sp = random_molecule(k, 0.08, 0.95, 3, rng)
        if spread:
            pos = pos + 30.0 * np.array([m % 8, (m // 8) % 8, m // 64])
        mols.append((pos, sp))
    return mols


def test_batch_equals_separate_evaluations(engine_lib, small_model_path):
    from symmetrix_gb300 import MACE
    m = MACE(small_model_path)
    mols = molecules(40, 3)
    E, node_e, F = m.compute_molecules(mols)
    for q, (pos, sp) in enumerate(mols):
        e1, ne1, f1, _ = m.compute_atoms(pos, sp, None)
        assert E[q] == pytest.approx(e1, abs=1e-9)
        assert np.abs(F[q] - f1).max() < 2e-6
    for q in (0, 7, 19):  # against the oracle
        pos, sp = mols[q]
        nl = neighbor_list(pos, m.r_cut)
        ev = Evaluator(small_model_path, "port")
        ev.compute_node_energies_forces(len(pos), sp, nl["num_neigh"], nl["neigh_indices"], sp[nl["neigh_indices"]],
                                        nl["xyz"].reshape(-1), nl["r"])
        Fr = atomic_forces(len(pos), nl["i"], nl["neigh_indices"], ev.node_forces)
        assert abs(E[q] - np.sum(ev.node_energies)) < 2e-5 * len(pos)
        assert np.abs(F[q] - Fr).max() < 1e-5


def test_overlapping_molecules_stay_independent(engine_lib, small_model_path):
    from symmetrix_gb300 import MACE
    m = MACE(small_model_path)
    spread = molecules(12, 5)
    stacked = molecules(12, 5, spread=False)  # same molecules, all centred at the origin
    Ea, _, Fa = m.compute_molecules(spread)
    Eb, _, Fb = m.compute_molecules(stacked)
    assert np.allclose(Ea, Eb, atol=1e-9)
    for fa, fb in zip(Fa, Fb):
        assert np.abs(fa - fb).max() < 2e-6
    with pytest.raises(ValueError):
        m._lib  # noqa: B018 - keep a handle
        from symmetrix_gb300 import _lib
        import ctypes
        bad = np.array([0, 5, 3], dtype=np.int32)
        x = np.zeros((3, 3))
        s = np.zeros(3, dtype=np.int32)
        _lib.raise_for(m._lib.smx_compute_molecules(m._h, 2, ctypes.c_void_p(bad.ctypes.data),
                                                    ctypes.c_void_p(x.ctypes.data), ctypes.c_void_p(s.ctypes.data),
                                                    None, None, ctypes.c_void_p(x.ctypes.data)), m._lib)


def test_batch_md_conserves_energy(engine_lib, small_model_path):
    from symmetrix_gb300 import MACE
    from symmetrix_gb300.md import MD
    m = MACE(small_model_path)
    mols = molecules(24, 9)
    pos = np.concatenate([p for p, _ in mols])
    sp = np.concatenate([s for _, s in mols]).astype(np.int32)
    first = np.concatenate([[0], np.cumsum([len(p) for p, _ in mols])])
    masses = species_masses(m.atomic_numbers, sp)
    vel = maxwell_boltzmann(masses, 300.0, np.random.default_rng(2))
    md = MD(m, pos, sp, masses, velocities=vel, dt=0.25, skin=1.0, rebuild_every=10, mol_first=first)
    acc = 9.648533212331e-3
    tot = []
    for _ in range(5):
        st = md.state()
        tot.append(st["potential_energy"] + 0.5 * float((masses[:, None] * st["velocities"] ** 2).sum()) / acc)
        md.run(8)
    md.sync()
    drift = (max(tot) - min(tot)) / len(pos)
    print(f"batch MD: total energy range per atom over 32 steps = {drift:.3e} eV")
    assert drift < 2e-4
