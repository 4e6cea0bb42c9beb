"""GPU neighbour lists, atom-level evaluation and the velocity-Verlet driver.

Checks: the GPU list reproduces the host list (cell-list and all-pairs paths) and
atomic forces / virial / energy from smx_compute_atoms equal the edge-level call
followed by the reference's own scatter (pair_symmetrix_mace.cpp:324-368); MD with
the graph-captured loop equals step-by-step velocity Verlet driven from the host,
and conserves energy.
"""
import numpy as np
import pytest

from helpers import atomic_forces, edge_args, virial
from symmetrix_gb300.synth.structures import (KB_EV, maxwell_boltzmann, neighbor_list, random_box,
                                              species_masses)

pytestmark = pytest.mark.gpu
ACC = 9.648533212331e-3  # (eV/A)/amu in A/fs^2


def _engine(path):
    from symmetrix_gb300 import MACE
    return MACE(path)


@pytest.mark.parametrize("n,density", [(64, 0.064), (400, 0.064)])  # 10 A box: all-pairs path; larger: cells
def test_compute_atoms_matches_edge_api(engine_lib, small_model_path, n, density):
    pos, L, sp = random_box(n, density, 0.9, 3, seed=31)
    m = _engine(small_model_path)
    E, node_e, F, W = m.compute_atoms(pos, sp, box=L)
    nl = neighbor_list(pos, m.r_cut, L)
    m.compute_node_energies_forces(*edge_args(sp, nl))
    Fh = atomic_forces(n, nl["i"], nl["neigh_indices"], m.node_forces)
    Wh = virial(nl["xyz"], m.node_forces)
    assert abs(E - m.node_energies.sum()) < 1e-6 * n
    # the GPU list orders a node's edges differently, so float32 sums differ by round-off
    np.testing.assert_allclose(node_e, m.node_energies, atol=1e-5)
    np.testing.assert_allclose(F, Fh, atol=1e-5)
    np.testing.assert_allclose(W, Wh, atol=1e-4 * max(1.0, np.abs(Wh).max()))
    np.testing.assert_allclose(F.sum(0), 0.0, atol=1e-6)


def test_compute_atoms_nonperiodic(engine_lib, small_model_path):
    rng = np.random.default_rng(4)
    pos = rng.normal(size=(30, 3)) * 2.5
    sp = rng.integers(0, 3, size=30).astype(np.int32)
    m = _engine(small_model_path)
    E, node_e, F, W = m.compute_atoms(pos, sp)
    nl = neighbor_list(pos, m.r_cut)
    m.compute_node_energies_forces(*edge_args(sp, nl))
    np.testing.assert_allclose(F, atomic_forces(30, nl["i"], nl["neigh_indices"], m.node_forces), atol=1e-5)


def test_md_graph_loop_matches_host_stepping(engine_lib, small_model_path):
    """12 steps (one graph-captured segment of 10, a rebuild, 2 eager steps) against
    velocity Verlet driven from the host with atom-level evaluations."""
    from symmetrix_gb300.md import MD
    pos, L, sp = random_box(400, 0.064, 0.9, 3, seed=5)
    m = _engine(small_model_path)
    masses = species_masses(m.atomic_numbers, sp)
    v = maxwell_boltzmann(masses, 300.0, np.random.default_rng(6))
    md = MD(m, pos, sp, masses, box=L, velocities=v, dt=0.25, skin=1.0, rebuild_every=10)
    md.run(12)
    st = md.state()
    x, vv = pos.copy(), v.copy()
    _, _, F, _ = m.compute_atoms(x, sp, box=L)
    for _ in range(12):
        vv += 0.5 * 0.25 * ACC * F / masses[:, None]
        x += 0.25 * vv
        _, _, F, _ = m.compute_atoms(x, sp, box=L)
        vv += 0.5 * 0.25 * ACC * F / masses[:, None]
    d = st["positions"] - x
    d -= L * np.round(d / L)  # the driver wraps positions at rebuilds
    print(f"MD vs host stepping after 12 steps: max|dx|={np.abs(d).max():.2e} A, "
          f"max|dv|={np.abs(st['velocities'] - vv).max():.2e} A/fs")
    assert np.abs(d).max() < 1e-6
    np.testing.assert_allclose(st["velocities"], vv, atol=1e-6)
    assert st["step"] == 12


def test_md_conserves_energy(engine_lib, small_model_path):
    """NVE with carbon and oxygen only over 5 fs (the random synthetic potential has no
    short-range repulsion: after ~10 fs its random structure starts to collapse, and the
    close encounters would make any fixed-step integrator lose energy)."""
    from symmetrix_gb300.md import MD
    pos, L, sp = random_box(256, 0.064, 0.9, 2, seed=8)
    sp = (sp + 1).astype(np.int32)  # species indices 1, 2 = C, O
    m = _engine(small_model_path)
    masses = species_masses(m.atomic_numbers, sp)
    v = maxwell_boltzmann(masses, 300.0, np.random.default_rng(9))
    md = MD(m, pos, sp, masses, box=L, velocities=v, dt=0.1, skin=1.0, rebuild_every=10)
    tot = []
    for _ in range(6):
        st = md.state()
        ke = 0.5 * (masses[:, None] * st["velocities"] ** 2).sum() / ACC
        tot.append(st["potential_energy"] + ke)
        md.run(10)
    drift = (max(tot) - min(tot)) / 256
    print(f"NVE: total energy range per atom over 50 steps of 0.1 fs = {drift:.3e} eV")
    assert drift < 1e-4


@pytest.mark.parametrize("precision", ["float32", "bfloat16"])
def test_gpu_forces_are_energy_gradients(engine_lib, small_model_path, precision):
    """The reference's finite-difference check (symmetrix/test/test_mace.py:655-704) on the
    GPU path: central differences of the GPU energy match the GPU forces (tolerance from
    the float32 energy rounding over the step)."""
    from symmetrix_gb300 import MACE
    rng = np.random.default_rng(21)
    pos = rng.normal(size=(20, 3)) * 1.8
    species = rng.integers(0, 3, size=20).astype(np.int32)
    m = MACE(small_model_path, precision=precision)
    e0, _, F, _ = m.compute_atoms(pos, species)
    h = 5e-3
    for a in (0, 7, 13):
        for c in range(3):
            p, q = pos.copy(), pos.copy()
            p[a, c] += h
            q[a, c] -= h
            fd = -(m.compute_atoms(p, species)[0] - m.compute_atoms(q, species)[0]) / (2 * h)
            assert abs(fd - F[a, c]) < 5e-3 * max(1.0, abs(F[a, c])), (a, c, fd, F[a, c])


def test_md_renumbering_keeps_caller_order(engine_lib, small_model_path):
    """Periodic MD renumbers the atoms spatially at the first rebuild and every 200 steps;
    the state is reported in the caller's order: after 205 steps (two renumberings) the
    reported forces are those of an evaluation at the reported positions with the
    caller's species."""
    from symmetrix_gb300.md import MD
    pos, L, sp = random_box(400, 0.064, 0.9, 2, seed=15)
    sp = (sp + 1).astype(np.int32)  # C and O
    m = _engine(small_model_path)
    masses = species_masses(m.atomic_numbers, sp)
    v = maxwell_boltzmann(masses, 300.0, np.random.default_rng(16))
    md = MD(m, pos, sp, masses, box=L, velocities=v, dt=0.1, skin=1.0, rebuild_every=10)
    md.run(205)
    st = md.state()
    assert st["step"] == 205
    E, _, F, W = m.compute_atoms(st["positions"], sp, box=L)
    np.testing.assert_allclose(st["forces"], F, atol=1e-5)
    # the energy and virial sums over the skin list (its geometry and per-edge forces are
    # filled for the read-out from the packed in-cut-off edges)
    assert abs(st["potential_energy"] - E) < 1e-6 * len(sp)
    np.testing.assert_allclose(st["virial"], W, atol=1e-4 * max(1.0, np.abs(W).max()))
    # momentum is conserved in the caller's order too (masses of the caller's species)
    p = (masses[:, None] * st["velocities"]).sum(0)
    p0 = (masses[:, None] * v).sum(0)
    np.testing.assert_allclose(p, p0, atol=1e-6 * np.abs(masses[:, None] * v).sum())
