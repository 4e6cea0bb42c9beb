"""LAMMPS pair-style adapter (smx_pair_compute_mode) against the engine's own periodic
path and the oracle.

A fake LAMMPS setup (tests/helpers.py fake_lammps): a periodic box of local atoms plus a
ghost shell of their periodic images (tags -> local owners), full neighbour lists within
r_cut + 1 A skin with some entries carrying special-bond flag bits, and a LAMMPS-type ->
species map that is not the identity.  In the default mode the adapter's energy, forces
on local atoms and virial must equal smx_compute_atoms on the same box up to the float32
rounding of a different edge order (per-atom energy 2e-5 eV, forces 2e-5 eV/A), and a
second call with moved positions and the old topology must equal a fresh evaluation.
The two MPI modes run on one rank as the reference's tests run them
(pair_symmetrix/test/test_pair_symmetrix_mace.py:28-39): their forces before LAMMPS's
reverse communication are checked row by row, ghosts included, against the oracle, and
after folding each ghost onto its owner against the default mode.
"""
import numpy as np
import pytest

from helpers import NEIGHMASK, atomic_forces, fake_lammps, halo_graph
from oracle.pyoracle import Evaluator
from symmetrix_gb300.lammps import MODES, PairAdapter
from symmetrix_gb300.synth.structures import random_box

pytestmark = pytest.mark.gpu


def test_pair_adapter_matches_engine(engine_lib, small_model_path):
    from symmetrix_gb300 import MACE
    rng = np.random.default_rng(21)
    pos, L, species = random_box(90, 0.09, 0.9, 3, seed=13)
    pos = pos - L * np.floor(pos / L)
    m = MACE(small_model_path)
    mace_types = np.array([2, 0, 1], dtype=np.int32)  # LAMMPS types 1, 2, 3 -> species 2, 0, 1
    inv = np.argsort(mace_types)                        # species -> LAMMPS type - 1
    x, local_of, nbrs = fake_lammps(pos, L, m.r_cut + 1.0, rng)
    types = (inv[species[local_of]] + 1).astype(np.int32)
    assert (np.concatenate(nbrs) & NEIGHMASK).max() < len(x)
    pair = PairAdapter(m, mace_types)
    for step in range(2):
        if step == 1:  # positions move, topology kept (no re-neighbouring)
            d = 0.05 * rng.standard_normal(pos.shape)
            pos = pos + d
            x = x + d[local_of]
        e, f, eatom, vir = pair.compute(x, types, local_of, np.arange(len(pos)), nbrs, neigh_changed=(step == 0),
                                        eflag_atom=True)
        E, node_e, F, W = m.compute_atoms(pos, species, L)
        Wv = np.array([W[0, 0], W[1, 1], W[2, 2], 0.5 * (W[0, 1] + W[1, 0]), 0.5 * (W[0, 2] + W[2, 0]),
                       0.5 * (W[1, 2] + W[2, 1])])
        print(f"step {step}: dE {abs(e - E):.2e}  max|dF| {np.abs(f[:len(pos)] - F).max():.2e}  "
              f"max|dW| {np.abs(vir - Wv).max():.2e}")
        assert abs(e - E) < 2e-5 * len(pos)
        assert np.abs(f[:len(pos)] - F).max() < 2e-5
        assert np.abs(f[len(pos):]).max() == 0.0  # forces land on local owners
        assert np.abs(eatom - node_e).max() < 2e-5
        assert np.abs(vir - Wv).max() < 1e-4 * max(1.0, np.abs(Wv).max())


def test_pair_adapter_rejects_bad_lists(engine_lib, small_model_path):
    from symmetrix_gb300 import MACE
    m = MACE(small_model_path)
    pair = PairAdapter(m, [0, 1, 2])
    x = np.zeros((2, 3))
    x[1, 0] = 1.5
    with pytest.raises(ValueError):
        pair.compute(x, [1, 1], [0, 1], [0, 1], [np.array([5]), np.array([0])])  # neighbour index out of range
    with pytest.raises(ValueError):
        pair.compute(x, [1, 4], [0, 1], [0, 1], [np.array([1]), np.array([0])])  # type out of range


def _fold(f, local_of):
    out = np.zeros((int(local_of.max()) + 1, 3))
    np.add.at(out, local_of, f)
    return out


def test_pair_modes_on_one_rank(engine_lib, small_model_path):
    """All three modes on one box: the ghost shell is 2 r_cut + 1 A deep with lists for
    every atom, as the no-MPI-message-passing mode makes LAMMPS provide."""
    from symmetrix_gb300 import MACE
    rng = np.random.default_rng(5)
    pos, L, species = random_box(90, 0.09, 0.9, 3, seed=13)
    pos = pos - L * np.floor(pos / L)
    n = len(pos)
    m = MACE(small_model_path)
    rc = m.r_cut
    mace_types = np.array([2, 0, 1], dtype=np.int32)
    inv = np.argsort(mace_types)
    x, local_of, nbrs = fake_lammps(pos, L, rc + 1.0, rng, shell=2 * rc + 1.0, ghost_lists=True)
    nall = len(x)
    sp = species[local_of].astype(np.int32)
    types = (inv[sp] + 1).astype(np.int32)
    res = {}
    for mode in MODES:
        pair = PairAdapter(m, mace_types, mode)
        if mode == "no_mpi_message_passing":
            res[mode] = pair.compute(x, types, None, np.arange(nall), nbrs, eflag_atom=True, gnum=nall - n)
        else:
            res[mode] = pair.compute(x, types, local_of, np.arange(n), nbrs[:n], eflag_atom=True)
    e0, f0, ea0, v0 = res["no_domain_decomposition"]
    assert np.abs(f0[n:]).max() == 0.0

    # mpi_message_passing: the same evaluation; ghost neighbours keep their forces
    e1, f1, ea1, v1 = res["mpi_message_passing"]
    print(f"mpi: dE {abs(e1 - e0):.2e} dEi {np.abs(ea1 - ea0).max():.2e} dW {np.abs(v1 - v0).max():.2e}")
    assert abs(e1 - e0) <= 1e-12 * abs(e0) and np.abs(ea1 - ea0).max() <= 1e-12
    assert np.abs(v1 - v0).max() <= 1e-12 * np.abs(v0).max()
    assert np.abs(f1[n:]).max() > 0.0
    assert np.abs(_fold(f1, local_of) - f0[:n]).max() < 1e-10
    # its rows against the oracle: edges i -> j (ghost indices), H1 of j from its owner
    lists = [np.asarray(nb).view(np.uint32).astype(np.int64) & NEIGHMASK for nb in nbrs[:n]]
    ei, ej = [], []
    for i in range(n):
        d = x[lists[i]] - x[i]
        keep = (d * d).sum(1) < rc * rc
        ei.append(np.full(keep.sum(), i))
        ej.append(lists[i][keep])
    ei, ej = np.concatenate(ei), np.concatenate(ej)
    xyz = x[ej] - x[ei]
    ref = Evaluator(small_model_path, "port")
    ref.compute_node_energies_forces(n, sp[:n], np.bincount(ei, minlength=n), local_of[ej], sp[ej], xyz,
                                     np.sqrt((xyz * xyz).sum(1)))
    F1 = atomic_forces(nall, ei, ej, ref.node_forces)
    print(f"mpi rows vs oracle: {np.abs(f1 - F1).max():.2e}")
    assert np.abs(f1 - F1).max() < 2e-5

    # no_mpi_message_passing: layer 0 also over the ghosts within r_cut of a local atom
    e2, f2, ea2, v2 = res["no_mpi_message_passing"]
    node_atom, nn, ni, natom, hxyz, hr = halo_graph(x, n, nbrs, rc)
    ref.compute_halo(n, len(node_atom), sp[node_atom], nn, ni, sp[natom], hxyz, hr)
    F2 = atomic_forces(nall, np.repeat(node_atom, nn), natom, ref.node_forces)
    print(f"halo: N0 {len(node_atom)} dE {abs(e2 - ref.node_energies.sum()):.2e} "
          f"rows vs oracle {np.abs(f2 - F2).max():.2e} folded vs default {np.abs(_fold(f2, local_of) - f0[:n]).max():.2e}")
    assert abs(e2 - ref.node_energies.sum()) < 2e-5 * n
    assert np.abs(ea2 - ref.node_energies).max() < 2e-5
    assert np.abs(f2 - F2).max() < 2e-5
    assert abs(e2 - e0) < 2e-5 * n and np.abs(ea2 - ea0).max() < 2e-5
    assert np.abs(_fold(f2, local_of) - f0[:n]).max() < 2e-5
    assert np.abs(v2 - v0).max() < 1e-4 * max(1.0, np.abs(v0).max())


def test_halo_mode_needs_ghost_lists(engine_lib, small_model_path):
    from symmetrix_gb300 import MACE
    pos, L, species = random_box(40, 0.09, 0.9, 3, seed=3)
    pos = pos - L * np.floor(pos / L)
    m = MACE(small_model_path)
    x, local_of, nbrs = fake_lammps(pos, L, m.r_cut + 1.0)
    types = (species[local_of] + 1).astype(np.int32)
    pair = PairAdapter(m, [0, 1, 2], "no_mpi_message_passing")
    with pytest.raises(ValueError, match="ghost neighbour list"):
        pair.compute(x, types, None, np.arange(len(pos)), nbrs)
    with pytest.raises(ValueError):
        PairAdapter(m, [0, 1, 2], "domain_decomposition")
