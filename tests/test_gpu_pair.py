"""LAMMPS pair-style adapter (smx_pair_compute) against the engine's own periodic path.

A fake LAMMPS setup: a periodic box of local atoms plus a ghost shell of their
periodic images (tags -> local owners), a full neighbour list over local and ghost
atoms within r_cut + 1 A skin with some entries carrying special-bond flag bits, and
a LAMMPS-type -> species map that is not the identity.  The adapter's energy, forces
on local atoms and virial must equal smx_compute_atoms on the same box up to the
float32 rounding of a different edge order (per-atom energy 2e-5 eV, forces 2e-5
eV/A), and a second call with moved positions and the old topology must equal a
fresh evaluation.
"""
import numpy as np
import pytest

from symmetrix_gb300.lammps import NEIGHMASK, PairAdapter
from symmetrix_gb300.synth.structures import random_box

pytestmark = pytest.mark.gpu


def fake_lammps(pos, L, shell, rng):
    n = len(pos)
    xs, owner = [pos], [np.arange(n)]
    for s in np.array(np.meshgrid(*[[-1, 0, 1]] * 3, indexing="ij")).reshape(3, -1).T:
        if not s.any():
            continue
        p = pos + s * L
        keep = np.all((p > -shell) & (p < L + shell), axis=1)
        xs.append(p[keep])
        owner.append(np.nonzero(keep)[0])
    x = np.concatenate(xs)
    local_of = np.concatenate(owner).astype(np.int32)
    neighbors = []
    for i in range(n):
        d = np.linalg.norm(x - x[i], axis=1)
        js = np.nonzero((d < shell) & (np.arange(len(x)) != i))[0].astype(np.int64)
        flags = rng.integers(0, 4, len(js)) << 30  # special-bond bits above NEIGHMASK
        neighbors.append(((js | flags) & 0xFFFFFFFF).astype(np.uint32).view(np.int32))
    return x, local_of, neighbors


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
