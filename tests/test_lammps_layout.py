"""Host-side LAMMPS layouts (no GPU): the k-d-tree builder the bench uses
(symmetrix_gb300.synth.structures.lammps_rank) against the brute-force one of the tests
(helpers.fake_lammps), and the halo graph of the no-MPI-message-passing mode
(helpers.halo_graph) against the reference pair style's rules
(pair_symmetrix/pair_symmetrix_mace.cpp:557-655): every local atom is a node, every ghost
within r_cut of a local atom is a node after them in ascending index order, and a local
node's edges reach only nodes.
"""
import numpy as np

from helpers import NEIGHMASK, fake_lammps, halo_graph
from symmetrix_gb300.synth.structures import lammps_rank, random_box


def test_kdtree_layout_matches_brute_force():
    pos, L, _ = random_box(90, 0.09, 0.9, 3, seed=13)
    pos = pos - L * np.floor(pos / L)
    xa, la, na = fake_lammps(pos, L, 6.0, None, shell=11.0, ghost_lists=True)
    xb, lb, nb = lammps_rank(pos, L, 6.0, 11.0)
    assert np.array_equal(xa, xb) and np.array_equal(la, lb)
    assert len(na) == len(nb) == len(xa)
    for a, b in zip(na, nb):
        assert np.array_equal(np.sort(np.asarray(a) & NEIGHMASK), b)
    # the images are the local atoms shifted by whole box vectors
    d = (xb - pos[lb]) / L
    assert np.allclose(d, np.round(d), atol=1e-12)
    xc, lc, nc = lammps_rank(pos, L, 6.0, 11.0, ghost_lists=False)
    assert len(nc) == len(pos) and all(np.array_equal(a, b) for a, b in zip(nb, nc))


def test_halo_graph_follows_the_pair_style_rules():
    pos, L, _ = random_box(40, 0.09, 0.9, 3, seed=3)
    n, rc = len(pos), 5.0
    x, local_of, lists = lammps_rank(pos, L, rc + 1.0, 2 * rc + 1.0)
    node_atom, nn, ni, natom, xyz, r = halo_graph(x, n, lists, rc)
    assert np.array_equal(node_atom[:n], np.arange(n))
    ghosts = node_atom[n:]
    assert np.all(ghosts >= n) and np.all(np.diff(ghosts) > 0)
    near = set()
    for i in range(n):
        d = np.linalg.norm(x[lists[i]] - x[i], axis=1)
        near.update(int(j) for j in lists[i][d < rc] if j >= n)
    assert set(int(g) for g in ghosts) == near
    assert np.all((r > 0) & (r < rc)) and np.allclose(np.linalg.norm(xyz, axis=1), r)
    E1 = int(nn[:n].sum())
    assert np.array_equal(node_atom[ni[:E1]], natom[:E1])  # local edges reach nodes
    assert np.allclose(xyz, x[natom] - x[np.repeat(node_atom, nn)])
