"""Shared helpers for the tests: structures, atomic forces, rotations."""
import numpy as np


def atomic_forces(n_atoms, edge_i, neigh_indices, node_forces):
    """F_j += f_e, F_i -= f_e (pair_symmetrix_mace.cpp:334-347; symmetrix_calc.py:92-99)."""
    f = np.asarray(node_forces).reshape(-1, 3)
    F = np.zeros((n_atoms, 3))
    np.add.at(F, neigh_indices, f)
    np.add.at(F, edge_i, -f)
    return F


def virial(xyz, node_forces):
    """sum_e xyz_e (x) f_e (pair_symmetrix_mace.cpp:349-368, unsymmetrised)."""
    return np.asarray(xyz).reshape(-1, 3).T @ np.asarray(node_forces).reshape(-1, 3)


def random_rotation(rng):
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def edge_args(species, nl):
    return (len(species), species, nl["num_neigh"], nl["neigh_indices"], species[nl["neigh_indices"]],
            nl["xyz"], nl["r"])


NEIGHMASK = 0x1FFFFFFF  # LAMMPS: the bits above it flag special bonds


def fake_lammps(pos, L, cutoff, rng=None, shell=None, ghost_lists=False):
    """A periodic box as LAMMPS holds it on one rank: the local atoms pos[n], then their
    periodic images within `shell` (default `cutoff`) of the box as ghosts, with
    local_of[a] the local atom that atom a is an image of, and full neighbour lists (all
    atoms within `cutoff`, the pair cutoff plus skin) of the local atoms or, with
    ghost_lists (LAMMPS's ghost neighbour request), of every atom.  rng: random
    special-bond flag bits above NEIGHMASK on the list entries."""
    shell = cutoff if shell is None else shell
    n = len(pos)
    k = int(np.ceil(shell / L))
    xs, owner = [pos], [np.arange(n)]
    for s in np.array(np.meshgrid(*[np.arange(-k, k + 1)] * 3, indexing="ij")).reshape(3, -1).T:
        if not s.any():
            continue
        p = pos + s * L
        keep = np.all((p > -shell) & (p < L + shell), axis=1)
        xs.append(p[keep])
        owner.append(np.nonzero(keep)[0])
    x = np.concatenate(xs)
    local_of = np.concatenate(owner).astype(np.int32)
    neighbors = []
    for i in range(len(x) if ghost_lists else n):
        d = np.linalg.norm(x - x[i], axis=1)
        js = np.nonzero((d < cutoff) & (np.arange(len(x)) != i))[0].astype(np.int64)
        if rng is not None:
            js = js | (rng.integers(0, 4, len(js)) << 30)
        neighbors.append((js & 0xFFFFFFFF).astype(np.uint32).view(np.int32))
    return x, local_of, neighbors


def halo_graph(x, n_local, neighbors, r_cut):
    """Nodes and edges of the pair style's no-MPI-message-passing mode
    (pair_symmetrix/pair_symmetrix_mace.cpp:557-655) on one rank: the local atoms
    0..n_local-1, then the ghost atoms within r_cut of a local one in ascending index
    order; per node the list entries within r_cut, in list order.  The neighbour index
    is the neighbour's node, or 0 where a halo node's neighbour is no node (never read).
    Returns node_atom[N0], num_neigh[N0], neigh_indices[E], neigh_atom[E], xyz[E, 3], r[E]."""
    nall = len(x)
    lists = [np.asarray(nb).view(np.uint32).astype(np.int64) & NEIGHMASK for nb in neighbors]
    is_ghost = np.zeros(nall, dtype=bool)
    for i in range(n_local):
        d = x[lists[i]] - x[i]
        near = lists[i][(d * d).sum(1) < r_cut * r_cut]
        is_ghost[near[near >= n_local]] = True
    node_atom = np.concatenate([np.arange(n_local), np.nonzero(is_ghost)[0]])
    node_of = np.zeros(nall, dtype=np.int64)
    node_of[node_atom] = np.arange(len(node_atom))
    num_neigh, nidx, natom, xyz = [], [], [], []
    for a in node_atom:
        d = x[lists[a]] - x[a]
        keep = (d * d).sum(1) < r_cut * r_cut
        num_neigh.append(int(keep.sum()))
        natom.append(lists[a][keep])
        nidx.append(node_of[lists[a][keep]])
        xyz.append(d[keep])
    xyz = np.concatenate(xyz)
    return (node_atom, np.array(num_neigh, dtype=np.int32), np.concatenate(nidx).astype(np.int32),
            np.concatenate(natom), xyz, np.sqrt((xyz * xyz).sum(1)))


def fold_halo_forces(nall, local_of, node_atom, num_neigh, neigh_atom, node_forces):
    """Atomic forces of a halo evaluation after LAMMPS's reverse communication on one
    rank: F_i -= f_e, F_j += f_e on the atoms of each edge, then each ghost's force added
    to the local atom it is an image of."""
    edge_i = np.repeat(node_atom, num_neigh)
    F = atomic_forces(nall, edge_i, neigh_atom, node_forces)
    out = np.zeros((int(local_of.max()) + 1, 3))
    np.add.at(out, local_of, F)
    return out
