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
