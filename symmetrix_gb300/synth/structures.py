"""Seeded synthetic structures and host-side neighbour lists.

Structures are built by random sequential insertion with a minimum pair
distance: periodic cubic boxes sized from a number density, or non-periodic
molecules in spheres.  `neighbor_list` returns the full directed list in the
layout the evaluator takes (libsymmetrix/source/mace.hpp:29-35): edges grouped
by centre atom i in increasing i, num_neigh[i], neigh_indices[e] = j,
xyz[e] = x_j - x_i (+ periodic image), r[e] = |xyz[e]|, as the LAMMPS pair style
builds them (pair_pair_symmetrix_mace.cpp:242-315) and as ASE's
neighbor_list('ijdD') returns them (symmetrix_calc.py:77).
"""
import numpy as np

from .model import atomic_number

# standard atomic masses (amu) for the species the workloads use
MASSES = {1: 1.008, 6: 12.011, 7: 14.007, 8: 15.999, 9: 18.998, 11: 22.990, 12: 24.305, 13: 26.982,
          14: 28.085, 16: 32.06, 17: 35.45}
KB_EV = 8.617333262e-5          # eV / K
TIME_UNIT_FS = 10.180505710774  # sqrt(amu A^2 / eV) in fs


def _insert(rng, n, lo, hi, min_dist, inside, periodic_L=None, max_tries=2000, cell=None):
    """Random sequential insertion on a hash grid (cell >= min_dist)."""
    cell = min_dist if cell is None else cell
    grid = {}
    pos = np.zeros((n, 3))
    md2 = min_dist * min_dist
    for a in range(n):
        for _ in range(max_tries):
            p = lo + (hi - lo) * rng.random(3)
            if not inside(p):
                continue
            c = np.floor(p / cell).astype(int)
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        key = (c[0] + dx, c[1] + dy, c[2] + dz)
                        if periodic_L is not None:
                            nc = int(np.floor(periodic_L / cell))
                            key = (key[0] % nc, key[1] % nc, key[2] % nc)
                        for b in grid.get(key, ()):
                            d = p - pos[b]
                            if periodic_L is not None:
                                d -= periodic_L * np.round(d / periodic_L)
                            if d @ d < md2:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                pos[a] = p
                key = tuple(c)
                if periodic_L is not None:
                    nc = int(np.floor(periodic_L / cell))
                    key = (key[0] % nc, key[1] % nc, key[2] % nc)
                grid.setdefault(key, []).append(a)
                break
        else:
            raise RuntimeError("random insertion failed: density too high for min_dist")
    return pos


def random_box(n_atoms, density, min_dist, n_species, seed, probs=None):
    """Periodic cubic box: (positions [n,3], box length, species index per atom)."""
    rng = np.random.default_rng(seed)
    L = (n_atoms / density) ** (1.0 / 3.0)
    # the hash-grid cell must tile the box exactly for the periodic check
    cell = L / np.floor(L / min_dist)
    pos = _insert(rng, n_atoms, np.zeros(3), np.full(3, L), min_dist, lambda p: True, periodic_L=L, cell=cell)
    species = rng.choice(n_species, size=n_atoms, p=probs)
    return pos, L, species.astype(np.int32)


def random_molecule(n_atoms, density, min_dist, n_species, rng, probs=None):
    """Non-periodic cluster in a sphere of the given number density."""
    R = (3.0 * n_atoms / (4.0 * np.pi * density)) ** (1.0 / 3.0)
    pos = _insert(rng, n_atoms, np.full(3, -R), np.full(3, R), min_dist, lambda p: p @ p <= R * R)
    species = rng.choice(n_species, size=n_atoms, p=probs)
    return pos, species.astype(np.int32)


def neighbor_list(pos, cutoff, box=None):
    """Full directed neighbour list in evaluator layout.

    Returns dict(num_neigh[N] int32, neigh_indices[E] int32, xyz[E,3] f64, r[E] f64,
    i[E] int32, shift[E,3] f64).  Periodic images are enumerated explicitly, so any
    box size works; edges are sorted by (i, j, image).
    """
    pos = np.asarray(pos, dtype=np.float64)
    N = len(pos)
    if box is None:
        images = np.zeros((1, 3))
    else:
        n = int(np.ceil(cutoff / box))
        rngi = np.arange(-n, n + 1)
        images = np.array(np.meshgrid(rngi, rngi, rngi, indexing="ij")).reshape(3, -1).T * box
        pos = pos - box * np.floor(pos / box)
    try:
        from scipy.spatial import cKDTree
    except ImportError:  # pragma: no cover
        cKDTree = None
    I, J, S = [], [], []
    if cKDTree is not None and N > 64:
        tree = cKDTree(pos)
        for s in images:
            pairs = tree.query_ball_point(pos + s, cutoff, return_sorted=False)
            # pos[j] + s is a neighbour of pos[i]  <=>  |pos[j] + s - pos[i]| < cutoff
            # query_ball_point(pos + s) finds, for each k, atoms j with |pos[j] - (pos[k] + s)| < c,
            # i.e. centre k sees atom j through image -s.
            for k, js in enumerate(pairs):
                if js:
                    js = np.asarray(js)
                    I.append(np.full(len(js), k))
                    J.append(js)
                    S.append(np.repeat(-s[None, :], len(js), axis=0))
    else:
        for s in images:
            d = pos[None, :, :] + s[None, None, :] - pos[:, None, :]
            r2 = np.einsum("ijk,ijk->ij", d, d)
            ii, jj = np.nonzero(r2 < cutoff * cutoff)
            I.append(ii)
            J.append(jj)
            S.append(np.repeat(s[None, :], len(ii), axis=0))
    I = np.concatenate(I) if I else np.zeros(0, int)
    J = np.concatenate(J) if J else np.zeros(0, int)
    S = np.concatenate(S) if S else np.zeros((0, 3))
    D = pos[J] + S - pos[I]
    r = np.linalg.norm(D, axis=1)
    keep = (r > 1e-8) & (r < cutoff)
    I, J, S, D, r = I[keep], J[keep], S[keep], D[keep], r[keep]
    order = np.lexsort((S[:, 2], S[:, 1], S[:, 0], J, I))
    I, J, S, D, r = I[order], J[order], S[order], D[order], r[order]
    num_neigh = np.bincount(I, minlength=N).astype(np.int32)
    return dict(num_neigh=num_neigh, neigh_indices=J.astype(np.int32), xyz=np.ascontiguousarray(D),
                r=np.ascontiguousarray(r), i=I.astype(np.int32), shift=S)


def lammps_rank(pos, box, cutoff, shell, ghost_lists=True):
    """A periodic cubic box as one LAMMPS rank holds it (one process, no domain
    decomposition): the local atoms pos[n] wrapped into the box, then their periodic
    images within `shell` of it as ghosts; local_of[a] is the local atom that atom a is
    an image of (atom->map(atom->tag[a])), and lists[a] the full neighbour list of atom a
    (all atoms within `cutoff`, LAMMPS's pair cutoff plus skin, ascending index) for
    the local atoms or, with ghost_lists (LAMMPS's ghost neighbour request), for every
    atom.  Returns x[nall, 3], local_of[nall] int32, lists (int32 arrays)."""
    pos = np.asarray(pos, dtype=np.float64)
    pos = pos - box * np.floor(pos / box)
    n = len(pos)
    k = int(np.ceil(shell / box))
    xs, owner = [pos], [np.arange(n)]
    for s in np.array(np.meshgrid(*[np.arange(-k, k + 1)] * 3, indexing="ij")).reshape(3, -1).T:
        if not s.any():
            continue
        p = pos + s * box
        keep = np.all((p > -shell) & (p < box + shell), axis=1)
        xs.append(p[keep])
        owner.append(np.nonzero(keep)[0])
    x = np.concatenate(xs)
    local_of = np.concatenate(owner).astype(np.int32)
    from scipy.spatial import cKDTree
    centres = x if ghost_lists else x[:n]
    found = cKDTree(x).query_ball_point(centres, cutoff, return_sorted=True)
    lists = []
    for a, js in enumerate(found):
        js = np.asarray(js, dtype=np.int32)
        lists.append(js[js != a])
    return x, local_of, lists


def maxwell_boltzmann(masses, T, rng):
    """Velocities in A/fs at temperature T (K) with zero net momentum (masses in amu)."""
    m = np.asarray(masses, dtype=np.float64)[:, None]
    v = rng.normal(size=(len(m), 3)) * np.sqrt(KB_EV * T / m) / TIME_UNIT_FS
    v -= (m * v).sum(0) / m.sum()
    return v


def species_masses(atomic_numbers, species):
    return np.array([MASSES[atomic_numbers[s]] for s in species])
