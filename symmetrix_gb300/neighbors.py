"""Host neighbour list for general (triclinic, mixed-periodicity) cells.

Returns the full directed list in the evaluator's layout (libsymmetrix/source/mace.hpp:29-35),
the same list ASE's neighbor_list('ijdD') gives the reference calculator
(symmetrix/source/symmetrix/symmetrix_calc.py:77): edges grouped by centre i in increasing
order, num_neigh[i], neigh_indices[e] = j, xyz[e] = x_j + S_e - x_i with S_e a lattice
translation, r[e] = |xyz[e]| < cutoff; self pairs only through a non-zero translation.

Orthorhombic fully periodic and non-periodic systems are better served by the engine's
GPU cell list (MACE.compute_atoms); this list is the general fallback of the calculator.
"""
import numpy as np


def _image_range(cell, pbc, cutoff):
    """Translations n (integers per axis) whose lattice vectors can bring an atom inside the cutoff."""
    cell = np.asarray(cell, dtype=np.float64)
    vol = abs(np.linalg.det(cell))
    n = [0, 0, 0]
    for a in range(3):
        if not pbc[a]:
            continue
        b, c = cell[(a + 1) % 3], cell[(a + 2) % 3]
        area = np.linalg.norm(np.cross(b, c))
        if vol <= 0.0 or area <= 0.0:
            raise ValueError("periodic direction with a degenerate cell")
        spacing = vol / area  # distance between lattice planes normal to axis a
        n[a] = int(np.ceil(cutoff / spacing))
    return n


def neighbor_list_cell(positions, cell, pbc, cutoff):
    pos = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
    N = len(pos)
    cell = np.asarray(cell, dtype=np.float64).reshape(3, 3)
    pbc = [bool(p) for p in np.broadcast_to(pbc, 3)]
    nr = _image_range(cell, pbc, cutoff)
    grids = [np.arange(-nr[a], nr[a] + 1) for a in range(3)]
    shifts = np.array(np.meshgrid(*grids, indexing="ij")).reshape(3, -1).T.astype(np.float64) @ cell
    I, J, D = [], [], []
    try:
        from scipy.spatial import cKDTree
    except ImportError:  # pragma: no cover
        cKDTree = None
    if cKDTree is not None and N > 64:
        tree = cKDTree(pos)
        for s in shifts:
            # atoms j with |pos[j] + s - pos[i]| < cutoff  <=>  j within cutoff of pos[i] - s
            found = tree.query_ball_point(pos - s, cutoff, return_sorted=False)
            for i, js in enumerate(found):
                if js:
                    js = np.asarray(js)
                    I.append(np.full(len(js), i))
                    J.append(js)
                    D.append(pos[js] + s - pos[i])
    else:
        for s in shifts:
            d = pos[None, :, :] + s - pos[:, None, :]
            r2 = np.einsum("ijk,ijk->ij", d, d)
            ii, jj = np.nonzero(r2 < cutoff * cutoff)
            I.append(ii)
            J.append(jj)
            D.append(d[ii, jj])
    I = np.concatenate(I) if I else np.zeros(0, np.int64)
    J = np.concatenate(J) if J else np.zeros(0, np.int64)
    D = np.concatenate(D) if D else np.zeros((0, 3))
    r = np.linalg.norm(D, axis=1)
    keep = (r > 1e-8) & (r < cutoff)
    I, J, D, r = I[keep], J[keep], D[keep], r[keep]
    order = np.lexsort((D[:, 2], D[:, 1], D[:, 0], J, I))
    I, J, D, r = I[order], J[order], D[order], r[order]
    return dict(num_neigh=np.bincount(I, minlength=N).astype(np.int32), neigh_indices=J.astype(np.int32),
                xyz=np.ascontiguousarray(D), r=np.ascontiguousarray(r), i=I.astype(np.int32))
