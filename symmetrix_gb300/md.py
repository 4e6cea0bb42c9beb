"""GPU-resident velocity-Verlet molecular dynamics over the engine (smx_md_* in the C ABI).

Units: A, fs, amu, eV.  The neighbour list uses r_cut + skin and is rebuilt every
`rebuild_every` steps; the steps in between run as one captured CUDA graph.
"""
import ctypes

import numpy as np

from . import _lib
from .mace import _ptr


class MD:
    def __init__(self, engine, positions, species, masses, box=None, velocities=None, dt=0.5, skin=1.0,
                 rebuild_every=10, mol_first=None):
        """mol_first: optional molecule offsets (batching form): the atoms form independent
        non-periodic molecules [mol_first[m], mol_first[m+1]); box must then be None."""
        self._lib = _lib.load()
        self.engine = engine  # keeps the engine alive
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        self.n = len(pos)
        sp = np.ascontiguousarray(species, dtype=np.int32)
        m = np.ascontiguousarray(masses, dtype=np.float64)
        v = None if velocities is None else np.ascontiguousarray(velocities, dtype=np.float64).reshape(-1, 3)
        bx = None if box is None else np.ascontiguousarray(np.broadcast_to(box, 3), dtype=np.float64)
        if mol_first is not None:
            if box is not None:
                raise ValueError("a batch of molecules is non-periodic: box must be None")
            mf = np.ascontiguousarray(mol_first, dtype=np.int32)
            h = self._lib.smx_md_create_molecules(engine._h, len(mf) - 1, _ptr(mf), _ptr(pos), _ptr(v), _ptr(sp),
                                                  _ptr(m), float(dt), float(skin), int(rebuild_every))
        else:
            h = self._lib.smx_md_create(engine._h, self.n, _ptr(pos), _ptr(v), _ptr(sp), _ptr(m), _ptr(bx),
                                        float(dt), float(skin), int(rebuild_every))
        if not h:
            raise RuntimeError(self._lib.smx_last_error().decode(errors="replace"))
        self._h = ctypes.c_void_p(h)

    def run(self, steps):
        _lib.raise_for(self._lib.smx_md_run(self._h, int(steps)), self._lib)

    def sync(self):
        _lib.raise_for(self._lib.smx_md_sync(self._h), self._lib)

    def state(self):
        pos = np.zeros((self.n, 3))
        vel = np.zeros((self.n, 3))
        f = np.zeros((self.n, 3))
        e = ctypes.c_double(0.0)
        w = np.zeros(9)
        step = ctypes.c_long(0)
        _lib.raise_for(self._lib.smx_md_state(self._h, _ptr(pos), _ptr(vel), _ptr(f), ctypes.byref(e), _ptr(w),
                                              ctypes.byref(step)), self._lib)
        return dict(positions=pos, velocities=vel, forces=f, potential_energy=e.value, virial=w.reshape(3, 3),
                    step=step.value)

    @property
    def num_edges(self):
        return self._lib.smx_md_num_edges(self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.smx_md_destroy(h)
            self._h = None


def relax_fire(engine, positions, species, box=None, steps=300, fmax=0.05, dt=0.5, dt_max=2.0, maxmove=0.1):
    """FIRE minimisation (Bitzek et al., PRL 97, 170201 (2006)) with atom-level GPU
    evaluations; unit masses, time in fs.  Returns (positions, energy, max |F|)."""
    x = np.array(positions, dtype=np.float64).reshape(-1, 3)
    v = np.zeros_like(x)
    alpha, n_pos = 0.1, 0
    E, _, F, _ = engine.compute_atoms(x, species, box=box)
    for _ in range(steps):
        fm = np.abs(F).max()
        if fm < fmax:
            break
        P = float((F * v).sum())
        if P > 0:
            vn, fn = np.linalg.norm(v), np.linalg.norm(F)
            v = (1 - alpha) * v + alpha * F * (vn / max(fn, 1e-300))
            n_pos += 1
            if n_pos > 5:
                dt = min(dt * 1.1, dt_max)
                alpha *= 0.99
        else:
            v[:] = 0.0
            dt *= 0.5
            alpha, n_pos = 0.1, 0
        v += dt * F
        dx = dt * v
        big = np.linalg.norm(dx, axis=1).max()
        if big > maxmove:
            dx *= maxmove / big
        x += dx
        E, _, F, _ = engine.compute_atoms(x, species, box=box)
    return x, E, float(np.abs(F).max())
