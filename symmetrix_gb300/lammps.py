"""Python handle on the LAMMPS pair-style adapter (smx_pair_* in include/smx_gb300.h).

LAMMPS itself drives the adapter from C++ (the pair style's compute() passes its own
neighbour list and atom arrays to smx_pair_compute_mode); this wrapper exposes the
same call with numpy arrays for testing and for Python MD drivers that keep
LAMMPS-style ghost atoms.  Semantics follow pair_symmetrix/pair_symmetrix_mace.cpp:
64-77 (the three modes) and :242-748, on one rank.
"""
import ctypes

import numpy as np

from . import _lib

NEIGHMASK = 0x1FFFFFFF  # LAMMPS: the top bits of a neighbour entry flag special bonds

# pair_style symmetrix/mace <mode> -> SMX_PAIR_*
MODES = {"no_domain_decomposition": 0, "mpi_message_passing": 1, "no_mpi_message_passing": 2}


class PairAdapter:
    def __init__(self, mace, mace_types, mode="no_domain_decomposition"):
        """mace: a symmetrix_gb300.MACE; mace_types[t - 1] = model species of LAMMPS type t;
        mode: the pair style's argument (pair_symmetrix_mace.cpp:95-109)."""
        if mode not in MODES:
            raise ValueError(f"The command 'pair_style symmetrix/mace {mode}' is invalid")
        self._mace = mace
        self._lib = mace._lib
        self.mode = mode
        self.mace_types = np.ascontiguousarray(mace_types, dtype=np.int32)
        h = self._lib.smx_pair_create(mace._h)
        if not h:
            raise RuntimeError(self._lib.smx_last_error().decode(errors="replace"))
        self._h = ctypes.c_void_p(h)
        self._keep = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.smx_pair_destroy(h)
            self._h = None

    def compute(self, x, types, local_of, ilist, neighbors, neigh_changed=True, eflag_atom=False, gnum=0):
        """x[nall, 3], types[nall] (1-based), local_of[nall] (may be None in the
        no_mpi_message_passing mode), ilist[inum + gnum] (the local atoms, then gnum ghosts
        with lists), neighbors: one int array of (possibly special-bond flagged) neighbour
        indices per entry of ilist.  Returns (energy, f[nall, 3], eatom[inum] or None,
        virial[6]); f holds the forces before LAMMPS's reverse communication."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        nall = len(x)
        ilist = np.ascontiguousarray(ilist, dtype=np.int32)
        inum = len(ilist) - int(gnum)
        if neigh_changed or self._keep is None:
            numneigh = np.zeros(nall, dtype=np.int32)
            lists = [np.ascontiguousarray(nb, dtype=np.int32) for nb in neighbors]
            ptrs = (ctypes.c_void_p * nall)()
            for ii, i in enumerate(ilist):
                numneigh[i] = len(lists[ii])
                ptrs[i] = lists[ii].ctypes.data if len(lists[ii]) else None
            lo = None if local_of is None else np.ascontiguousarray(local_of, dtype=np.int32)
            self._keep = (numneigh, lists, ptrs, np.ascontiguousarray(types, dtype=np.int32), lo, ilist)
        numneigh, lists, ptrs, t, lo, il = self._keep
        f = np.zeros((nall, 3))
        e = ctypes.c_double(0.0)
        eatom = np.zeros(inum) if eflag_atom else None
        vir = np.zeros(6)
        P = lambda a: ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else None
        code = self._lib.smx_pair_compute_mode(self._h, MODES[self.mode], inum, int(gnum), nall, P(il), P(numneigh),
                                               ctypes.cast(ptrs, ctypes.c_void_p), NEIGHMASK,
                                               int(bool(neigh_changed)), P(x), P(t), P(lo), P(self.mace_types),
                                               len(self.mace_types), 1, int(eflag_atom), 1, P(f), ctypes.byref(e),
                                               P(eatom), P(vir))
        _lib.raise_for(code, self._lib)
        return e.value, f, eatom, vir
