"""ctypes front-end to the oracle libraries (test infrastructure only).

`Evaluator(path, which)` drives either the float64 restatement (which="port",
oracle/_build/liborc.so) or the reference's own evaluator (which="reference",
oracle/_ref/libsmx_ref.so) through the same calls, mirroring the reference's
Python binding (symmetrix/source/cpp/mace.cpp:12-243): compute_node_energies_forces
and read-only stage buffers.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_LIBS = {}


def library(which="port"):
    if which in _LIBS:
        return _LIBS[which]
    if which == "port":
        path, pre = _build.build_oracle(), "orc_"
    elif which == "reference":
        path, pre = _build.build_reference(), "ref_"
        if path is None:
            raise FileNotFoundError("reference tree absent: oracle/_ref cannot be built here")
    else:
        raise ValueError(which)
    lib = ctypes.CDLL(path)
    P, I, L, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_double
    ip, dp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
    f = lambda n: getattr(lib, pre + n)
    f("load").restype = P
    f("load").argtypes = [ctypes.c_char_p]
    f("free").argtypes = [P]
    if pre == "orc_":
        f("clone").restype = P
        f("clone").argtypes = [P]
    f("info").argtypes = [P, ip]
    if pre == "orc_":
        f("set_threads").argtypes = [P, I]
        f("set_lean").argtypes = [P, I]
    f("compute").restype = I
    f("compute").argtypes = [P, I, ip, ip, ip, ip, L, dp, dp]
    f("compute_halo").restype = I
    f("compute_halo").argtypes = [P, I, I, ip, ip, ip, ip, L, dp, dp]
    if pre == "ref_":
        f("compute_message_passing").restype = I
        f("compute_message_passing").argtypes = [P, I, I, ip, ip, ip, ip, L, dp, dp, ip]
    f("get").restype = L
    f("get").argtypes = [P, ctypes.c_char_p, dp, L]
    f("last_error").restype = ctypes.c_char_p
    f("zbl_envelope").restype = D
    f("zbl_envelope").argtypes = [D, D, I]
    f("zbl_compute").restype = D
    f("zbl_compute").argtypes = [D, D, dp, dp, I, I, I, I, D, dp]
    f("spline_eval").restype = I
    f("spline_eval").argtypes = [D, dp, dp, I, dp, I, dp, dp]
    f("poly_eval").restype = D
    f("poly_eval").argtypes = [I, dp, I, ip, ip, dp, dp]
    f("mlp_eval").restype = D
    f("mlp_eval").argtypes = [I, I, dp, dp, D, dp, dp]
    _LIBS[which] = (lib, pre)
    return _LIBS[which]


def _ip(a):
    return np.ascontiguousarray(a, dtype=np.int32).ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _dp(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Evaluator:
    def __init__(self, model_path, which="port", _clone_of=None):
        self.lib, self.pre = library(which)
        if _clone_of is not None:
            self.h = getattr(self.lib, "orc_clone")(_clone_of.h)
        else:
            self.h = getattr(self.lib, self.pre + "load")(str(model_path).encode())
        if not self.h:
            raise RuntimeError(getattr(self.lib, self.pre + "last_error")().decode())
        info = (ctypes.c_int * 6)()
        getattr(self.lib, self.pre + "info")(self.h, info)
        self.num_elements, self.num_channels, self.l_max, self.L_max, self.num_lme, self.num_lelm1lm2 = list(info)

    def clone(self):
        """An independent evaluator with the same model (port only), for parallel threads."""
        if self.pre != "orc_":
            raise ValueError("clone() is available for the port only")
        return Evaluator(None, "port", _clone_of=self)

    def set_threads(self, n):
        """Split each stage of one evaluation over n threads (port only; same results bit
        for bit as a serial evaluation)."""
        if self.pre != "orc_":
            raise ValueError("set_threads() is available for the port only")
        getattr(self.lib, "orc_set_threads")(self.h, int(n))
        return self

    def set_lean(self, on=True):
        """Evaluate the radials where they are used instead of storing them per edge (port
        only; for boxes whose per-edge radial rows would not fit in memory).  Same results."""
        if self.pre != "orc_":
            raise ValueError("set_lean() is available for the port only")
        getattr(self.lib, "orc_set_lean")(self.h, 1 if on else 0)
        return self

    def __del__(self):
        if getattr(self, "h", None):
            getattr(self.lib, self.pre + "free")(self.h)
            self.h = None

    def compute_node_energies_forces(self, num_nodes, node_types, num_neigh, neigh_indices, neigh_types, xyz, r):
        keep = [np.ascontiguousarray(node_types, np.int32), np.ascontiguousarray(num_neigh, np.int32),
                np.ascontiguousarray(neigh_indices, np.int32), np.ascontiguousarray(neigh_types, np.int32),
                np.ascontiguousarray(xyz, np.float64).reshape(-1), np.ascontiguousarray(r, np.float64)]
        rc = getattr(self.lib, self.pre + "compute")(self.h, int(num_nodes), _ip(keep[0]), _ip(keep[1]),
                                                     _ip(keep[2]), _ip(keep[3]), len(keep[5]), _dp(keep[4]),
                                                     _dp(keep[5]))
        if rc != 0:
            raise RuntimeError(getattr(self.lib, self.pre + "last_error")().decode())

    def compute_halo(self, num_local_nodes, num_nodes, node_types, num_neigh, neigh_indices, neigh_types, xyz, r):
        """Layer 0 over num_nodes nodes; layer 1, readouts and ZBL over the first
        num_local_nodes (the stage calls of pair_symmetrix_mace.cpp:672-698)."""
        keep = [np.ascontiguousarray(node_types, np.int32), np.ascontiguousarray(num_neigh, np.int32),
                np.ascontiguousarray(neigh_indices, np.int32), np.ascontiguousarray(neigh_types, np.int32),
                np.ascontiguousarray(xyz, np.float64).reshape(-1), np.ascontiguousarray(r, np.float64)]
        rc = getattr(self.lib, self.pre + "compute_halo")(self.h, int(num_local_nodes), int(num_nodes), _ip(keep[0]),
                                                          _ip(keep[1]), _ip(keep[2]), _ip(keep[3]), len(keep[5]),
                                                          _dp(keep[4]), _dp(keep[5]))
        if rc != 0:
            raise RuntimeError(getattr(self.lib, self.pre + "last_error")().decode())

    def compute_message_passing(self, num_nodes, num_atoms, node_types, num_neigh, neigh_atoms, neigh_types, xyz, r,
                                owner):
        """(reference only) The stage calls of the pair style's MPI-message-passing mode on
        one rank (pair_symmetrix_mace.cpp:438-497), the two communications done through
        owner[atom]."""
        if self.pre != "ref_":
            raise ValueError("compute_message_passing() drives the reference build only")
        keep = [np.ascontiguousarray(node_types, np.int32), np.ascontiguousarray(num_neigh, np.int32),
                np.ascontiguousarray(neigh_atoms, np.int32), np.ascontiguousarray(neigh_types, np.int32),
                np.ascontiguousarray(xyz, np.float64).reshape(-1), np.ascontiguousarray(r, np.float64),
                np.ascontiguousarray(owner, np.int32)]
        rc = getattr(self.lib, "ref_compute_message_passing")(
            self.h, int(num_nodes), int(num_atoms), _ip(keep[0]), _ip(keep[1]), _ip(keep[2]), _ip(keep[3]),
            len(keep[5]), _dp(keep[4]), _dp(keep[5]), _ip(keep[6]))
        if rc != 0:
            raise RuntimeError(getattr(self.lib, self.pre + "last_error")().decode())

    def get(self, name):
        n = getattr(self.lib, self.pre + "get")(self.h, name.encode(), None, 0)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n)
        getattr(self.lib, self.pre + "get")(self.h, name.encode(), _dp(out), n)
        return out

    @property
    def node_energies(self):
        return self.get("node_energies")

    @property
    def node_forces(self):
        return self.get("node_forces")
