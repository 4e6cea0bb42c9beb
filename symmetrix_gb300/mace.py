"""`MACE`: the Python face of the GB300 engine, shaped like the reference binding.

Mirrors `symmetrix.MACE` (symmetrix/source/cpp/mace.cpp:12-243): construct from a
JSON model path, call `compute_node_energies_forces(num_nodes, node_types,
num_neigh, neigh_indices, neigh_types, xyz, r)`, then read `node_energies` and
`node_forces` (= -dE/dxyz per directed edge).  Stage buffers (`A0`, `M0`, `H1`,
`Phi1`, `A1`, `M1`, `H2` and the `*_adj` adjoints) are attributes as in the reference
binding; those of the separately launched stages are also writable (`M0`, `H1`, `Phi1`,
`A1`, `M0_adj`, `H1_adj`, `Phi1_adj`, `A1_adj`), and the binding's per-stage calls
compute_H1 / reverse_H1, compute_Phi1 / reverse_Phi1 and compute_A1 / reverse_A1 run
single GPU launches on them, so stage-level checks read like the reference's
test_mace.py.  compute_R1 and compute_Y record their edge inputs for compute_Phi1,
which evaluates R1 and Y in its own kernel; the stages fused into one kernel (the
layer-0 stages; compute_A1_scaled, compute_M1, compute_H2, compute_readouts and their
reverses) run only inside compute_node_energies_forces.  Errors raise ValueError /
RuntimeError like the reference binding.
"""
import ctypes

import numpy as np

from . import _lib

STAGES = ("A0", "M0", "H1", "Phi1", "A1", "M1", "H2", "A0_adj", "M0_adj", "H1_adj", "Phi1_adj", "A1_adj",
          "M1_adj", "H2_adj")
WRITABLE = ("M0", "H1", "Phi1", "A1", "M0_adj", "H1_adj", "Phi1_adj", "A1_adj")


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else None


def save_model_cache(model_path, cache_path):
    """Parse a JSON model once and write the binary model cache that MACE() loads in its place."""
    lib = _lib.load()
    _lib.raise_for(lib.smx_save_model_cache(str(model_path).encode(), str(cache_path).encode()), lib)


# precision names -> SMX_PRECISION_* (include/smx_gb300.h)
PRECISIONS = {"float32": 0, "fp32": 0, "bfloat16": 1, "bf16": 1}


class MACE:
    def __init__(self, filename, device=0, precision="float32", keep_stages=False):
        self._lib = _lib.load()
        if precision not in PRECISIONS:
            raise ValueError(f"unsupported precision '{precision}'")
        self.precision = "bfloat16" if PRECISIONS[precision] == 1 else "float32"
        h = self._lib.smx_create(str(filename).encode(), PRECISIONS[precision], int(device))
        if not h:
            msg = self._lib.smx_last_error().decode(errors="replace")
            raise RuntimeError(msg)
        self._h = ctypes.c_void_p(h)
        if keep_stages:
            _lib.raise_for(self._lib.smx_set_option(self._h, b"keep_stages", 1))
        n = self._lib.smx_num_elements(self._h)
        buf = (ctypes.c_int * n)()
        self._lib.smx_atomic_numbers(self._h, ctypes.cast(buf, ctypes.c_void_p), n)
        self.atomic_numbers = list(buf)
        self.num_elements = n
        self.num_channels = self._lib.smx_num_channels(self._h)
        self.r_cut = self._lib.smx_r_cut(self._h)
        self.l_max = self._lib.smx_l_max(self._h)
        self.L_max = self._lib.smx_L_max(self._h)
        self.num_LM = self._lib.smx_num_LM(self._h)
        self.node_energies = np.zeros(0)
        self.node_forces = np.zeros(0)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.smx_destroy(h)
            self._h = None

    @property
    def has_zbl(self):
        """Whether the model adds the ZBL pair repulsion (MACE::has_zbl)."""
        return self._lib.smx_has_zbl(self._h) == 1

    def compute_node_energies_forces(self, num_nodes, node_types, num_neigh, neigh_indices, neigh_types, xyz, r):
        node_types = np.ascontiguousarray(node_types, dtype=np.int32)[:num_nodes]
        num_neigh = np.ascontiguousarray(num_neigh, dtype=np.int32)[:num_nodes]
        neigh_indices = np.ascontiguousarray(neigh_indices, dtype=np.int32)
        neigh_types = np.ascontiguousarray(neigh_types, dtype=np.int32)
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        r = np.ascontiguousarray(r, dtype=np.float64)
        E = len(r)
        if len(neigh_indices) != E or len(neigh_types) != E or len(xyz) != 3 * E:
            raise ValueError("edge arrays have inconsistent lengths")
        energies = np.zeros(num_nodes)
        forces = np.zeros(3 * E)
        code = self._lib.smx_compute_node_energies_forces(
            self._h, int(num_nodes), _ptr(node_types), _ptr(num_neigh), _ptr(neigh_indices), _ptr(neigh_types), E,
            _ptr(xyz), _ptr(r), _ptr(energies), _ptr(forces))
        _lib.raise_for(code, self._lib)
        self.node_energies = energies
        self.node_forces = forces

    def compute_halo(self, num_local_nodes, num_nodes, node_types, num_neigh, neigh_indices, neigh_types, xyz, r):
        """The stage calls of the pair style's no-MPI-message-passing mode
        (pair_symmetrix_mace.cpp:672-698): layer 0 over all num_nodes nodes; ZBL, layer 1
        and the readouts over the first num_local_nodes.  node_energies gets
        num_local_nodes values, node_forces one triple per edge of every node."""
        node_types = np.ascontiguousarray(node_types, dtype=np.int32)[:num_nodes]
        num_neigh = np.ascontiguousarray(num_neigh, dtype=np.int32)[:num_nodes]
        neigh_indices = np.ascontiguousarray(neigh_indices, dtype=np.int32)
        neigh_types = np.ascontiguousarray(neigh_types, dtype=np.int32)
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        r = np.ascontiguousarray(r, dtype=np.float64)
        E = len(r)
        if len(neigh_indices) != E or len(neigh_types) != E or len(xyz) != 3 * E:
            raise ValueError("edge arrays have inconsistent lengths")
        energies = np.zeros(max(int(num_local_nodes), 0))
        forces = np.zeros(3 * E)
        code = self._lib.smx_compute_halo(
            self._h, int(num_local_nodes), int(num_nodes), _ptr(node_types), _ptr(num_neigh), _ptr(neigh_indices),
            _ptr(neigh_types), E, _ptr(xyz), _ptr(r), _ptr(energies), _ptr(forces))
        _lib.raise_for(code, self._lib)
        self.node_energies = energies
        self.node_forces = forces

    def compute_device(self, num_nodes, node_types, num_neigh, neigh_indices, neigh_types, num_edges, xyz, r,
                       node_energies, node_forces, stream=None):
        """Device-pointer variant: every argument is an integer device address."""
        code = self._lib.smx_compute_node_energies_forces_device(
            self._h, int(num_nodes), node_types, num_neigh, neigh_indices, neigh_types, int(num_edges), xyz, r,
            node_energies, node_forces, stream)
        _lib.raise_for(code, self._lib)

    def sync(self, stream=None):
        """Wait for `stream` (default: the engine's) and raise TimeoutError if a bounded
        device-side wait gave up in the work enqueued since the last check."""
        _lib.raise_for(self._lib.smx_sync(self._h, stream), self._lib)

    def compute_atoms(self, positions, species, box=None):
        """Energy, node energies, atomic forces (n, 3) and virial (3, 3) of a structure.

        Builds the neighbour list on the GPU (box = three orthorhombic lengths, or None
        for a non-periodic system), like the reference's callers do around
        compute_node_energies_forces (symmetrix_calc.py:72-102).
        """
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        n = len(pos)
        sp = np.ascontiguousarray(species, dtype=np.int32)
        if len(sp) != n:
            raise ValueError("species and positions differ in length")
        bx = None if box is None else np.ascontiguousarray(np.broadcast_to(box, 3), dtype=np.float64)
        e = ctypes.c_double(0.0)
        node_e = np.zeros(n)
        forces = np.zeros((n, 3))
        virial = np.zeros(9)
        code = self._lib.smx_compute_atoms(self._h, n, _ptr(pos), _ptr(sp), _ptr(bx), ctypes.byref(e), _ptr(node_e),
                                           _ptr(forces), _ptr(virial))
        _lib.raise_for(code, self._lib)
        return e.value, node_e, forces, virial.reshape(3, 3)

    def compute_molecules(self, molecules):
        """Batching form: evaluate many independent non-periodic molecules in one pass.

        molecules: sequence of (positions (n, 3), species (n,)).  Returns (energies per
        molecule, list of node-energy arrays, list of force arrays)."""
        pos = [np.asarray(p, dtype=np.float64).reshape(-1, 3) for p, _ in molecules]
        sp = [np.asarray(s, dtype=np.int32).reshape(-1) for _, s in molecules]
        counts = np.array([len(p) for p in pos], dtype=np.int64)
        if any(len(a) != len(b) for a, b in zip(pos, sp)):
            raise ValueError("species and positions differ in length")
        first = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        X = np.ascontiguousarray(np.concatenate(pos) if pos else np.zeros((0, 3)))
        S = np.ascontiguousarray(np.concatenate(sp) if sp else np.zeros(0, np.int32))
        n = len(X)
        e_mol = np.zeros(len(pos))
        node_e = np.zeros(n)
        F = np.zeros((n, 3))
        code = self._lib.smx_compute_molecules(self._h, len(pos), _ptr(first), _ptr(X), _ptr(S), _ptr(e_mol),
                                               _ptr(node_e), _ptr(F))
        _lib.raise_for(code, self._lib)
        return e_mol, np.split(node_e, first[1:-1]), np.split(F, first[1:-1])

    @property
    def stream(self):
        """Address of the engine's CUDA stream (host-pointer calls and MD run on it)."""
        return self._lib.smx_engine_stream(self._h)

    def set_option(self, key, value):
        _lib.raise_for(self._lib.smx_set_option(self._h, key.encode(), int(value)), self._lib)

    def get_option(self, key):
        return self._lib.smx_get_option(self._h, key.encode())

    def gemm_schedule(self):
        """The tensor-core GEMM schedule the autotuner picked (BF16 form)."""
        return {g: {"NT": self.get_option(f"tc_nt_{g}"), "stages": self.get_option(f"tc_stages_{g}"),
                    "us": self.get_option(f"tc_tuned_ns_{g}") / 1e3} for g in ("H1", "A1", "Phi1_adj", "M0_adj")}

    def stage_times(self):
        """Per-stage device times (ms) of the last evaluation; needs set_option('profile', 1)."""
        out = np.zeros(16)
        n = self._lib.smx_stage_times(self._h, _ptr(out), 16)
        if n < 0:
            _lib.raise_for(-n, self._lib)
        return dict(zip(_lib.STAGE_NAMES, out[:n]))

    def stage(self, name):
        """A stage buffer of the last evaluation as float64 (reference layout)."""
        n = self._lib.smx_get_stage(self._h, name.encode(), None, 0)
        if n == -1:
            raise KeyError(name)
        if n < 0:
            raise RuntimeError(self._lib.smx_last_error().decode(errors="replace"))
        out = np.zeros(n)
        if n > 0 and self._lib.smx_get_stage(self._h, name.encode(), _ptr(out), n) < 0:
            raise RuntimeError(self._lib.smx_last_error().decode(errors="replace"))
        return out

    def __getattr__(self, name):
        if name in STAGES:
            return self.stage(name)
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in WRITABLE:
            self.set_stage(name, value)
        else:
            object.__setattr__(self, name, value)

    def set_stage(self, name, values):
        """Write a stage buffer of the current node count (float64 values, the layout stage() reads)."""
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        n = self._lib.smx_set_stage(self._h, name.encode(), _ptr(v), v.size)
        if n < 0:
            _lib.raise_for(-n, self._lib)

    # ---- per-stage calls (symmetrix/source/cpp/mace.cpp:52-179) ----
    def _run(self, stage, num_nodes, edges=None, flags=0):
        if edges is None:
            code = self._lib.smx_run_stage(self._h, stage.encode(), int(num_nodes), None, None, None, None, 0, None,
                                           None, flags)
        else:
            node_types, num_neigh, neigh_indices, neigh_types, xyz, r = edges
            a = [np.ascontiguousarray(node_types, np.int32)[:num_nodes],
                 np.ascontiguousarray(num_neigh, np.int32)[:num_nodes], np.ascontiguousarray(neigh_indices, np.int32),
                 np.ascontiguousarray(neigh_types, np.int32), np.ascontiguousarray(xyz, np.float64).reshape(-1),
                 np.ascontiguousarray(r, np.float64)]
            E = len(a[5])
            if len(a[2]) != E or len(a[3]) != E or len(a[4]) != 3 * E:
                raise ValueError("edge arrays have inconsistent lengths")
            code = self._lib.smx_run_stage(self._h, stage.encode(), int(num_nodes), _ptr(a[0]), _ptr(a[1]),
                                           _ptr(a[2]), _ptr(a[3]), E, _ptr(a[4]), _ptr(a[5]), flags)
        _lib.raise_for(code, self._lib)

    def compute_R1(self, num_nodes, node_types, num_neigh, neigh_types, r):
        """Records the centre/neighbour species and edge lengths for compute_Phi1, whose
        kernel evaluates the radials R1 itself (no R1 buffer)."""
        object.__setattr__(self, "_r1_args", (np.array(node_types), np.array(neigh_types), np.array(r)))

    def compute_Y(self, xyz):
        """Records the edge vectors for compute_Phi1, whose kernel evaluates Y itself."""
        object.__setattr__(self, "_y_args", np.array(xyz, dtype=np.float64))

    def compute_Phi1(self, num_nodes, num_neigh, neigh_indices):
        """Phi1 from H1 on the edges of compute_R1 / compute_Y (mace.cpp:453-502)."""
        node_types, neigh_types, r = self._r1_args
        self._run("compute_Phi1", num_nodes, (node_types, num_neigh, neigh_indices, neigh_types, self._y_args, r))

    def reverse_Phi1(self, num_nodes, num_neigh, neigh_indices, xyz, r, zero_dxyz, zero_H1_adj):
        """H1_adj and node_forces from Phi1_adj (mace.cpp:504-605), with the reference's two flags."""
        node_types, neigh_types, _ = self._r1_args
        if not zero_dxyz:  # add to the current node_forces, as the reference does
            self.set_stage("node_forces", self.node_forces)
        self._run("reverse_Phi1", num_nodes, (node_types, num_neigh, neigh_indices, neigh_types, xyz, r),
                  (1 if zero_dxyz else 0) | (2 if zero_H1_adj else 0))
        object.__setattr__(self, "node_forces", self.stage("node_forces"))

    def compute_H1(self, num_nodes):
        self._run("compute_H1", num_nodes)

    def reverse_H1(self, num_nodes):
        self._run("reverse_H1", num_nodes)

    def compute_A1(self, num_nodes):
        self._run("compute_A1", num_nodes)

    def reverse_A1(self, num_nodes):
        self._run("reverse_A1", num_nodes)


class MACEKokkos(MACE):
    """The name of the reference's Kokkos evaluator class (symmetrix/source/cpp/mace_kokkos.cpp),
    which the reference's calculator picks for dtype "float64" (symmetrix_calc.py:49): here the
    FP32 plain form, the engine having no float64 GPU form (its forces are within 1e-5 eV/A
    of the float64 evaluator)."""

    def __init__(self, filename, device=0, keep_stages=False):
        super().__init__(filename, device=device, precision="float32", keep_stages=keep_stages)


class MACEKokkosFloat(MACEKokkos):
    """The reference's single-precision Kokkos class name: the FP32 plain form."""


_kokkos_ready = False


def _init_kokkos():
    """The reference initialises Kokkos once per process before building a Kokkos
    evaluator (symmetrix_calc.py:47-48); the engine needs no runtime set-up, so this
    only records the call."""
    global _kokkos_ready
    _kokkos_ready = True


def _kokkos_is_initialized():
    return _kokkos_ready
