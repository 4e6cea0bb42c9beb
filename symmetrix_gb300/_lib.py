"""ctypes binding of libsmx_gb300.so (include/smx_gb300.h).

The engine is native only: if the library has not been built, or no CUDA
device is usable, calls raise instead of falling back to anything else.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsmx_gb300.so")

SMX_OK = 0
ERRORS = {1: ValueError, 2: RuntimeError, 3: RuntimeError, 4: MemoryError, 5: TimeoutError}

# (name, restype, argtypes) for every entry point declared in include/smx_gb300.h
_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_long
_D = ctypes.c_double
_S = ctypes.c_char_p
SIGNATURES = [
    ("smx_save_model_cache", _I, [_S, _S]),
    ("smx_create", _P, [_S, _I, _I]),
    ("smx_destroy", None, [_P]),
    ("smx_last_error", _S, []),
    ("smx_num_elements", _I, [_P]),
    ("smx_num_channels", _I, [_P]),
    ("smx_r_cut", _D, [_P]),
    ("smx_l_max", _I, [_P]),
    ("smx_L_max", _I, [_P]),
    ("smx_num_LM", _I, [_P]),
    ("smx_has_zbl", _I, [_P]),
    ("smx_atomic_numbers", _I, [_P, _P, _I]),
    ("smx_compute_node_energies_forces", _I, [_P, _I, _P, _P, _P, _P, _L, _P, _P, _P, _P]),
    ("smx_compute_halo", _I, [_P, _I, _I, _P, _P, _P, _P, _L, _P, _P, _P, _P]),
    ("smx_compute_node_energies_forces_device", _I, [_P, _I, _P, _P, _P, _P, _L, _P, _P, _P, _P, _P]),
    ("smx_sync", _I, [_P, _P]),
    ("smx_get_stage", _L, [_P, _S, _P, _L]),
    ("smx_set_stage", _L, [_P, _S, _P, _L]),
    ("smx_run_stage", _I, [_P, _S, _I, _P, _P, _P, _P, _L, _P, _P, _I]),
    ("smx_set_option", _I, [_P, _S, _L]),
    ("smx_get_option", _L, [_P, _S]),
    ("smx_engine_stream", _P, [_P]),
    ("smx_stage_times", _I, [_P, _P, _I]),
    ("smx_compute_atoms", _I, [_P, _I, _P, _P, _P, _P, _P, _P, _P]),
    ("smx_md_create", _P, [_P, _I, _P, _P, _P, _P, _P, _D, _D, _I]),
    ("smx_md_run", _I, [_P, _I]),
    ("smx_md_sync", _I, [_P]),
    ("smx_md_state", _I, [_P, _P, _P, _P, _P, _P, _P]),
    ("smx_md_num_edges", _L, [_P]),
    ("smx_md_destroy", None, [_P]),
    ("smx_energy_virial_device_noalloc", _I, [_I, _L, _P, _P, _P, _P, _P]),
    ("smx_compute_molecules", _I, [_P, _I, _P, _P, _P, _P, _P, _P]),
    ("smx_md_create_molecules", _P, [_P, _I, _P, _P, _P, _P, _P, _D, _D, _I]),
    ("smx_pair_create", _P, [_P]),
    ("smx_pair_destroy", None, [_P]),
    ("smx_pair_compute", _I, [_P, _I, _I, _P, _P, _P, _I, _I, _P, _P, _P, _P, _I, _I, _I, _I, _P, _P, _P, _P]),
    ("smx_pair_compute_mode", _I, [_P, _I, _I, _I, _I, _P, _P, _P, _I, _I, _P, _P, _P, _P, _I, _I, _I, _I, _P, _P,
                                   _P, _P]),
]

STAGE_NAMES = ("layer0_fwd", "gemm_H1", "layer1_fwd", "gemm_A1", "node_tail", "gemm_Phi1_adj", "layer1_rev",
               "gemm_M0_adj", "layer0_rev")

_lib = None


def load(path=None):
    """Load (once) and return the ctypes library handle."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            f"libsmx_gb300.so not found at {path}: build it first "
            "(python -c 'import __graft_entry__ as g; g.build()' or python symmetrix_gb300/build.py)")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def raise_for(code, lib=None):
    if code == SMX_OK:
        return
    lib = lib or load()
    msg = lib.smx_last_error().decode(errors="replace")
    raise ERRORS.get(code, RuntimeError)(msg)
