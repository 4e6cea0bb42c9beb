"""GB300-native MACE energy/force engine, a drop-in for libsymmetrix's evaluator path.

`MACE` mirrors the reference's `symmetrix.MACE` binding (with the names its
calculator also looks for: `MACEKokkos`, `MACEKokkosFloat`, `_init_kokkos`,
`_kokkos_is_initialized`) over the C ABI declared in
include/smx_gb300.h; the kernels are hand-written CUDA for sm_103a
(symmetrix_gb300/csrc).  `symmetrix_gb300.synth` generates seeded synthetic models
in the reference's JSON format and synthetic structures.
"""
from .mace import MACE, MACEKokkos, MACEKokkosFloat, _init_kokkos, _kokkos_is_initialized, save_model_cache  # noqa: F401

__version__ = "0.1.0"
