"""The allocation-free energy/virial entry point (smx_energy_virial_device_noalloc).

It exists for callers that cannot allocate device memory where they need the sum,
e.g. a Kokkos pair style whose device memory belongs to Kokkos's pools.  Its scratch
is a fixed array inside the library, so these tests check, through the C ABI, that two
calls in a row each reproduce the energy and virial of the allocating atom-level entry
point (smx_compute_atoms) and each other, that they agree to float64 rounding with a
float64 host sum of the very same device arrays (one box within one 4096-element chunk,
one spanning several, and the empty call), and that oversized inputs are refused
before anything is launched.  This file is collected last, so that a run stopping at
its first failure has already run every other test.
"""
import ctypes
import math

import numpy as np
import pytest

from helpers import edge_args
from symmetrix_gb300.synth.structures import neighbor_list, random_box

pytestmark = pytest.mark.gpu


def _noalloc(lib, n, E, e_d, xyz_d, f_d, out, stream):
    from symmetrix_gb300 import _lib
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    code = lib.smx_energy_virial_device_noalloc(n, E, ptr(e_d), ptr(xyz_d), ptr(f_d), ptr(out), ctypes.c_void_p(stream))
    _lib.raise_for(code, lib)


def _host_sums(e, xyz, f):
    """float64 sums of the same arrays, exactly rounded (math.fsum)."""
    x, fe = np.asarray(xyz).reshape(-1, 3), np.asarray(f).reshape(-1, 3)
    out = [math.fsum(e)]
    for a in range(3):
        for c in range(3):
            out.append(math.fsum(x[:, a] * fe[:, c]))
    return np.array(out)


@pytest.mark.parametrize("n", [400, 5000])
def test_noalloc_energy_virial_matches_compute_atoms(engine_lib, small_model_path, n):
    torch = pytest.importorskip("torch")
    from symmetrix_gb300 import MACE, _lib
    lib = _lib.load()
    pos, L, sp = random_box(n, 0.064, 0.9, 3, seed=31)
    m = MACE(small_model_path)
    E_ref, _, _, W_ref = m.compute_atoms(pos, sp, box=L)  # allocating entry point
    nl = neighbor_list(pos, m.r_cut, L)
    m.compute_node_energies_forces(*edge_args(sp, nl))
    E_edges = len(nl["r"])
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), dtype=torch.float64, device="cuda")
    e_d, xyz_d, f_d = dev(m.node_energies), dev(nl["xyz"]), dev(m.node_forces)
    out = torch.empty(10, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    host = _host_sums(m.node_energies, nl["xyz"], m.node_forces)
    results = []
    for _ in range(2):
        out.fill_(float("nan"))
        _noalloc(lib, n, E_edges, e_d, xyz_d, f_d, out, stream)
        torch.cuda.synchronize()
        res = out.cpu().numpy()
        assert abs(res[0] - E_ref) < 1e-6 * n
        np.testing.assert_allclose(res[1:].reshape(3, 3), W_ref, atol=1e-4 * max(1.0, np.abs(W_ref).max()))
        # the same device arrays summed on the host in float64
        scale = np.array([np.abs(m.node_energies).sum()] + [np.abs(nl["xyz"].reshape(-1, 3)[:, a] *
                         m.node_forces.reshape(-1, 3)[:, c]).sum() for a in range(3) for c in range(3)])
        assert np.all(np.abs(res - host) <= 1e-12 * np.maximum(scale, 1e-300)), (res - host) / scale
        results.append(res)
    assert np.array_equal(results[0], results[1])


def test_noalloc_empty_input_writes_zeros(engine_lib):
    torch = pytest.importorskip("torch")
    from symmetrix_gb300 import _lib
    lib = _lib.load()
    out = torch.full((10,), float("nan"), dtype=torch.float64, device="cuda")
    _noalloc(lib, 0, 0, None, None, None, out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), np.zeros(10))


def test_noalloc_refuses_oversized_input(engine_lib):
    from symmetrix_gb300 import _lib
    lib = _lib.load()
    too_many = 16384 * 4096 + 1
    code = lib.smx_energy_virial_device_noalloc(1, too_many, None, None, None, None, None)
    assert code == 4  # SMX_ERR_CAPACITY, refused before any launch
    assert b"at most" in lib.smx_last_error()
