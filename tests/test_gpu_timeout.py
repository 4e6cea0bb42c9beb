"""The timeout path of the bounded device waits, exercised without any fault.

With the test option "test_gemm_timeout" the next tensor-core GEMM launch issues no TMA
load, so its MMA thread's bounded wait (2 ms here) runs out with no copy or MMA in
flight: the kernel records the timeout in the engine's status word, frees its tensor
memory and returns.  The call reports SMX_ERR_TIMEOUT (TimeoutError in Python; code 5
from smx_sync after a device-pointer call), and the engine stays usable: the next
evaluation succeeds and matches the oracle.
"""
import ctypes

import numpy as np
import pytest

from helpers import edge_args
from oracle.pyoracle import Evaluator
from symmetrix_gb300.synth.model import make_model, write_model
from symmetrix_gb300.synth.structures import neighbor_list, random_box

pytestmark = pytest.mark.gpu


def test_gemm_wait_timeout_is_reported_and_recoverable(engine_lib, tmp_path):
    import torch

    from symmetrix_gb300 import MACE, _lib
    path = write_model(make_model(num_channels=64, species=("H", "C", "O"), r_cut=5.0, L_max=1, num_knots=40, seed=8),
                       str(tmp_path / "m.json"))
    pos, L, species = random_box(96, 0.08, 0.9, 3, seed=9)
    nl = neighbor_list(pos, 5.0, L)
    args = edge_args(species, nl)
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*args)
    m = MACE(path, precision="bfloat16")
    m.compute_node_energies_forces(*args)  # first evaluation (tunes the GEMM schedule)
    f_ok = m.node_forces.copy()
    # host-pointer call: one GEMM launch gives up
    m.set_option("test_gemm_timeout", 1)
    with pytest.raises(TimeoutError):
        m.compute_node_energies_forces(*args)
    # the engine recovers
    m.compute_node_energies_forces(*args)
    assert np.array_equal(m.node_forces, f_ok)
    assert np.abs(m.node_forces - ref.node_forces).max() < 1e-2
    # device-pointer call: the timeout is reported by smx_sync
    dev = torch.device("cuda", 0)
    n, E = len(species), len(nl["r"])
    t = [torch.as_tensor(np.ascontiguousarray(a), device=dev) for a in
         (species.astype(np.int32), nl["num_neigh"].astype(np.int32), nl["neigh_indices"].astype(np.int32),
          species[nl["neigh_indices"]].astype(np.int32), nl["xyz"].reshape(-1), nl["r"])]
    e_out = torch.zeros(n, dtype=torch.float64, device=dev)
    f_out = torch.zeros(3 * E, dtype=torch.float64, device=dev)
    lib = _lib.load()
    torch.cuda.synchronize()  # the engine's stream does not wait for torch's copies
    m.set_option("test_gemm_timeout", 1)
    m.compute_device(n, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(), E, t[4].data_ptr(),
                     t[5].data_ptr(), e_out.data_ptr(), f_out.data_ptr(), None)
    assert lib.smx_sync(m._h, None) == 5  # SMX_ERR_TIMEOUT
    assert lib.smx_sync(m._h, None) == 0  # the status word is cleared once read
    m.compute_device(n, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(), E, t[4].data_ptr(),
                     t[5].data_ptr(), e_out.data_ptr(), f_out.data_ptr(), None)
    assert lib.smx_sync(m._h, None) == 0
    assert np.array_equal(f_out.cpu().numpy(), f_ok)
    with pytest.raises(ValueError):
        MACE(path, precision="float32").set_option("test_gemm_timeout", 1)
