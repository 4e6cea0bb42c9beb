"""Run-to-run reproducibility of the GPU engine.

The layer-1 adjoint scatters every edge's contribution into H1_adj of the neighbour
node; the engine adds those terms as 64-bit fixed-point integers (order-independent),
and every other stage computes each atom's and edge's results in a fixed order.  So the
energies and the per-edge forces are the same bit pattern on every evaluation of the
same inputs, whichever order the blocks run in: repeated calls, a fresh engine, the
persistent atom schedule and the species-sorted centre order all agree bitwise.  The
reference's Kokkos evaluator scatters with float atomics (mace_kokkos.cpp:1008) and
has no such property.
"""
import numpy as np
import pytest

from helpers import edge_args
from oracle.pyoracle import Evaluator
from symmetrix_gb300.synth.model import CONFIGS, make_model, write_model
from symmetrix_gb300.synth.structures import neighbor_list, random_box

pytestmark = pytest.mark.gpu


def _engine(path, **kw):
    from symmetrix_gb300 import MACE
    return MACE(path, **kw)


def _same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


@pytest.mark.parametrize("L_max,precision", [(1, "float32"), (1, "bfloat16"), (2, "float32")])
def test_forces_bitwise_reproducible(engine_lib, tmp_path, L_max, precision):
    cfg = dict(CONFIGS["fp32_4096"], num_knots=50) if L_max == 1 else dict(
        num_channels=64, species=("H", "C", "O"), r_cut=5.0, L_max=2, num_knots=50)
    path = write_model(make_model(**cfg, seed=21), str(tmp_path / "m.json"))
    pos, L, species = random_box(400, 0.10, 0.9, len(cfg["species"]), seed=22)
    nl = neighbor_list(pos, cfg["r_cut"], L)
    args = edge_args(species, nl)
    m = _engine(path, precision=precision)
    m.set_option("persistent", 0)
    m.set_option("species_order", 0)
    m.compute_node_energies_forces(*args)
    e0, f0 = m.node_energies.copy(), m.node_forces.copy()
    for rep in range(3):
        m.compute_node_energies_forces(*args)
        assert _same(m.node_energies, e0), rep
        assert _same(m.node_forces, f0), rep
    # other block orders: persistent grids claiming atoms from a counter, species-sorted centres
    m.set_option("persistent", 1)
    m.compute_node_energies_forces(*args)
    assert _same(m.node_energies, e0) and _same(m.node_forces, f0)
    m.set_option("species_order", 1)
    m.compute_node_energies_forces(*args)
    assert _same(m.node_energies, e0) and _same(m.node_forces, f0)
    # a fresh engine
    m2 = _engine(path, precision=precision)
    m2.set_option("persistent", 0)
    m2.compute_node_energies_forces(*args)
    assert _same(m2.node_energies, e0) and _same(m2.node_forces, f0)
    # plain launches instead of programmatic dependent launches (a process-wide option)
    assert m2.get_option("pdl") == 1
    m2.set_option("pdl", 0)
    try:
        m2.compute_node_energies_forces(*args)
        assert _same(m2.node_energies, e0) and _same(m2.node_forces, f0)
    finally:
        m2.set_option("pdl", 1)
    # and the result is the right one
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*args)
    tol = 1e-5 if precision == "float32" else 1e-2
    assert np.abs(f0 - ref.node_forces).max() < tol
