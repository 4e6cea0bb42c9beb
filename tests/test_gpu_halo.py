"""The halo evaluation on the GPU (smx_compute_halo: the stage calls of the pair style's
no-MPI-message-passing mode, pair_symmetrix/pair_symmetrix_mace.cpp:672-698) against the
float64 oracle's, which the reference's own stages pin (tests/test_oracle.py).

Layer 0 runs over all nodes, ZBL, layer 1 and the readouts over the first
num_local_nodes.  Tolerances are the plain evaluation's: FP32 form 2e-5 eV per atom and
1e-5 eV/A per edge force; BF16 form 5 meV per atom and 10 meV/A.
"""
import numpy as np
import pytest

from helpers import edge_args
from oracle.pyoracle import Evaluator
from symmetrix_gb300.synth.model import make_model, write_model
from symmetrix_gb300.synth.structures import neighbor_list, random_box

pytestmark = pytest.mark.gpu

TOL = {"float32": (2e-5, 1e-5), "bfloat16": (5e-3, 1e-2)}


def _max(a, b):
    d = np.abs(np.asarray(a) - np.asarray(b))
    return d.max() if d.size else 0.0


@pytest.fixture(scope="module")
def periodic_halo(tmp_path_factory):
    from make_golden import HALO_ATOMS, halo_case, halo_model
    path = halo_model(str(tmp_path_factory.mktemp("halo") / "halo.json"))
    return path, halo_case(), HALO_ATOMS


@pytest.mark.parametrize("precision", ["float32", "bfloat16"])
def test_periodic_halo_matches_oracle(engine_lib, periodic_halo, precision):
    """A 24-atom box as one LAMMPS rank holds it (the halo fixture's case: density-scaled
    ZBL model, ZBL-range pairs on local and halo edges)."""
    from symmetrix_gb300 import MACE
    path, c, n = periodic_halo
    N0 = len(c["node_atom"])
    args = (c["node_types"], c["num_neigh"], c["neigh_indices"], c["neigh_types"], c["xyz"], c["r"])
    ref = Evaluator(path, "port")
    ref.compute_halo(n, N0, *args)
    m = MACE(path, precision=precision, keep_stages=True)
    m.compute_halo(n, N0, *args)
    e_tol, f_tol = TOL[precision]
    assert m.node_energies.shape == (n,)
    de, df = _max(m.node_energies, ref.node_energies), _max(m.node_forces, ref.node_forces)
    E1 = int(c["num_neigh"][:n].sum())
    dfh = _max(m.node_forces[3 * E1:], ref.node_forces[3 * E1:])
    print(f"{precision}: N0={N0} E={len(c['r'])} dE_i={de:.2e} df_edge={df:.2e} df_halo_edges={dfh:.2e}")
    assert de < e_tol and df < f_tol
    # stage buffers have the reference's sizes: layer-0 stages per node, layer-1 per local node
    for s in ("A0", "M0", "H1", "A0_adj", "M0_adj", "H1_adj", "Phi1", "A1", "H2", "Phi1_adj", "A1_adj", "H2_adj"):
        a, b = m.stage(s), ref.get(s)
        assert a.shape == b.shape, s
        if precision == "float32":
            assert _max(a, b) <= 1e-4 * max(np.abs(b).max(), 1e-30), s


@pytest.mark.parametrize("precision", ["float32", "bfloat16"])
def test_any_trailing_halo_matches_oracle(engine_lib, small_model_path, precision):
    """Layer 1 over the first n1 of 64 nodes of a periodic box (the trailing nodes are no
    images, so the results differ from the full evaluation); n1 = 64 is the plain
    evaluation bit for bit."""
    from symmetrix_gb300 import MACE
    pos, L, species = random_box(64, 0.064, 0.9, 3, seed=4)
    nl = neighbor_list(pos, 5.0, L)
    args = edge_args(species, nl)[1:]
    m = MACE(small_model_path, precision=precision)
    ref = Evaluator(small_model_path, "port")
    e_tol, f_tol = TOL[precision]
    for n1 in (7, 40, 64):
        ref.compute_halo(n1, 64, *args)
        m.compute_halo(n1, 64, *args)
        de, df = _max(m.node_energies, ref.node_energies), _max(m.node_forces, ref.node_forces)
        print(f"{precision} n1={n1}: dE_i={de:.2e} df_edge={df:.2e}")
        assert m.node_energies.shape == (n1,)
        assert de < e_tol and df < f_tol
    e_h, f_h = m.node_energies.copy(), m.node_forces.copy()
    m.compute_node_energies_forces(64, *args)
    assert np.array_equal(m.node_energies, e_h) and np.array_equal(m.node_forces, f_h)


@pytest.mark.parametrize("precision", ["float32", "bfloat16"])
def test_lmax2_halo_and_schedules_match_oracle(engine_lib, tmp_path, precision):
    """L_max = 2 (17 instructions, four instruction groups; 64 channels, so the layer-1
    kernels may run two channel slices per node, both tried while tuning) with density
    scaling and ZBL, in both atom schedules (one block per atom, persistent grids)."""
    from symmetrix_gb300 import MACE
    path = write_model(make_model(num_channels=64, species=("H", "C", "O"), r_cut=5.0, L_max=2, num_knots=60,
                                  seed=3, density_scaled=True, zbl=True), str(tmp_path / "l2.json"))
    pos, L, species = random_box(64, 0.064, 0.9, 3, seed=4)
    nl = neighbor_list(pos, 5.0, L)
    args = edge_args(species, nl)[1:]
    ref = Evaluator(path, "port")
    ref.compute_halo(40, 64, *args)
    m = MACE(path, precision=precision)
    e_tol, f_tol = TOL[precision]
    for persistent in (-1, 0, 1):
        m.set_option("persistent", persistent)
        m.compute_halo(40, 64, *args)
        de, df = _max(m.node_energies, ref.node_energies), _max(m.node_forces, ref.node_forces)
        print(f"{precision} persistent={persistent} l2_split={m.get_option('l2_split')}: dE_i={de:.2e} "
              f"df_edge={df:.2e}")
        assert de < e_tol and df < f_tol


def test_halo_with_species_order(engine_lib, small_model_path):
    """Centre atoms sorted by species (as for spline tables larger than L2): layer 0 visits
    all nodes in one species order, layer 1 the local nodes in an order of their own."""
    from symmetrix_gb300 import MACE
    pos, L, species = random_box(64, 0.064, 0.9, 3, seed=4)
    nl = neighbor_list(pos, 5.0, L)
    args = edge_args(species, nl)[1:]
    m = MACE(small_model_path)
    m.set_option("species_order", 1)
    assert m.get_option("species_order") == 1
    ref = Evaluator(small_model_path, "port")
    for n1 in (7, 40, 64):
        ref.compute_halo(n1, 64, *args)
        m.compute_halo(n1, 64, *args)
        de, df = _max(m.node_energies, ref.node_energies), _max(m.node_forces, ref.node_forces)
        print(f"species order n1={n1}: dE_i={de:.2e} df_edge={df:.2e}")
        assert de < TOL["float32"][0] and df < TOL["float32"][1]


def test_halo_rejects_bad_counts(engine_lib, small_model_path):
    from symmetrix_gb300 import MACE
    pos, L, species = random_box(16, 0.064, 0.9, 3, seed=4)
    nl = neighbor_list(pos, 5.0, L)
    args = edge_args(species, nl)[1:]
    m = MACE(small_model_path)
    with pytest.raises(ValueError):
        m.compute_halo(17, 16, *args)
    with pytest.raises(ValueError):
        m.compute_halo(-1, 16, *args)
    m.compute_halo(0, 16, *args)  # no layer-1 node: no energy and no force
    assert m.node_energies.shape == (0,) and np.abs(m.node_forces).max() == 0.0
