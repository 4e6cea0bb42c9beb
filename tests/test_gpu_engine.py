"""GPU engine parity: the FP32 CUDA path through the C ABI against the float64 oracle.

Tolerances (FP32 plain form vs the FP64 oracle): per-atom energies 2e-5 eV,
per-edge and per-atom forces 1e-5 eV/A on the seeded workloads below; stage
buffers to 1e-4 relative of their scale.
"""
import numpy as np
import pytest

from helpers import atomic_forces, edge_args
from oracle.pyoracle import Evaluator
from symmetrix_gb300.synth.model import CONFIGS, make_model, write_model
from symmetrix_gb300.synth.structures import neighbor_list, random_box

pytestmark = pytest.mark.gpu

E_TOL = 2e-5
F_TOL = 1e-5


def _report(tag, a, b):
    d = np.abs(np.asarray(a) - np.asarray(b))
    print(f"{tag}: max|d|={d.max() if d.size else 0:.3e} rms={np.sqrt((d ** 2).mean()) if d.size else 0:.3e}")
    return d.max() if d.size else 0.0


def _engine(path, **kw):
    from symmetrix_gb300 import MACE
    return MACE(path, **kw)


def test_small_workload_matches_reference_golden(engine_lib, small_model_path, small_golden):
    g = small_golden
    species = g["species"].astype(np.int32)
    nl = {k: g[k] for k in ("num_neigh", "neigh_indices", "xyz", "r")}
    m = _engine(small_model_path)
    assert not m.has_zbl
    m.compute_node_energies_forces(*edge_args(species, nl))
    assert _report("E_i", m.node_energies, g["node_energies"]) < E_TOL
    assert _report("f_edge", m.node_forces, g["node_forces"]) < F_TOL
    Fg = atomic_forces(64, g["edge_i"], g["neigh_indices"], g["node_forces"])
    F = atomic_forces(64, g["edge_i"], g["neigh_indices"], m.node_forces)
    assert _report("F_atom", F, Fg) < F_TOL


def test_stages_match_oracle(engine_lib, small_model_path, small_golden):
    g = small_golden
    species = g["species"].astype(np.int32)
    nl = {k: g[k] for k in ("num_neigh", "neigh_indices", "xyz", "r")}
    m = _engine(small_model_path, keep_stages=True)
    m.compute_node_energies_forces(*edge_args(species, nl))
    ref = Evaluator(small_model_path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    for s in ("A0", "M0", "H1", "Phi1", "A1", "M1", "H2", "H2_adj", "M1_adj", "A1_adj", "Phi1_adj", "H1_adj",
              "M0_adj", "A0_adj"):
        a, b = m.stage(s), ref.get(s)
        assert a.shape == b.shape, s
        scale = max(np.abs(b).max(), 1e-30)
        assert _report(s, a, b) <= 1e-4 * scale, s


def test_isolated_and_ragged_nodes(engine_lib, small_model_path):
    pos = np.array([[0, 0, 0], [1.2, 0.1, 0], [0.3, 1.4, 0.2], [20.0, 20, 20], [-1.0, -0.8, 0.9]], dtype=float)
    species = np.array([0, 1, 2, 1, 0], dtype=np.int32)
    nl = neighbor_list(pos, 5.0)
    m = _engine(small_model_path)
    m.compute_node_energies_forces(*edge_args(species, nl))
    ref = Evaluator(small_model_path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    assert _report("E_i", m.node_energies, ref.node_energies) < E_TOL
    assert _report("f_edge", m.node_forces, ref.node_forces) < F_TOL


def test_empty_and_single_atom(engine_lib, small_model_path):
    m = _engine(small_model_path)
    m.compute_node_energies_forces(0, [], [], [], [], np.zeros((0, 3)), np.zeros(0))
    assert m.node_energies.shape == (0,) and m.node_forces.shape == (0,)
    m.compute_node_energies_forces(1, [2], [0], [], [], np.zeros((0, 3)), np.zeros(0))
    ref = Evaluator(small_model_path, "port")
    ref.compute_node_energies_forces(1, [2], [0], [], [], np.zeros((0, 3)), np.zeros(0))
    assert abs(m.node_energies[0] - ref.node_energies[0]) < E_TOL


def test_invalid_inputs_are_rejected(engine_lib, small_model_path):
    m = _engine(small_model_path)
    xyz = np.array([[1.0, 0.5, 0.2], [-1.0, -0.5, -0.2]])
    r = np.linalg.norm(xyz, axis=1)
    with pytest.raises(ValueError):  # neighbour index out of range
        m.compute_node_energies_forces(2, [0, 1], [1, 1], [1, 2], [1, 0], xyz, r)
    with pytest.raises(ValueError):  # species out of range
        m.compute_node_energies_forces(2, [0, 7], [1, 1], [1, 0], [7, 0], xyz, r)
    with pytest.raises(ValueError):  # r >= r_cut
        m.compute_node_energies_forces(2, [0, 1], [1, 1], [1, 0], [1, 0], xyz * 10, r * 10)
    with pytest.raises(ValueError):  # sum(num_neigh) != edges
        m.compute_node_energies_forces(2, [0, 1], [2, 1], [1, 0], [1, 0], xyz, r)
    with pytest.raises(RuntimeError):
        _engine("/nonexistent/model.json")


@pytest.fixture(scope="module")
def wide_model(tmp_path_factory):
    """128x0e+128x1o, H/C/N/O (the 4096-atom workload's shape), 50 knots to keep the file small."""
    cfg = dict(CONFIGS["fp32_4096"], num_knots=50)
    return write_model(make_model(**cfg, seed=7), str(tmp_path_factory.mktemp("wide") / "wide.json"))


def test_wide_model_periodic_box(engine_lib, wide_model):
    pos, L, species = random_box(160, 0.10, 0.9, 4, seed=9)
    nl = neighbor_list(pos, 5.0, L)
    m = _engine(wide_model)
    m.compute_node_energies_forces(*edge_args(species, nl))
    ref = Evaluator(wide_model, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    assert _report("E_i", m.node_energies, ref.node_energies) < E_TOL
    assert _report("f_edge", m.node_forces, ref.node_forces) < F_TOL
    F = atomic_forces(160, nl["i"], nl["neigh_indices"], m.node_forces)
    Fr = atomic_forces(160, nl["i"], nl["neigh_indices"], ref.node_forces)
    assert _report("F_atom", F, Fr) < F_TOL


def test_device_api_matches_host_api(engine_lib, small_model_path, small_golden):
    torch = pytest.importorskip("torch")
    g = small_golden
    species = g["species"].astype(np.int32)
    m = _engine(small_model_path)
    m.compute_node_energies_forces(64, species, g["num_neigh"], g["neigh_indices"],
                                   species[g["neigh_indices"]], g["xyz"], g["r"])
    dev = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
    t = [dev(species, torch.int32), dev(g["num_neigh"], torch.int32), dev(g["neigh_indices"], torch.int32),
         dev(species[g["neigh_indices"]], torch.int32), dev(g["xyz"].reshape(-1), torch.float64),
         dev(g["r"], torch.float64)]
    E = len(g["r"])
    e_out = torch.zeros(64, dtype=torch.float64, device="cuda")
    f_out = torch.zeros(3 * E, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    m.compute_device(64, *[x.data_ptr() for x in t[:4]], E, t[4].data_ptr(), t[5].data_ptr(), e_out.data_ptr(),
                     f_out.data_ptr(), stream)
    m.sync(stream)  # waits for the caller's stream; no bounded device wait gave up
    # H1_adj is accumulated with float atomics, so two runs agree to float32 rounding only
    np.testing.assert_allclose(e_out.cpu().numpy(), m.node_energies, rtol=0, atol=1e-6)
    np.testing.assert_allclose(f_out.cpu().numpy(), m.node_forces, rtol=0, atol=2e-6)


def test_zbl_model_matches_oracle(engine_lib, tmp_path):
    """ZBL pair repulsion (zbl.cpp:22-125) on close pairs, against the oracle."""
    path = write_model(make_model(num_channels=32, species=("H", "C", "O"), num_knots=60, seed=4, zbl=True),
                       str(tmp_path / "zbl.json"))
    pos, L, species = random_box(120, 0.10, 0.9, 3, seed=12)
    nl = neighbor_list(pos, 5.0, L)
    assert (nl["r"] < 1.3).sum() > 0  # C/O pairs inside the ZBL range (r_max = 1.32-1.52 A)
    m = _engine(path)
    assert m.has_zbl
    m.compute_node_energies_forces(*edge_args(species, nl))
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    assert _report("E_i", m.node_energies, ref.node_energies) < E_TOL
    assert _report("f_edge", m.node_forces, ref.node_forces) < F_TOL


def _edited_model(src, dst, edit):
    import json
    with open(src) as f:
        m = json.load(f)
    edit(m)
    with open(dst, "w") as f:
        json.dump(m, f)
    return dst


@pytest.mark.parametrize("variant", ["shuffled", "extra_monomial"])
def test_polynomial_paths(engine_lib, small_model_path, small_golden, tmp_path, variant):
    """Monomial lists in another order (generated canonical kernels through the loader's
    mapping) and with a monomial outside the canonical sets (data-driven kernels)."""
    rng = np.random.default_rng(3)

    def shuffle(m):
        for LM, monos in m["M0_monomials"].items():
            perm = rng.permutation(len(monos))
            m["M0_monomials"][LM] = [monos[p] for p in perm]
            for s in m["M0_weights"]:
                for k, c in m["M0_weights"][s][LM].items():
                    m["M0_weights"][s][LM][k] = [c[p] for p in perm]

    def extra(m):
        m["M0_monomials"]["0"].append([0, 1, 4])  # parity-odd: not an equivariant term
        for s in m["M0_weights"]:
            for k in m["M0_weights"][s]["0"]:
                m["M0_weights"][s]["0"][k].append(float(rng.normal() * 0.1))
        m["M1_monomials"].append([2, 3])
        for s in m["M1_weights"]:
            for k in m["M1_weights"][s]:
                m["M1_weights"][s][k].append(float(rng.normal() * 0.1))

    path = _edited_model(small_model_path, str(tmp_path / f"{variant}.json"), shuffle if variant == "shuffled" else extra)
    g = small_golden
    species = g["species"].astype(np.int32)
    nl = {k: g[k] for k in ("num_neigh", "neigh_indices", "xyz", "r")}
    m = _engine(path)
    m.compute_node_energies_forces(*edge_args(species, nl))
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    assert _report("E_i", m.node_energies, ref.node_energies) < E_TOL
    assert _report("f_edge", m.node_forces, ref.node_forces) < F_TOL


def test_model_cache_gives_identical_results(engine_lib, small_model_path, small_golden, tmp_path):
    from symmetrix_gb300 import save_model_cache
    g = small_golden
    species = g["species"].astype(np.int32)
    nl = {k: g[k] for k in ("num_neigh", "neigh_indices", "xyz", "r")}
    cache = str(tmp_path / "small.smxb")
    save_model_cache(small_model_path, cache)
    a, b = _engine(small_model_path), _engine(cache)
    a.compute_node_energies_forces(*edge_args(species, nl))
    b.compute_node_energies_forces(*edge_args(species, nl))
    assert b.atomic_numbers == a.atomic_numbers and b.r_cut == a.r_cut
    # the forward pass is deterministic: bitwise equal; the adjoint's H1_adj scatter uses
    # float atomics, so forces agree to float32 rounding of the summation order
    assert np.array_equal(a.node_energies, b.node_energies)
    assert np.abs(a.node_forces - b.node_forces).max() < 1e-6


@pytest.mark.parametrize("zbl", [False, True])
def test_density_scaled_model_matches_oracle(engine_lib, tmp_path, zbl):
    """Density-normalised interaction blocks (A0_scaled, A1_scaled; mace.cpp:273-346,
    :681-757): energies, edge forces and the scaled stage buffers against the oracle."""
    path = write_model(make_model(**CONFIGS["small"], seed=5, density_scaled=True, zbl=zbl),
                       str(tmp_path / "dens.json"))
    pos, L, species = random_box(64, 0.064, 0.9, 3, seed=4)
    nl = neighbor_list(pos, 5.0, L)
    m = _engine(path, keep_stages=True)
    m.compute_node_energies_forces(*edge_args(species, nl))
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    assert _report("E_i", m.node_energies, ref.node_energies) < E_TOL
    assert _report("f_edge", m.node_forces, ref.node_forces) < F_TOL
    for s in ("A0", "A1", "A0_adj", "A1_adj", "Phi1_adj"):
        a, b = m.stage(s), ref.get(s)
        assert _report(s, a, b) <= 1e-4 * max(np.abs(b).max(), 1e-30), s


@pytest.mark.parametrize("variant", ["plain", "density_zbl"])
def test_lmax2_model_matches_oracle(engine_lib, tmp_path, variant):
    """L_max = 2 hidden irreps (17 layer-1 instructions, 243 paths, nine LM outputs):
    energies, edge forces and stage buffers against the oracle."""
    extra = dict(density_scaled=True, zbl=True) if variant == "density_zbl" else {}
    path = write_model(make_model(num_channels=32, species=("H", "C", "O"), r_cut=5.0, L_max=2, num_knots=60,
                                  seed=3, **extra), str(tmp_path / "l2.json"))
    pos, L, species = random_box(64, 0.064, 0.9, 3, seed=4)
    nl = neighbor_list(pos, 5.0, L)
    m = _engine(path, keep_stages=True)
    assert m.L_max == 2 and m.num_LM == 9
    assert m.get_option("poly_canon") == 1  # generated polynomial kernels for LM = 0..8
    m.compute_node_energies_forces(*edge_args(species, nl))
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    assert _report("E_i", m.node_energies, ref.node_energies) < E_TOL
    assert _report("f_edge", m.node_forces, ref.node_forces) < F_TOL
    for s in ("M0", "H1", "Phi1", "A1", "H1_adj", "Phi1_adj", "M0_adj", "A0_adj"):
        a, b = m.stage(s), ref.get(s)
        assert a.shape == b.shape, s
        assert _report(s, a, b) <= 1e-4 * max(np.abs(b).max(), 1e-30), s


def test_lmax2_wide_model(engine_lib, tmp_path):
    """L_max = 2 at 128 channels (the precision-form shape), both forms against the oracle."""
    path = write_model(make_model(num_channels=128, species=("H", "C", "N", "O"), r_cut=5.0, L_max=2,
                                  num_knots=40, seed=8), str(tmp_path / "l2w.json"))
    pos, L, species = random_box(96, 0.09, 0.9, 4, seed=6)
    nl = neighbor_list(pos, 5.0, L)
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    Fr = atomic_forces(96, nl["i"], nl["neigh_indices"], ref.node_forces)
    for precision, tol in (("float32", F_TOL), ("bfloat16", 1e-2)):
        m = _engine(path, precision=precision)
        m.compute_node_energies_forces(*edge_args(species, nl))
        assert m.get_option("l2_split") in (1, 2)  # tuned on the first evaluation
        F = atomic_forces(96, nl["i"], nl["neigh_indices"], m.node_forces)
        assert _report(f"{precision} E_i", m.node_energies, ref.node_energies) < (E_TOL if tol == F_TOL else 5e-3)
        assert _report(f"{precision} F_atom", F, Fr) < tol


@pytest.mark.parametrize("L_max", [1, 2])
def test_persistent_atom_schedule(engine_lib, tmp_path, L_max):
    """The per-atom kernels as persistent grids claiming atoms from a counter: the same
    energies as one block per atom (bitwise: the forward pass is deterministic), forces
    against the oracle, and the counter is reset between launches (repeat evaluations).
    The tuned schedule is a mask over the six per-atom kernels."""
    # 64 channels at L_max = 2: the layer-1 kernels run two channel slices per node
    path = write_model(make_model(num_channels=32 * L_max, species=("H", "C", "O"), r_cut=5.0, L_max=L_max,
                                  num_knots=60, seed=5), str(tmp_path / "m.json"))
    pos, L, species = random_box(300, 0.08, 0.9, 3, seed=12)
    nl = neighbor_list(pos, 5.0, L)
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    m = _engine(path)
    m.set_option("persistent", 0)
    m.compute_node_energies_forces(*edge_args(species, nl))
    e_block = m.node_energies.copy()
    assert m.get_option("persistent") == 0
    m.set_option("persistent", 1)
    assert m.get_option("persistent") == 63
    for rep in range(3):
        m.compute_node_energies_forces(*edge_args(species, nl))
        assert np.array_equal(m.node_energies, e_block), rep
        assert _report("f_edge", m.node_forces, ref.node_forces) < F_TOL
    m.set_option("persistent", -1)  # tuned on the next evaluation
    m.compute_node_energies_forces(*edge_args(species, nl))
    assert 0 <= m.get_option("persistent") <= 63
    assert np.array_equal(m.node_energies, e_block)
    assert _report("f_edge", m.node_forces, ref.node_forces) < F_TOL
    # fewer atoms than the persistent grid has blocks
    sub = neighbor_list(pos[:7], 5.0)
    m.set_option("persistent", 1)
    m.compute_node_energies_forces(*edge_args(species[:7], sub))
    ref.compute_node_energies_forces(*edge_args(species[:7], sub))
    assert _report("E_i small", m.node_energies, ref.node_energies) < E_TOL
    assert _report("f_edge small", m.node_forces, ref.node_forces) < F_TOL


def test_species_sorted_atom_order(engine_lib, tmp_path):
    """Centre atoms taken in species order (the layout for tables larger than L2): the
    same energies as the input order, bitwise, and forces against the oracle."""
    path = write_model(make_model(num_channels=32, species=("H", "C", "N", "O"), r_cut=5.0, L_max=1, num_knots=60,
                                  seed=6, zbl=True), str(tmp_path / "m.json"))
    pos, L, species = random_box(250, 0.09, 0.9, 4, seed=13)
    nl = neighbor_list(pos, 5.0, L)
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    m = _engine(path)
    m.set_option("species_order", 0)
    assert m.get_option("species_order") == 0  # a small table: input order by default too
    m.compute_node_energies_forces(*edge_args(species, nl))
    e0 = m.node_energies.copy()
    m.set_option("species_order", 1)
    assert m.get_option("species_order") == 1
    for persistent in (0, 1):
        m.set_option("persistent", persistent)
        m.compute_node_energies_forces(*edge_args(species, nl))
        assert np.array_equal(m.node_energies, e0), persistent
        assert _report("f_edge", m.node_forces, ref.node_forces) < F_TOL


def test_lmax2_data_driven_polynomials(engine_lib, tmp_path):
    """An L_max = 2 model with a monomial outside the canonical sets runs the data-driven
    polynomial kernels; energies and forces against the oracle."""
    import json
    path = write_model(make_model(num_channels=32, species=("H", "C", "O"), r_cut=5.0, L_max=2, num_knots=60,
                                  seed=9), str(tmp_path / "l2.json"))
    with open(path) as f:
        model = json.load(f)
    rng = np.random.default_rng(4)
    model["M0_monomials"]["5"].append([0, 1, 4])
    for s in model["M0_weights"]:
        for k in model["M0_weights"][s]["5"]:
            model["M0_weights"][s]["5"][k].append(float(rng.normal() * 0.1))
    with open(path, "w") as f:
        json.dump(model, f)
    pos, L, species = random_box(64, 0.064, 0.9, 3, seed=5)
    nl = neighbor_list(pos, 5.0, L)
    m = _engine(path)
    assert m.get_option("poly_canon") == 0
    m.compute_node_energies_forces(*edge_args(species, nl))
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    assert _report("E_i", m.node_energies, ref.node_energies) < E_TOL
    assert _report("f_edge", m.node_forces, ref.node_forces) < F_TOL


@pytest.mark.parametrize("L_max", [1, 2])
def test_rotation_invariance_on_gpu(engine_lib, tmp_path, L_max):
    """The CUDA path: energies invariant and atomic forces covariant under O(3) (float32
    tolerances), for both hidden-irrep sizes."""
    from helpers import random_rotation
    path = write_model(make_model(num_channels=32, species=("H", "C", "O"), r_cut=5.0, L_max=L_max, num_knots=60,
                                  seed=11), str(tmp_path / "m.json"))
    rng = np.random.default_rng(8)
    pos = rng.normal(size=(40, 3)) * 2.2
    species = rng.integers(0, 3, size=40).astype(np.int32)
    m = _engine(path)
    out = []
    for Q in (np.eye(3), random_rotation(rng), -random_rotation(rng)):
        nl = neighbor_list(pos @ Q.T, 5.0)
        m.compute_node_energies_forces(*edge_args(species, nl))
        F = atomic_forces(40, nl["i"], nl["neigh_indices"], m.node_forces)
        out.append((m.node_energies.copy(), F @ Q))
    scale_e = max(1.0, np.abs(out[0][0]).max())
    scale_f = max(1.0, np.abs(out[0][1]).max())
    for e, F in out[1:]:
        assert _report("E_i rotated", e, out[0][0]) < 1e-5 * scale_e
        assert _report("F rotated", F, out[0][1]) < 1e-5 * scale_f


@pytest.mark.parametrize("L_max", [1, 2])
def test_cg_table_forms_agree(engine_lib, tmp_path, L_max):
    """The layer-1 Clebsch-Gordan contractions through the padded tables (default) and
    through the compressed rows: the same energies and forces to float32 rounding."""
    path = write_model(make_model(num_channels=32 * L_max, species=("H", "C", "O"), r_cut=5.0, L_max=L_max,
                                  num_knots=60, seed=12), str(tmp_path / "m.json"))
    pos, L, species = random_box(120, 0.08, 0.9, 3, seed=14)
    nl = neighbor_list(pos, 5.0, L)
    m = _engine(path)
    assert m.get_option("cg_padded") == 1
    m.compute_node_energies_forces(*edge_args(species, nl))
    e_pad, f_pad = m.node_energies.copy(), m.node_forces.copy()
    m.set_option("cg_padded", 0)
    assert m.get_option("cg_padded") == 0
    m.compute_node_energies_forces(*edge_args(species, nl))
    assert _report("E_i", m.node_energies, e_pad) < 1e-5 * max(1.0, np.abs(e_pad).max())
    assert _report("f_edge", m.node_forces, f_pad) < 1e-5 * max(1.0, np.abs(f_pad).max())


@pytest.mark.parametrize("C,L_max", [(96, 1), (256, 1), (96, 2), (160, 1)])
def test_channel_widths(engine_lib, tmp_path, C, L_max):
    """Channel counts off the compile-time specialisations (96, 160: the generic kernels;
    96 at L_max = 2: a partly filled second channel slice) and the widest (256), both
    forms, against the oracle."""
    path = write_model(make_model(num_channels=C, species=("H", "C", "O"), r_cut=5.0, L_max=L_max, num_knots=40,
                                  seed=13), str(tmp_path / "m.json"))
    pos, L, species = random_box(48, 0.07, 0.9, 3, seed=15)
    nl = neighbor_list(pos, 5.0, L)
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    Fr = atomic_forces(48, nl["i"], nl["neigh_indices"], ref.node_forces)
    scale = max(1.0, np.abs(Fr).max())
    for precision, tol in (("float32", F_TOL), ("bfloat16", 1e-3 * scale)):
        m = _engine(path, precision=precision)
        m.compute_node_energies_forces(*edge_args(species, nl))
        F = atomic_forces(48, nl["i"], nl["neigh_indices"], m.node_forces)
        assert _report(f"C={C} {precision} E_i", m.node_energies, ref.node_energies) < (
            E_TOL if precision == "float32" else 1e-3 * max(1.0, np.abs(ref.node_energies).max()))
        assert _report(f"C={C} {precision} F", F, Fr) < max(tol, F_TOL)


@pytest.mark.parametrize("precision", ["float32", "bfloat16"])
def test_twenty_species_model(engine_lib, tmp_path, precision):
    """20 species, as the reference's high-entropy-alloy case
    (pair_symmetrix/test/test_pair_symmetrix_mace.py:300-393): 210 unordered and 400 ordered
    pair tables; every species present; against the oracle in both forms, and the same
    results with the centre atoms taken in input or species-sorted order."""
    Z = list(range(21, 31)) + list(range(39, 49))
    path = write_model(make_model(num_channels=32, species=Z, num_knots=20, seed=20), str(tmp_path / "hea.json"))
    pos, L, species = random_box(240, 0.08, 1.2, 20, seed=21)
    assert len(np.unique(species)) == 20
    nl = neighbor_list(pos, 5.0, L)
    ref = Evaluator(path, "port")
    ref.compute_node_energies_forces(*edge_args(species, nl))
    out = {}
    m = _engine(path, precision=precision)
    for order in (0, 1):
        m.set_option("species_order", order)
        m.compute_node_energies_forces(*edge_args(species, nl))
        out[order] = (m.node_energies.copy(), m.node_forces.copy())
    e_tol, f_tol = (E_TOL, F_TOL) if precision == "float32" else (0.005, 0.010)
    assert _report("E_i", out[1][0], ref.node_energies) < e_tol
    assert _report("f_edge", out[1][1], ref.node_forces) < f_tol
    F = atomic_forces(240, nl["i"], nl["neigh_indices"], out[1][1])
    Fr = atomic_forces(240, nl["i"], nl["neigh_indices"], ref.node_forces)
    assert _report("F_atom", F, Fr) < f_tol
    # the forward pass does not depend on the order; the adjoint's atomics to float32 rounding
    assert np.array_equal(out[0][0], out[1][0])
    assert _report("order", out[0][1], out[1][1]) < 1e-6
