"""The oracle (float64 restatement of libsymmetrix's evaluator) pinned against the reference.

Pins, in order of strength:
  * golden outputs of the reference's own evaluator (tests/golden, made by
    tests/golden/make_golden.py from oracle/_ref);
  * the reference build itself, stage by stage, when the reference tree is present;
  * the reference's model-free known-answer tests (symmetrix/test/test_zbl.py,
    test_cubic_spline.py, test_multivariate_polynomial.py, test_multilayer_perceptron.py);
  * the reference's finite-difference adjoint check (symmetrix/test/test_mace.py:73-84,
    655-704) and O(3) invariance.
"""
import ctypes
import json
import os

import numpy as np
import pytest

from helpers import atomic_forces, edge_args, random_rotation
from oracle import build as oracle_build
from oracle.pyoracle import Evaluator, library
from symmetrix_gb300.synth.structures import neighbor_list, random_box

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
HAVE_REF = os.path.isdir(oracle_build.REF_SRC)
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference tree absent (oracle/_ref not buildable here)")


def _tiny():
    with open(os.path.join(GOLD, "tiny_golden.json")) as f:
        g = json.load(f)
    nl = {k: np.asarray(g[k]) for k in ("num_neigh", "neigh_indices", "xyz", "r")}
    return g, np.asarray(g["species"], dtype=np.int32), nl


def test_tiny_golden_matches_reference_outputs():
    g, species, nl = _tiny()
    ev = Evaluator(os.path.join(GOLD, "tiny_model.json"), "port")
    ev.compute_node_energies_forces(*edge_args(species, nl))
    np.testing.assert_allclose(ev.node_energies, g["node_energies"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(ev.node_forces, g["node_forces"], rtol=1e-10, atol=1e-12)
    for s in ("A0", "M0", "H1", "Phi1", "A1", "M1", "H2", "H1_adj", "M0_adj", "A0_adj", "Phi1_adj"):
        assert ev.get(s).sum() == pytest.approx(g["sum_" + s], rel=1e-10, abs=1e-12), s


def test_regenerated_model_matches_golden_fingerprint(small_model_path, small_golden):
    """The seeded generator must rebuild the exact model the goldens were made with."""
    from make_golden import model_fingerprint
    np.testing.assert_allclose(model_fingerprint(small_model_path), small_golden["model_fingerprint"], rtol=1e-10)


def test_small_golden_matches_reference_outputs(small_model_path, small_golden):
    g = small_golden
    species = g["species"].astype(np.int32)
    nl = {k: g[k] for k in ("num_neigh", "neigh_indices", "xyz", "r")}
    ev = Evaluator(small_model_path, "port")
    ev.compute_node_energies_forces(*edge_args(species, nl))
    np.testing.assert_allclose(ev.node_energies, g["node_energies"], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(ev.node_forces, g["node_forces"], rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("threads,lean", [(2, False), (5, False), (3, True)])
def test_threaded_evaluation_is_bitwise_serial(small_model_path, small_golden, threads, lean):
    """One evaluation split over node ranges (the H1_adj scatter as an ordered gather),
    and the lean form that evaluates the radials where they are used, give the serial
    result bit for bit, stage buffers included."""
    g = small_golden
    species = g["species"].astype(np.int32)
    nl = {k: g[k] for k in ("num_neigh", "neigh_indices", "xyz", "r")}
    serial = Evaluator(small_model_path, "port")
    par = Evaluator(small_model_path, "port").set_threads(threads).set_lean(lean)
    for ev in (serial, par):
        ev.compute_node_energies_forces(*edge_args(species, nl))
    for name in ("node_energies", "node_forces", "A0", "M0", "H1", "Phi1", "A1", "M1", "H2", "H2_adj", "M1_adj",
                 "A1_adj", "Phi1_adj", "H1_adj", "M0_adj", "A0_adj"):
        a, b = serial.get(name), par.get(name)
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), name


@needs_ref
def test_port_matches_reference_stagewise(small_model_path):
    pos, L, species = random_box(48, 0.064, 0.9, 3, seed=21)
    nl = neighbor_list(pos, 5.0, L)
    port, ref = Evaluator(small_model_path, "port"), Evaluator(small_model_path, "reference")
    for ev in (port, ref):
        ev.compute_node_energies_forces(*edge_args(species, nl))
    for name in ("Y", "Y_grad", "R0", "R0_deriv", "R1", "R1_deriv", "A0", "M0", "H1", "Phi1r", "Phi1", "A1", "M1",
                 "H2", "node_energies", "H2_adj", "M1_adj", "A1_adj", "Phi1_adj", "H1_adj", "M0_adj", "A0_adj",
                 "node_forces"):
        a, b = port.get(name), ref.get(name)
        assert a.shape == b.shape, name
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12 * max(1.0, np.abs(b).max()), err_msg=name)


@needs_ref
def test_port_matches_reference_isolated_and_ragged(small_model_path):
    # node 3 has no neighbours; neighbour counts are uneven
    pos = np.array([[0, 0, 0], [1.2, 0.1, 0], [0.3, 1.4, 0.2], [20.0, 20, 20], [-1.0, -0.8, 0.9]], dtype=float)
    species = np.array([0, 1, 2, 1, 0], dtype=np.int32)
    nl = neighbor_list(pos, 5.0)
    assert nl["num_neigh"][3] == 0
    port, ref = Evaluator(small_model_path, "port"), Evaluator(small_model_path, "reference")
    for ev in (port, ref):
        ev.compute_node_energies_forces(*edge_args(species, nl))
    np.testing.assert_allclose(port.node_energies, ref.node_energies, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(port.node_forces, ref.node_forces, rtol=1e-10, atol=1e-13)


def test_finite_difference_edge_forces():
    """node_forces = -dE/dxyz per edge, as the reference checks it (test_mace.py:655-704)."""
    g, species, nl = _tiny()
    ev = Evaluator(os.path.join(GOLD, "tiny_model.json"), "port")
    xyz = nl["xyz"].copy()
    r = nl["r"].copy()

    def energy(x):
        rr = np.linalg.norm(x, axis=1)
        ev.compute_node_energies_forces(len(species), species, nl["num_neigh"], nl["neigh_indices"],
                                        species[nl["neigh_indices"]], x, rr)
        return ev.node_energies.sum()

    energy(xyz)
    f = ev.node_forces.reshape(-1, 3).copy()
    h = 1e-4
    for e in range(0, len(r), 5):
        for a in range(3):
            xp = xyz.copy(); xp[e, a] += h
            xm = xyz.copy(); xm[e, a] -= h
            fd = -(energy(xp) - energy(xm)) / (2 * h)
            assert fd == pytest.approx(f[e, a], rel=1e-4, abs=1e-6)


def test_rotation_invariance(small_model_path):
    """E invariant and atomic forces covariant under O(3): checks the Y_lm convention against
    the generator's Clebsch-Gordan and U tables (parity with e3nn itself is unpinned here)."""
    rng = np.random.default_rng(5)
    pos = rng.normal(size=(12, 3)) * 1.6
    species = rng.integers(0, 3, size=12).astype(np.int32)
    ev = Evaluator(small_model_path, "port")
    out = []
    for Q in (np.eye(3), random_rotation(rng), -random_rotation(rng)):
        nl = neighbor_list(pos @ Q.T, 5.0)
        ev.compute_node_energies_forces(*edge_args(species, nl))
        F = atomic_forces(12, nl["i"], nl["neigh_indices"], ev.node_forces)
        out.append((ev.node_energies.copy(), F @ Q))
    for e, F in out[1:]:
        np.testing.assert_allclose(e, out[0][0], rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(F, out[0][1], rtol=1e-8, atol=1e-9)


def test_total_force_and_torque_vanish(small_golden, small_model_path):
    g = small_golden
    species = g["species"].astype(np.int32)
    F = atomic_forces(64, g["edge_i"], g["neigh_indices"], g["node_forces"])
    np.testing.assert_allclose(F.sum(0), 0.0, atol=1e-10)


def test_invalid_inputs_raise(small_model_path):
    ev = Evaluator(small_model_path, "port")
    with pytest.raises(RuntimeError):
        ev.compute_node_energies_forces(2, [0, 1], [1, 1], [1, 5], [1, 0], np.ones((2, 3)), np.full(2, 1.7))
    with pytest.raises(RuntimeError):
        Evaluator(os.path.join(GOLD, "does_not_exist.json"), "port")


# ----- model-free primitives: the reference's known-answer tests -----

def _libs():
    out = [library("port")]
    if HAVE_REF:
        out.append(library("reference"))
    return out


def _dp(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@pytest.mark.parametrize("which", [0, 1])
def test_zbl_known_answers(which):
    libs = _libs()
    if which >= len(libs):
        pytest.skip("reference tree absent")
    lib, pre = libs[which]
    radii = np.array([0.2, 0.31, 0.28, 1.28, 0.96, 0.84, 0.76, 0.71, 0.66, 0.57, 0.58])
    c = np.array([0.1818, 0.5099, 0.2802, 0.02817])
    r_max = radii[5] + radii[10]
    env = getattr(lib, pre + "zbl_envelope")
    assert env(r_max, r_max, 6) == 0.0
    assert env(1.0, r_max, 6) == pytest.approx(0.4374788794430078)  # symmetrix/test/test_zbl.py:26
    comp = getattr(lib, pre + "zbl_compute")
    g = np.zeros(1)
    assert comp(0.3, 0.4543, _dp(c), _dp(radii), len(radii), 6, 5, 10, 1.0, _dp(g)) == pytest.approx(
        0.3166652764835175)  # test_zbl.py:42
    vp = comp(0.3, 0.4543, _dp(c), _dp(radii), len(radii), 6, 5, 10, 1.0001, None)
    vm = comp(0.3, 0.4543, _dp(c), _dp(radii), len(radii), 6, 5, 10, 0.9999, None)
    comp(0.3, 0.4543, _dp(c), _dp(radii), len(radii), 6, 5, 10, 1.0, _dp(g))
    assert g[0] == pytest.approx((vp - vm) / 2e-4, rel=1e-6)


@pytest.mark.parametrize("which", [0, 1])
def test_spline_matches_scipy(which):
    from scipy.interpolate import CubicSpline
    libs = _libs()
    if which >= len(libs):
        pytest.skip("reference tree absent")
    lib, pre = libs[which]
    rc = 5.0
    r, h = np.linspace(0, rc, 20, retstep=True)
    f = np.sin(r) * r ** 2 * (rc - r) ** 2  # symmetrix/test/test_cubic_spline.py:13-16
    spl = CubicSpline(r, f)
    d = spl.derivative()(r)
    r2 = np.linspace(0, rc, 1000, endpoint=False)
    fo, do = np.zeros(1000), np.zeros(1000)
    assert getattr(lib, pre + "spline_eval")(h, _dp(f), _dp(d), 20, _dp(r2), 1000, _dp(fo), _dp(do)) == 0
    np.testing.assert_allclose(fo, spl(r2), rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(do, spl.derivative()(r2), rtol=1e-6, atol=1e-9)
    for bad in (-1.0, 5.0, 9.0):  # out of bounds raises (test_cubic_spline.py:30-33)
        x = np.array([bad])
        assert getattr(lib, pre + "spline_eval")(h, _dp(f), _dp(d), 20, _dp(x), 1, _dp(fo), _dp(do)) != 0


@pytest.mark.parametrize("which", [0, 1])
def test_polynomial_matches_naive(which):
    libs = _libs()
    if which >= len(libs):
        pytest.skip("reference tree absent")
    lib, pre = libs[which]
    rng = np.random.default_rng(0)
    monos = [[7], [0, 1], [1, 3], [1, 1, 2], [0, 1, 2, 4], [4, 5, 6, 7]]  # test_multivariate_polynomial.py:22-23
    coef = rng.random(len(monos))
    x = rng.random(8)
    flat = np.array([v for m in monos for v in m], dtype=np.int32)
    lens = np.array([len(m) for m in monos], dtype=np.int32)
    g = np.zeros(8)
    ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    f = getattr(lib, pre + "poly_eval")(8, _dp(coef), len(monos), ip(flat), ip(lens), _dp(x), _dp(g))
    fn = sum(c * np.prod(x[m]) for c, m in zip(coef, monos))
    gn = np.zeros(8)
    for c, m in zip(coef, monos):
        for q in range(len(m)):
            gn[m[q]] += c * np.prod([x[m[u]] for u in range(len(m)) if u != q])
    assert f == pytest.approx(fn, rel=1e-12)
    np.testing.assert_allclose(g, gn, rtol=1e-12)


@pytest.mark.parametrize("which", [0, 1])
def test_mlp_matches_numpy(which):
    libs = _libs()
    if which >= len(libs):
        pytest.skip("reference tree absent")
    lib, pre = libs[which]
    rng = np.random.default_rng(1)
    w0, w1, s = rng.random((6, 3)), rng.random(6), 1.2  # test_multilayer_perceptron.py:92-95
    act = lambda x: s * x / (1 + np.exp(-x))
    x = rng.random(3)
    g = np.zeros(3)
    f = getattr(lib, pre + "mlp_eval")(3, 6, _dp(w0.flatten()), _dp(w1), s, _dp(x), _dp(g))
    assert f == pytest.approx(w1 @ act(w0 @ x), rel=1e-12)
    h = 1e-6
    gn = [(getattr(lib, pre + "mlp_eval")(3, 6, _dp(w0.flatten()), _dp(w1), s, _dp(x + h * e), _dp(np.zeros(3)))
           - getattr(lib, pre + "mlp_eval")(3, 6, _dp(w0.flatten()), _dp(w1), s, _dp(x - h * e), _dp(np.zeros(3))))
          / (2 * h) for e in np.eye(3)]
    np.testing.assert_allclose(g, gn, rtol=1e-6)


@needs_ref
def test_port_matches_reference_with_zbl(tmp_path):
    """Models with ZBL pair repulsion (zbl.cpp:96-125), close pairs inside r_max."""
    from symmetrix_gb300.synth.model import make_model, write_model
    path = write_model(make_model(num_channels=8, species=("H", "C", "O"), num_knots=40, seed=4, zbl=True,
                                  radial_hidden=(16,)), str(tmp_path / "zbl.json"))
    rng = np.random.default_rng(2)
    pos = rng.normal(size=(10, 3)) * 1.1
    species = rng.integers(0, 3, size=10).astype(np.int32)
    nl = neighbor_list(pos, 5.0)
    assert nl["r"].min() < 1.0
    port, ref = Evaluator(path, "port"), Evaluator(path, "reference")
    for ev in (port, ref):
        ev.compute_node_energies_forces(*edge_args(species, nl))
    np.testing.assert_allclose(port.node_energies, ref.node_energies, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(port.node_forces, ref.node_forces, rtol=1e-10, atol=1e-12)


def _halo_golden(tmp_path):
    from make_golden import halo_case, halo_model, model_fingerprint
    g = dict(np.load(os.path.join(GOLD, "halo_golden.npz")))
    path = halo_model(str(tmp_path / "halo.json"))
    np.testing.assert_allclose(model_fingerprint(path), g["model_fingerprint"], rtol=1e-10)
    c = halo_case()
    assert np.array_equal(c["node_atom"], g["node_atom"])
    assert np.array_equal(c["num_neigh"], g["num_neigh"])
    assert np.array_equal(c["neigh_indices"], g["neigh_indices"])
    return g, c, path


def _halo_eval(path, which, c, n_local):
    ev = Evaluator(path, which)
    ev.compute_halo(n_local, len(c["node_atom"]), c["node_types"], c["num_neigh"], c["neigh_indices"],
                    c["neigh_types"], c["xyz"], c["r"])
    return ev


def test_halo_golden_matches_reference_outputs(tmp_path):
    """The pair style's no-MPI-message-passing stage calls (pair_symmetrix_mace.cpp:672-698:
    layer 0 over local + halo nodes, layer 1, readouts and ZBL over the local ones) in
    the port, against the reference's outputs on the same halo graph."""
    g, c, path = _halo_golden(tmp_path)
    ev = _halo_eval(path, "port", c, int(g["n_local"]))
    assert len(ev.node_energies) == int(g["n_local"])
    np.testing.assert_allclose(ev.node_energies, g["node_energies"], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(ev.node_forces, g["node_forces"], rtol=1e-8, atol=1e-10)
    for s in ("A0", "M0", "H1", "Phi1", "A1", "M1", "H2", "H1_adj", "M0_adj", "A0_adj", "Phi1_adj"):
        assert ev.get(s).sum() == pytest.approx(g["sum_" + s], rel=1e-9, abs=1e-10), s


@needs_ref
def test_port_matches_reference_halo_stagewise(tmp_path):
    g, c, path = _halo_golden(tmp_path)
    port, ref = (_halo_eval(path, w, c, int(g["n_local"])) for w in ("port", "reference"))
    for name in ("A0", "M0", "H1", "Phi1", "A1", "M1", "H2", "node_energies", "H2_adj", "M1_adj", "A1_adj",
                 "Phi1_adj", "H1_adj", "M0_adj", "A0_adj", "node_forces"):
        a, b = port.get(name), ref.get(name)
        assert a.shape == b.shape, name
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12 * max(1.0, np.abs(b).max()), err_msg=name)


def test_halo_evaluation_equals_periodic_evaluation(tmp_path):
    """On one rank the halo nodes are periodic images, so the halo form gives the periodic
    box's node energies, and after each ghost's force is added to its local atom (LAMMPS's
    reverse communication) its atomic forces and virial."""
    from helpers import fold_halo_forces, virial
    g, c, path = _halo_golden(tmp_path)
    n = int(g["n_local"])
    halo = _halo_eval(path, "port", c, n)
    nl = neighbor_list(c["pos"], 5.0, c["L"])
    per = Evaluator(path, "port")
    per.compute_node_energies_forces(*edge_args(c["species"].astype(np.int32), nl))
    np.testing.assert_allclose(halo.node_energies, per.node_energies, rtol=1e-12, atol=1e-12)
    F_halo = fold_halo_forces(len(c["x"]), c["local_of"], c["node_atom"], c["num_neigh"], c["neigh_atom"],
                              halo.node_forces)
    F_per = atomic_forces(n, nl["i"], nl["neigh_indices"], per.node_forces)
    np.testing.assert_allclose(F_halo, F_per, rtol=1e-10, atol=1e-11)
    np.testing.assert_allclose(virial(c["xyz"], halo.node_forces), virial(nl["xyz"], per.node_forces), rtol=1e-10,
                               atol=1e-10)


@needs_ref
def test_reference_message_passing_on_one_rank_is_the_owner_map(tmp_path):
    """The identity the pair adapter's mpi_message_passing mode rests on, shown with the
    reference's own stages: its stage sequence on one rank, with the ghosts' H1 rows filled
    from their owners and their H1_adj rows added back (pair_symmetrix_mace.cpp:438-497),
    gives the energies and per-edge forces of the plain evaluation whose neighbour indices
    are the owners themselves."""
    from make_golden import halo_model
    from symmetrix_gb300.synth.structures import lammps_rank
    path = halo_model(str(tmp_path / "halo.json"))
    pos, L, species = random_box(24, 0.064, 0.9, 3, seed=7)
    n, rc = len(pos), 5.0
    x, owner, lists = lammps_rank(pos, L, rc + 0.5, rc + 0.5, ghost_lists=False)
    sp = species[owner].astype(np.int32)
    ei, ej = [], []
    for i in range(n):
        d = np.linalg.norm(x[lists[i]] - x[i], axis=1)
        js = lists[i][d < rc]
        ei.append(np.full(len(js), i))
        ej.append(js)
    ei, ej = np.concatenate(ei), np.concatenate(ej)
    assert (ej >= n).any()  # some neighbours are ghosts
    xyz = x[ej] - x[ei]
    r = np.linalg.norm(xyz, axis=1)
    nn = np.bincount(ei, minlength=n)
    mp, plain = Evaluator(path, "reference"), Evaluator(path, "reference")
    mp.compute_message_passing(n, len(x), sp[:n], nn, ej, sp[ej], xyz, r, owner)
    plain.compute_node_energies_forces(n, sp[:n], nn, owner[ej], sp[ej], xyz, r)
    np.testing.assert_allclose(mp.node_energies, plain.node_energies, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(mp.node_forces, plain.node_forces, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("threads,lean", [(3, False), (4, True)])
def test_threaded_halo_evaluation_is_bitwise_serial(tmp_path, threads, lean):
    """The halo evaluation split over node ranges (the H1_adj gather runs over every H1
    row, the halo's included) gives the serial result bit for bit; with no halo it is the
    plain evaluation bit for bit."""
    g, c, path = _halo_golden(tmp_path)
    n = int(g["n_local"])
    serial = _halo_eval(path, "port", c, n)
    par = Evaluator(path, "port").set_threads(threads).set_lean(lean)
    par.compute_halo(n, len(c["node_atom"]), c["node_types"], c["num_neigh"], c["neigh_indices"],
                     c["neigh_types"], c["xyz"], c["r"])
    for name in ("node_energies", "node_forces", "H1", "A1", "H1_adj", "M0_adj", "A0_adj", "Phi1_adj"):
        assert np.array_equal(serial.get(name).view(np.uint64), par.get(name).view(np.uint64)), name
    N0 = len(c["node_atom"])
    args = (c["node_types"], c["num_neigh"], c["neigh_indices"], c["neigh_types"], c["xyz"], c["r"])
    full, plain = Evaluator(path, "port"), Evaluator(path, "port")
    full.compute_halo(N0, N0, *args)
    plain.compute_node_energies_forces(N0, *args)
    for name in ("node_energies", "node_forces", "H1_adj", "A0_adj"):
        assert np.array_equal(full.get(name).view(np.uint64), plain.get(name).view(np.uint64)), name
