"""Generate the golden fixtures in this directory from the REFERENCE evaluator.

Run where the reference tree is present (it builds oracle/_ref from the
reference's own libsymmetrix sources):

    python tests/golden/make_golden.py

Writes
  tiny_model.json   a complete 2-species, 4-channel model in libsymmetrix's JSON format
  tiny_golden.json  a 7-atom cluster, its neighbour list, and the reference's node
                    energies, per-edge forces and stage sums on it
  small_golden.npz  the 64-atom, 3-species box of the CPU-runnable workload
                    (positions, species, neighbour list) with the reference's outputs
                    on the seeded 32-channel model `small_model()` regenerates
  halo_golden.npz   a 24-atom periodic box as one LAMMPS rank holds it, evaluated in the
                    pair style's no-MPI-message-passing form (layer 0 over the local
                    atoms and the ghosts within r_cut of them, layer 1 over the local
                    atoms) by the reference's own stages, on the density-scaled ZBL
                    model `halo_model()` regenerates; the node and edge arrays are
                    rebuilt from the positions by tests/helpers.py (halo_graph)

`python tests/golden/make_golden.py halo` writes halo_golden.npz alone.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import Evaluator  # noqa: E402
from symmetrix_gb300.synth.model import CONFIGS, make_model, write_model  # noqa: E402
from symmetrix_gb300.synth.structures import neighbor_list, random_box  # noqa: E402

STAGES = ["A0", "M0", "H1", "Phi1", "A1", "M1", "H2", "H2_adj", "M1_adj", "A1_adj", "Phi1_adj", "H1_adj",
          "M0_adj", "A0_adj"]

SMALL_SEED, SMALL_AVG_NEIGH, SMALL_STRUCT_SEED = 1, 33.5, 3
HALO_SEED, HALO_STRUCT_SEED, HALO_ATOMS = 5, 7, 24


def small_model(path):
    """The seeded model of the 64-atom CPU-runnable workload (32x0e+32x1o, H/C/O)."""
    return write_model(make_model(**CONFIGS["small"], seed=SMALL_SEED, avg_num_neighbors=SMALL_AVG_NEIGH), path)


def halo_model(path):
    """The seeded density-scaled ZBL model of the halo fixture (32 channels, H/C/O)."""
    return write_model(make_model(**CONFIGS["small"], seed=HALO_SEED, density_scaled=True, zbl=True), path)


def halo_case():
    """The 24-atom box of the halo fixture as one LAMMPS rank holds it: positions inside
    the box, then the halo graph (list cutoff r_cut + 0.5 A skin, ghost shell
    2 r_cut + 0.5 A, as the pair style sets the communication cutoff)."""
    sys.path.insert(0, os.path.dirname(HERE))
    from helpers import fake_lammps, halo_graph
    pos, L, species = random_box(HALO_ATOMS, 0.064, 0.9, 3, seed=HALO_STRUCT_SEED)
    pos = pos - L * np.floor(pos / L)
    x, local_of, nbrs = fake_lammps(pos, L, 5.5, shell=10.5, ghost_lists=True)
    node_atom, num_neigh, nidx, natom, xyz, r = halo_graph(x, len(pos), nbrs, 5.0)
    sp = species[local_of]
    return dict(pos=pos, L=L, species=species, x=x, local_of=local_of, node_atom=node_atom, num_neigh=num_neigh,
                neigh_indices=nidx, neigh_atom=natom, node_types=sp[node_atom].astype(np.int32),
                neigh_types=sp[natom].astype(np.int32), xyz=xyz, r=r)


def write_halo_golden():
    path = halo_model("/tmp/smx_halo_model.json")
    c = halo_case()
    ev = Evaluator(path, "reference")
    ev.compute_halo(HALO_ATOMS, len(c["node_atom"]), c["node_types"], c["num_neigh"], c["neigh_indices"],
                    c["neigh_types"], c["xyz"], c["r"])
    sums = {"sum_" + s: float(ev.get(s).sum()) for s in STAGES}
    np.savez_compressed(os.path.join(HERE, "halo_golden.npz"), positions=c["pos"], box=c["L"],
                        species=c["species"], n_local=HALO_ATOMS, node_atom=c["node_atom"],
                        num_neigh=c["num_neigh"], neigh_indices=c["neigh_indices"],
                        model_fingerprint=model_fingerprint(path), node_energies=ev.node_energies,
                        node_forces=ev.node_forces, **sums)
    print("halo: N0", len(c["node_atom"]), "E", len(c["r"]), "E_local", ev.node_energies.sum())


def model_fingerprint(path):
    """A few sums over the model file: regenerating the model must reproduce them."""
    with open(path) as f:
        m = json.load(f)
    return np.array([np.abs(np.asarray(m["radial_spline_values_1"])).sum(),
                     sum(np.abs(np.asarray(v)).sum() for s in m["M0_weights"].values() for l in s.values()
                         for v in l.values()),
                     sum(np.abs(np.asarray(v)).sum() for s in m["M1_weights"].values() for v in s.values()),
                     np.abs(np.asarray(m["A1_weights"][1])).sum(), np.abs(np.asarray(m["Phi1_clebsch_gordan"])).sum()])


def tiny_cluster():
    pos = np.array([[0.0, -2.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [2.1, 1.3, -0.4],
                    [-1.2, 0.4, 1.1], [0.7, -0.6, 1.9], [3.2, -0.9, 0.8]])
    species = np.array([1, 0, 0, 1, 0, 1, 0], dtype=np.int32)  # index into atomic_numbers [H, O]
    return pos, species


def run_reference(model_path, n, species, nl):
    ev = Evaluator(model_path, "reference")
    ev.compute_node_energies_forces(n, species, nl["num_neigh"], nl["neigh_indices"], species[nl["neigh_indices"]],
                                    nl["xyz"], nl["r"])
    out = {"node_energies": ev.node_energies, "node_forces": ev.node_forces}
    for s in STAGES:
        out["sum_" + s] = float(ev.get(s).sum())
    return out


def main():
    tiny_path = os.path.join(HERE, "tiny_model.json")
    model = make_model(num_channels=4, species=("H", "O"), r_cut=5.0, L_max=1, num_knots=12, seed=11,
                       avg_num_neighbors=6.0, radial_hidden=(8,))
    with open(tiny_path, "w") as f:
        json.dump(model, f)
    pos, species = tiny_cluster()
    nl = neighbor_list(pos, 5.0)
    out = run_reference(tiny_path, len(pos), species, nl)
    golden = {"positions": pos.tolist(), "species": species.tolist(), "num_neigh": nl["num_neigh"].tolist(),
              "neigh_indices": nl["neigh_indices"].tolist(), "xyz": nl["xyz"].tolist(), "r": nl["r"].tolist()}
    golden.update({k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in out.items()})
    with open(os.path.join(HERE, "tiny_golden.json"), "w") as f:
        json.dump(golden, f)

    small_path = "/tmp/smx_small_model.json"
    small_model(small_path)
    pos, L, species = random_box(64, 0.064, 0.9, 3, seed=SMALL_STRUCT_SEED)
    nl = neighbor_list(pos, 5.0, L)
    out = run_reference(small_path, 64, species, nl)
    np.savez_compressed(os.path.join(HERE, "small_golden.npz"), positions=pos, box=L, species=species,
                        num_neigh=nl["num_neigh"], neigh_indices=nl["neigh_indices"], xyz=nl["xyz"], r=nl["r"],
                        edge_i=nl["i"], model_fingerprint=model_fingerprint(small_path), **out)
    print("wrote", tiny_path, "and goldens; small E =", out["node_energies"].sum())
    write_halo_golden()


if __name__ == "__main__":
    if sys.argv[1:] == ["halo"]:
        write_halo_golden()
    else:
        main()
