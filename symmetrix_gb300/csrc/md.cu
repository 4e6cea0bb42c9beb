// Atom-level evaluation and the velocity-Verlet MD driver (C ABI in include/smx_gb300.h).
//
// These are the GPU-resident counterparts of what the reference's callers do
// around MACE::compute_node_energies_forces: build the neighbour list, call the
// evaluator, scatter per-edge forces to atoms and reduce the virial
// (pair_symmetrix/pair_symmetrix_mace.cpp:242-372; symmetrix_calc.py:72-102), and,
// for MD, LAMMPS's `fix nve` (the reference's tests run it in
// pair_symmetrix/test/test_pair_symmetrix_mace.py:253).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "engine.hpp"

using smx::fail;

namespace {

// Full directed neighbour list on the device with a skin, CSR by centre atom.
struct NeighList {
  int capN = 0, ncell_cap = 0, cell_atoms_cap = 0;
  long capE = 0;
  int *cell = nullptr, *cell_count = nullptr, *cell_start = nullptr, *cell_fill = nullptr, *cell_atoms = nullptr;
  int* cell_tmp = nullptr;  // the binned atoms before each cell is sorted
  float4* posf = nullptr;   // float32 positions of the neighbour search
  int* cellseg = nullptr;   // [N][28]: start of each of the 27 neighbour cells' segment in an atom's list, end
  int *num_neigh = nullptr, *first = nullptr, *nidx = nullptr, *ntype_e = nullptr, *edge_i = nullptr, *rev = nullptr;
  char4* shift = nullptr;
  double *xyz = nullptr, *r = nullptr, *forces = nullptr;
  // the edges inside the cut-off, packed per centre atom each step (a skin list)
  int *last = nullptr, *emap = nullptr, *pinv = nullptr, *nidx_p = nullptr, *ntype_p = nullptr;
  double *xyz_p = nullptr, *r_p = nullptr, *forces_p = nullptr;
  long E = 0;
  bool realloc_happened = false;

  ~NeighList() { release(); }
  void release() {
    void* ps[] = {cell,  cell_count, cell_start, cell_fill, cell_atoms, num_neigh, first, nidx,  ntype_e,
                  edge_i, rev,       shift,      xyz,       r,          forces,    last,  emap,  pinv,
                  nidx_p, ntype_p,   xyz_p,      r_p,       forces_p,   cell_tmp,  posf,  cellseg};
    for (void* p : ps)
      if (p) cudaFree(p);
    cell = cell_count = cell_start = cell_fill = cell_atoms = num_neigh = first = nidx = ntype_e = edge_i = rev = nullptr;
    last = emap = pinv = nidx_p = ntype_p = cell_tmp = nullptr;
    shift = nullptr;
    posf = nullptr;
    cellseg = nullptr;
    xyz = r = forces = xyz_p = r_p = forces_p = nullptr;
    capN = ncell_cap = cell_atoms_cap = 0;
    capE = 0;
  }
  void reserve_nodes(int N, int ncell) {
    if (N > capN) {
      for (int** p : {&cell, &num_neigh, &first, &last})
        if (*p) cudaFree(*p);
      if (posf) cudaFree(posf);
      if (cellseg) cudaFree(cellseg);
      cell = dalloc<int>(N);
      num_neigh = dalloc<int>(N);
      first = dalloc<int>(N + 1);
      last = dalloc<int>(N);
      posf = dalloc<float4>(N);
      cellseg = dalloc<int>(28L * N);
      capN = N;
      realloc_happened = true;
    }
    if (ncell + 1 > ncell_cap) {
      for (int** p : {&cell_count, &cell_start, &cell_fill})
        if (*p) cudaFree(*p);
      cell_count = dalloc<int>(ncell + 1);
      cell_start = dalloc<int>(ncell + 2);
      cell_fill = dalloc<int>(ncell + 1);
      ncell_cap = ncell + 1;
    }
    if (N > cell_atoms_cap) {
      for (int** p : {&cell_atoms, &cell_tmp})
        if (*p) cudaFree(*p);
      cell_atoms = dalloc<int>(N);
      cell_tmp = dalloc<int>(N);
      cell_atoms_cap = N;
    }
  }
  void reserve_edges(long E_) {
    if (E_ <= capE) return;
    const long nE = static_cast<long>(E_ * 1.25) + 1024;
    void* ps[] = {nidx, ntype_e, edge_i, rev, shift, xyz, r, forces, emap, pinv, nidx_p, ntype_p, xyz_p, r_p,
                  forces_p};
    for (void* p : ps)
      if (p) cudaFree(p);
    nidx = dalloc<int>(nE);
    ntype_e = dalloc<int>(nE);
    edge_i = dalloc<int>(nE);
    rev = dalloc<int>(nE);
    shift = dalloc<char4>(nE);
    xyz = dalloc<double>(3 * nE);
    r = dalloc<double>(nE);
    forces = dalloc<double>(3 * nE);
    emap = dalloc<int>(nE);
    pinv = dalloc<int>(nE);
    nidx_p = dalloc<int>(nE);
    ntype_p = dalloc<int>(nE);
    xyz_p = dalloc<double>(3 * nE);
    r_p = dalloc<double>(nE);
    forces_p = dalloc<double>(3 * nE);
    capE = nE;
    realloc_happened = true;
  }

  // Build the list for positions pos (wrapped in place for periodic axes).  With
  // segments (seg_of[atom], seg_first[segment]: a batch of non-periodic molecules) only
  // atoms of the same segment are neighbours.
  void build(double* pos, const int* species, int N, double3 box, int3 periodic, double rl, cudaStream_t s,
             const int* seg_of = nullptr, const int* seg_first = nullptr) {
    const double L[3] = {box.x, box.y, box.z};
    const int per[3] = {periodic.x, periodic.y, periodic.z};
    int n[3];
    bool brute = false;
    int3 nimg = make_int3(0, 0, 0);
    int* img[3] = {&nimg.x, &nimg.y, &nimg.z};
    for (int d = 0; d < 3; ++d) {
      if (!per[d]) {
        brute = true;
        n[d] = 1;
        continue;
      }
      n[d] = static_cast<int>(std::floor(L[d] / rl));
      *img[d] = static_cast<int>(std::ceil(rl / L[d]));
      if (n[d] < 3) brute = true;
    }
    if (brute && !seg_of && N > 200000)
      throw std::invalid_argument("non-periodic or small-box neighbour search is limited to 200000 atoms");
    const int3 nc = make_int3(n[0], n[1], n[2]);
    reserve_nodes(N, nc.x * nc.y * nc.z);
    smx::launch_wrap(N, box, periodic, pos, s);
    if (!brute)
      smx::launch_cell_list(pos, N, box, nc, cell, cell_count, cell_start, cell_fill, cell_tmp, cell_atoms, s);
    smx::launch_neigh_pass(false, brute, pos, posf, species, N, box, nc, periodic, nimg, rl, cell, cell_start,
                           cell_atoms, seg_of, seg_first, num_neigh, first, nidx, ntype_e, edge_i, shift, capE, s);
    smx::launch_scan_first(num_neigh, N, first, s);
    int total = 0;
    check(cudaMemcpyAsync(&total, first + N, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "neighbour count");
    E = total;
    reserve_edges(E);
    int* seg = brute ? nullptr : cellseg;
    smx::launch_neigh_pass(true, brute, pos, posf, species, N, box, nc, periodic, nimg, rl, cell, cell_start,
                           cell_atoms, seg_of, seg_first, num_neigh, first, nidx, ntype_e, edge_i, shift, capE, s,
                           seg);
    if (seg)
      smx::launch_reverse_edges_cells(capE, N, first, nidx, edge_i, shift, cell, nc, seg, rev, s);
    else
      smx::launch_reverse_edges(capE, N, first, nidx, edge_i, shift, rev, s);
  }
};

void box_args(const double* box_lengths, double3& box, int3& periodic) {
  if (box_lengths) {
    box = make_double3(box_lengths[0], box_lengths[1], box_lengths[2]);
    periodic = make_int3(1, 1, 1);
    if (!(box.x > 0 && box.y > 0 && box.z > 0)) throw std::invalid_argument("box lengths must be positive");
  } else {
    box = make_double3(1.0, 1.0, 1.0);
    periodic = make_int3(0, 0, 0);
  }
}

// Molecule offsets (mol_first[0] = 0 <= ... <= mol_first[n_mol] = n_atoms) -> the
// atom -> molecule map.
std::vector<int> molecule_of(int n_mol, const int* mol_first, int n_atoms) {
  if (n_mol < 0 || (n_mol > 0 && !mol_first)) throw std::invalid_argument("bad molecule offsets");
  if (n_mol == 0) {
    if (n_atoms != 0) throw std::invalid_argument("atoms outside every molecule");
    return {};
  }
  if (mol_first[0] != 0 || mol_first[n_mol] != n_atoms)
    throw std::invalid_argument("molecule offsets must start at 0 and end at n_atoms");
  std::vector<int> of(n_atoms);
  for (int m = 0; m < n_mol; ++m) {
    if (mol_first[m + 1] < mol_first[m]) throw std::invalid_argument("molecule offsets must not decrease");
    for (int a = mol_first[m]; a < mol_first[m + 1]; ++a) of[a] = m;
  }
  return of;
}

}  // namespace

// ---------------------------------------------------------------------------
// MD driver
// ---------------------------------------------------------------------------
struct smx_md {
  smx_engine* eng = nullptr;
  int device = 0;  // kept here: destruction must not touch the engine, which may be gone
  int N = 0;
  double3 box{};
  int3 periodic{};
  double dt = 0.5, skin = 1.0;
  int rebuild_every = 10;
  long step = 0;
  double *pos = nullptr, *vel = nullptr, *F = nullptr, *inv_m = nullptr, *energies = nullptr, *partial = nullptr,
         *reduced = nullptr;
  int* species = nullptr;
  int *seg_of = nullptr, *seg_first = nullptr;  // molecule batch: atom -> molecule, molecule atom offsets
  // Spatial renumbering (periodic boxes): every kSortEvery steps, at a neighbour rebuild, the
  // atoms are renumbered in cell-list order (cells in index order, atoms of a cell by index),
  // as MD codes sort their atoms: the neighbours of the centres that the blocks in flight
  // work on then sit in a few contiguous index ranges, so their node features (H1, the
  // fixed-point H1_adj rows, A0 ...) stay in L2 on boxes whose features exceed it.  orig[k]
  // is the caller's index of the atom in slot k; smx_md_state reports in the caller's order.
  bool sort_atoms = false;
  static constexpr int kSortEvery = 200;
  long last_sort = -1;
  int* orig = nullptr;
  double* tmp_d = nullptr;  // [10 N]: the gather of a renumbering
  int* tmp_i = nullptr;     // [2 N]
  NeighList nl;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  static constexpr int kReduceBlocks = 64;

  ~smx_md() {
    if (graph) cudaGraphExecDestroy(graph);
    void* ps[] = {pos, vel, F, inv_m, energies, partial, reduced, species, seg_of, seg_first, orig, tmp_d, tmp_i};
    for (void* p : ps)
      if (p) cudaFree(p);
  }

  smx::EdgeIn edges() const {
    return smx::EdgeIn{nl.first, species, nl.nidx, nl.ntype_e, nl.xyz, nl.r, N};
  }

  // forces at the current positions (geometry + evaluator + atomic forces), and with
  // kick the second velocity-Verlet half step; graph-capturable.  With a skin the
  // evaluator sees only the edges inside the cut-off, packed per atom (the skin edges
  // would cost it ~5% of its time), and the atomic forces come from the packed edges'
  // forces through the skin list's reverse-edge map (skin_view restores the skin list's
  // geometry and forces for a state read-out).
  void forces(cudaStream_t s, bool kick = false) {
    if (skin > 0.0) {
      smx::launch_edge_geometry_packed(N, nl.first, pos, box, nl.nidx, nl.ntype_e, nl.shift, eng->hm.r_cut, nl.pinv,
                                       nl.last, nl.emap, nl.nidx_p, nl.ntype_p, nl.xyz_p, nl.r_p, s);
      smx::EdgeIn in{nl.first, species, nl.nidx_p, nl.ntype_p, nl.xyz_p, nl.r_p, N};
      in.last = nl.last;
      eng->run(in, energies, nl.forces_p, s);
      smx::launch_atom_forces_packed(N, nl.first, nl.last, nl.emap, nl.rev, nl.pinv, nl.forces_p, F, kick ? dt : 0.0,
                                     inv_m, vel, s);
      return;
    }
    smx::launch_edge_geometry(nl.capE, N, nl.first, pos, box, nl.nidx, nl.edge_i, nl.shift, nl.xyz, nl.r, s);
    eng->run(edges(), energies, nl.forces, s);
    smx::launch_atom_forces(N, nl.first, nl.rev, nl.forces, F, s);
    if (kick) smx::launch_vv_second(N, dt, F, inv_m, vel, s);
  }

  // the skin list's edge vectors and per-edge forces (zero beyond the cut-off) of the last
  // force evaluation, for the energy and virial sums
  void skin_view(cudaStream_t s) {
    if (skin <= 0.0 || N == 0) return;
    smx::launch_edge_geometry(nl.capE, N, nl.first, pos, box, nl.nidx, nl.edge_i, nl.shift, nl.xyz, nl.r, s);
    check(cudaMemsetAsync(nl.forces, 0, sizeof(double) * 3 * nl.E, s), "cudaMemsetAsync");
    smx::launch_scatter_packed_forces(N, nl.first, nl.last, nl.emap, nl.forces_p, nl.forces, s);
  }

  void one_step(cudaStream_t s) {
    smx::launch_vv_first(N, dt, F, inv_m, vel, pos, s);
    forces(s, true);
  }

  // renumber the atoms in the cell list's order (no-op for boxes too small for cells)
  void renumber(cudaStream_t s) {
    const double rl = eng->hm.r_cut + skin;
    const double L[3] = {box.x, box.y, box.z};
    int n[3];
    for (int d = 0; d < 3; ++d) {
      n[d] = static_cast<int>(std::floor(L[d] / rl));
      if (n[d] < 3) return;
    }
    const int3 nc = make_int3(n[0], n[1], n[2]);
    nl.reserve_nodes(N, nc.x * nc.y * nc.z);
    smx::launch_wrap(N, box, periodic, pos, s);
    smx::launch_cell_list(pos, N, box, nc, nl.cell, nl.cell_count, nl.cell_start, nl.cell_fill, nl.cell_tmp,
                          nl.cell_atoms, s);
    smx::launch_permute_atoms(N, nl.cell_atoms, pos, vel, F, inv_m, species, orig, tmp_d, tmp_i, s);
    const size_t n3 = sizeof(double) * 3 * N;
    check(cudaMemcpyAsync(pos, tmp_d, n3, cudaMemcpyDeviceToDevice, s), "D2D");
    check(cudaMemcpyAsync(vel, tmp_d + 3L * N, n3, cudaMemcpyDeviceToDevice, s), "D2D");
    check(cudaMemcpyAsync(F, tmp_d + 6L * N, n3, cudaMemcpyDeviceToDevice, s), "D2D");
    check(cudaMemcpyAsync(inv_m, tmp_d + 9L * N, sizeof(double) * N, cudaMemcpyDeviceToDevice, s), "D2D");
    check(cudaMemcpyAsync(species, tmp_i, sizeof(int) * N, cudaMemcpyDeviceToDevice, s), "D2D");
    check(cudaMemcpyAsync(orig, tmp_i + N, sizeof(int) * N, cudaMemcpyDeviceToDevice, s), "D2D");
  }

  void rebuild(cudaStream_t s) {
    if (sort_atoms && (last_sort < 0 || step - last_sort >= kSortEvery)) {
      renumber(s);
      last_sort = step;
    }
    nl.realloc_happened = false;
    nl.build(pos, species, N, box, periodic, eng->hm.r_cut + skin, s, seg_of, seg_first);
    eng->reserve(N, nl.capE);
    if (nl.realloc_happened && graph) {
      cudaGraphExecDestroy(graph);
      graph = nullptr;
    }
  }

  // a batch of independent non-periodic molecules: neighbours only inside a molecule
  void set_molecules(int n_mol, const int* mol_first, cudaStream_t s) {
    const std::vector<int> of = molecule_of(n_mol, mol_first, N);
    seg_of = dalloc<int>(N);
    seg_first = dalloc<int>(n_mol + 1);
    check(cudaMemcpyAsync(seg_of, of.data(), sizeof(int) * N, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemcpyAsync(seg_first, mol_first, sizeof(int) * (n_mol + 1), cudaMemcpyHostToDevice, s), "H2D");
    check(cudaStreamSynchronize(s), "molecule upload");  // `of` goes out of scope
  }

  void run(int steps) {
    cudaStream_t s = eng->stream;
    const bool prof = eng->profile;
    eng->profile = false;
    while (steps > 0) {
      if (step % rebuild_every == 0) rebuild(s);
      const int seg = std::min<long>(steps, rebuild_every - step % rebuild_every);
      if (seg == rebuild_every) {
        if (!graph || graph_steps != seg) {
          if (graph) cudaGraphExecDestroy(graph);
          graph = nullptr;
          cudaGraph_t g;
          check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
          for (int q = 0; q < seg; ++q) one_step(s);
          check(cudaStreamEndCapture(s, &g), "cudaStreamEndCapture");
          check(cudaGraphInstantiate(&graph, g, 0), "cudaGraphInstantiate");
          cudaGraphDestroy(g);
          graph_steps = seg;
        }
        check(cudaGraphLaunch(graph, s), "cudaGraphLaunch");
      } else {
        for (int q = 0; q < seg; ++q) one_step(s);
      }
      step += seg;
      steps -= seg;
    }
    check(cudaGetLastError(), "MD launch");
    eng->profile = prof;
  }
};

extern "C" {

}  // extern "C"

namespace {

int compute_atoms_impl(smx_engine* eng, int n_atoms, const double* positions, const int* species,
                       const double* box_lengths, int n_mol, const int* mol_first, double* energy,
                       double* node_energies, double* forces, double* virial) {
  if (!eng) return fail(SMX_ERR_INVALID, "engine is NULL");
  if (n_atoms < 0 || (n_atoms > 0 && (!positions || !species || !forces)))
    return fail(SMX_ERR_INVALID, "bad atom arrays");
  for (int a = 0; a < n_atoms; ++a)
    if (species[a] < 0 || species[a] >= eng->hm.S) return fail(SMX_ERR_INVALID, "species out of range");
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    double3 box;
    int3 periodic;
    box_args(box_lengths, box, periodic);
    smx_md md;  // borrowed as a workspace: no dynamics
    md.eng = eng;
    md.N = n_atoms;
    md.box = box;
    md.periodic = periodic;
    md.skin = 0.0;
    cudaStream_t s = eng->stream;
    if (n_atoms == 0) {
      if (energy) *energy = 0.0;
      if (virial) std::memset(virial, 0, 9 * sizeof(double));
      return SMX_OK;
    }
    md.pos = dalloc<double>(3 * n_atoms);
    md.F = dalloc<double>(3 * n_atoms);
    md.energies = dalloc<double>(n_atoms);
    md.species = dalloc<int>(n_atoms);
    md.partial = dalloc<double>(10 * smx_md::kReduceBlocks);
    md.reduced = dalloc<double>(10);
    check(cudaMemcpyAsync(md.pos, positions, sizeof(double) * 3 * n_atoms, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemcpyAsync(md.species, species, sizeof(int) * n_atoms, cudaMemcpyHostToDevice, s), "H2D");
    if (mol_first) md.set_molecules(n_mol, mol_first, s);
    md.rebuild(s);
    md.forces(s);
    smx::launch_reduce(n_atoms, md.nl.first, md.energies, md.nl.xyz, md.nl.forces, md.partial, smx_md::kReduceBlocks,
                       md.reduced, s);
    double red[10];
    check(cudaMemcpyAsync(red, md.reduced, sizeof(red), cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaMemcpyAsync(forces, md.F, sizeof(double) * 3 * n_atoms, cudaMemcpyDeviceToHost, s), "D2H");
    if (node_energies)
      check(cudaMemcpyAsync(node_energies, md.energies, sizeof(double) * n_atoms, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "evaluation");
    if (energy) *energy = red[0];
    if (virial)
      for (int q = 0; q < 9; ++q) virial[q] = red[1 + q];
  } catch (const CudaError& e) {
    return fail(SMX_ERR_CUDA, e.what());
  } catch (const std::exception& e) {
    return fail(SMX_ERR_INVALID, e.what());
  }
  if (eng->take_status() != SMX_OK) return fail(SMX_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
  return SMX_OK;
}

smx_md* md_create_impl(smx_engine* eng, int n_atoms, const double* positions, const double* velocities,
                       const int* species, const double* masses, const double* box_lengths, int n_mol,
                       const int* mol_first, double dt_fs, double skin, int rebuild_every) {
  if (!eng || n_atoms <= 0 || !positions || !species || !masses || rebuild_every < 1 || !(dt_fs > 0) ||
      !(skin >= 0)) {
    fail(SMX_ERR_INVALID, "bad MD arguments");
    return nullptr;
  }
  for (int a = 0; a < n_atoms; ++a)
    if (species[a] < 0 || species[a] >= eng->hm.S || !(masses[a] > 0)) {
      fail(SMX_ERR_INVALID, "species out of range or non-positive mass");
      return nullptr;
    }
  auto md = std::make_unique<smx_md>();
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    box_args(box_lengths, md->box, md->periodic);
    md->eng = eng;
    md->device = eng->device;
    md->N = n_atoms;
    md->dt = dt_fs;
    md->skin = skin;
    md->rebuild_every = rebuild_every;
    cudaStream_t s = eng->stream;
    md->pos = dalloc<double>(3 * n_atoms);
    md->vel = dalloc<double>(3 * n_atoms);
    md->F = dalloc<double>(3 * n_atoms);
    md->inv_m = dalloc<double>(n_atoms);
    md->energies = dalloc<double>(n_atoms);
    md->species = dalloc<int>(n_atoms);
    md->partial = dalloc<double>(10 * smx_md::kReduceBlocks);
    md->reduced = dalloc<double>(10);
    std::vector<double> inv(n_atoms), v(3 * static_cast<size_t>(n_atoms), 0.0);
    for (int a = 0; a < n_atoms; ++a) inv[a] = 1.0 / masses[a];
    if (velocities) std::memcpy(v.data(), velocities, sizeof(double) * 3 * n_atoms);
    check(cudaMemcpyAsync(md->pos, positions, sizeof(double) * 3 * n_atoms, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemcpyAsync(md->vel, v.data(), sizeof(double) * 3 * n_atoms, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemcpyAsync(md->inv_m, inv.data(), sizeof(double) * n_atoms, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemcpyAsync(md->species, species, sizeof(int) * n_atoms, cudaMemcpyHostToDevice, s), "H2D");
    if (mol_first) md->set_molecules(n_mol, mol_first, s);
    if (box_lengths && !mol_first) {  // periodic box: spatial renumbering (see smx_md)
      md->sort_atoms = true;
      md->orig = dalloc<int>(n_atoms);
      md->tmp_d = dalloc<double>(10L * n_atoms);
      md->tmp_i = dalloc<int>(2L * n_atoms);
      std::vector<int> id(n_atoms);
      for (int a = 0; a < n_atoms; ++a) id[a] = a;
      check(cudaMemcpyAsync(md->orig, id.data(), sizeof(int) * n_atoms, cudaMemcpyHostToDevice, s), "H2D");
      check(cudaMemsetAsync(md->F, 0, sizeof(double) * 3 * n_atoms, s), "cudaMemsetAsync");
      check(cudaStreamSynchronize(s), "upload");  // `id` goes out of scope
    }
    md->rebuild(s);
    md->forces(s);
    check(cudaStreamSynchronize(s), "initial forces");
  } catch (const CudaError& e) {
    fail(SMX_ERR_CUDA, e.what());
    return nullptr;
  } catch (const std::exception& e) {
    fail(SMX_ERR_INVALID, e.what());
    return nullptr;
  }
  return md.release();
}

}  // namespace

extern "C" {

int smx_compute_atoms(smx_engine* eng, int n_atoms, const double* positions, const int* species,
                      const double* box_lengths, double* energy, double* node_energies, double* forces,
                      double* virial) {
  return compute_atoms_impl(eng, n_atoms, positions, species, box_lengths, 0, nullptr, energy, node_energies, forces,
                            virial);
}

int smx_compute_molecules(smx_engine* eng, int n_mol, const int* mol_first, const double* positions,
                          const int* species, double* mol_energies, double* node_energies, double* forces) {
  if (n_mol < 0 || (n_mol > 0 && !mol_first)) return fail(SMX_ERR_INVALID, "bad molecule offsets");
  const int n_atoms = n_mol > 0 ? mol_first[n_mol] : 0;
  std::vector<double> ne(static_cast<size_t>(n_atoms));
  const int code = compute_atoms_impl(eng, n_atoms, positions, species, nullptr, n_mol, n_mol > 0 ? mol_first : nullptr,
                                      nullptr, ne.data(), forces, nullptr);
  if (code != SMX_OK) return code;
  if (node_energies && n_atoms > 0) std::memcpy(node_energies, ne.data(), sizeof(double) * n_atoms);
  if (mol_energies)
    for (int m = 0; m < n_mol; ++m) {
      double e = 0.0;
      for (int a = mol_first[m]; a < mol_first[m + 1]; ++a) e += ne[a];
      mol_energies[m] = e;
    }
  return SMX_OK;
}

smx_md* smx_md_create(smx_engine* eng, int n_atoms, const double* positions, const double* velocities,
                      const int* species, const double* masses, const double* box_lengths, double dt_fs, double skin,
                      int rebuild_every) {
  return md_create_impl(eng, n_atoms, positions, velocities, species, masses, box_lengths, 0, nullptr, dt_fs, skin,
                        rebuild_every);
}

smx_md* smx_md_create_molecules(smx_engine* eng, int n_mol, const int* mol_first, const double* positions,
                                const double* velocities, const int* species, const double* masses, double dt_fs,
                                double skin, int rebuild_every) {
  if (n_mol <= 0 || !mol_first) {
    fail(SMX_ERR_INVALID, "bad molecule offsets");
    return nullptr;
  }
  return md_create_impl(eng, mol_first[n_mol], positions, velocities, species, masses, nullptr, n_mol, mol_first,
                        dt_fs, skin, rebuild_every);
}

int smx_md_run(smx_md* md, int steps) {
  if (!md || steps < 0) return fail(SMX_ERR_INVALID, "bad MD arguments");
  try {
    check(cudaSetDevice(md->eng->device), "cudaSetDevice");
    md->run(steps);
  } catch (const CudaError& e) {
    return fail(SMX_ERR_CUDA, e.what());
  } catch (const std::exception& e) {
    return fail(SMX_ERR_INVALID, e.what());
  }
  return SMX_OK;
}

int smx_md_sync(smx_md* md) {
  if (!md) return fail(SMX_ERR_INVALID, "md is NULL");
  const cudaError_t e = cudaStreamSynchronize(md->eng->stream);
  if (e != cudaSuccess) return fail(SMX_ERR_CUDA, cudaGetErrorString(e));
  if (md->eng->take_status() != SMX_OK) return fail(SMX_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
  return SMX_OK;
}

int smx_md_state(smx_md* md, double* positions, double* velocities, double* forces, double* potential_energy,
                 double* virial, long* step) {
  if (!md) return fail(SMX_ERR_INVALID, "md is NULL");
  try {
    cudaStream_t s = md->eng->stream;
    const int N = md->N;
    md->skin_view(s);
    smx::launch_reduce(N, md->nl.first, md->energies, md->nl.xyz, md->nl.forces, md->partial, smx_md::kReduceBlocks,
                       md->reduced, s);
    double red[10];
    check(cudaMemcpyAsync(red, md->reduced, sizeof(red), cudaMemcpyDeviceToHost, s), "D2H");
    if (!md->sort_atoms) {
      if (positions) check(cudaMemcpyAsync(positions, md->pos, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s), "D2H");
      if (velocities) check(cudaMemcpyAsync(velocities, md->vel, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s), "D2H");
      if (forces) check(cudaMemcpyAsync(forces, md->F, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s), "D2H");
      check(cudaStreamSynchronize(s), "MD state");
    } else {  // renumbered atoms: slot k back to the caller's index orig[k]
      std::vector<int> orig(N);
      std::vector<double> tmp(3 * static_cast<size_t>(N));
      check(cudaMemcpyAsync(orig.data(), md->orig, sizeof(int) * N, cudaMemcpyDeviceToHost, s), "D2H");
      check(cudaStreamSynchronize(s), "MD state");
      for (int q = 0; q < 3; ++q) {
        double* out = q == 0 ? positions : (q == 1 ? velocities : forces);
        const double* src = q == 0 ? md->pos : (q == 1 ? md->vel : md->F);
        if (!out) continue;
        check(cudaMemcpy(tmp.data(), src, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost), "D2H");
        for (int k = 0; k < N; ++k)
          for (int c = 0; c < 3; ++c) out[3 * static_cast<size_t>(orig[k]) + c] = tmp[3 * static_cast<size_t>(k) + c];
      }
    }
    if (potential_energy) *potential_energy = red[0];
    if (virial)
      for (int q = 0; q < 9; ++q) virial[q] = red[1 + q];
    if (step) *step = md->step;
  } catch (const std::exception& e) {
    return fail(SMX_ERR_CUDA, e.what());
  }
  if (md->eng->take_status() != SMX_OK) return fail(SMX_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
  return SMX_OK;
}

long smx_md_num_edges(smx_md* md) { return md ? md->nl.E : -1; }

void smx_md_destroy(smx_md* md) {
  if (!md) return;
  // the engine (and its stream) may already be destroyed: wait on the device instead
  cudaSetDevice(md->device);
  cudaDeviceSynchronize();
  delete md;
}

}  // extern "C"
