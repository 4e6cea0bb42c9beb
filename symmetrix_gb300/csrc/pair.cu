// LAMMPS pair-style adapter: one compute() of pair_style symmetrix/mace on one rank, in
// any of its three modes (pair_symmetrix/pair_symmetrix_mace.cpp:64-77), with the
// neighbour filtering, the evaluation and the force scatter on the GPU.
//
// The caller passes LAMMPS's own arrays: the full neighbour list (inum local entries of
// ilist, then gnum ghost entries when it asked for ghost lists, numneigh, firstneigh,
// NEIGHMASK), positions x[nall][3] of local and ghost atoms, atom types,
// local_of[j] = atom->map(atom->tag[j]) (the local owner of a ghost) and the LAMMPS
// type -> model species map.  The list topology is uploaded when the caller says it
// changed (LAMMPS re-neighbouring); every call uploads only x.
//
// Per call on the device: each node's list entries with 0 < r^2 < r_cut^2 become the
// engine's CSR edges (xyz = x_j - x_i), the engine evaluates, forces are scattered
// F_i -= f_e, F_target(j) += f_e (float64 atomics: the summation order, hence the last
// bits, may differ between runs), and energy and virial sum_e xyz_a f_b are reduced on
// the device.  The modes differ in the nodes, the node an edge's H1 row comes from and
// where its neighbour force lands:
//   no_domain_decomposition (:242-372): nodes = the local atoms; H1 row and force of
//     neighbour j at its owner local_of[j];
//   mpi_message_passing (:376-547): the same evaluation -- on one rank the forward
//     exchange of H1 to the ghosts and the reverse exchange of their H1_adj (:462-490)
//     are the ghost -> owner map itself -- with the force of j left on the ghost row j
//     for LAMMPS's own reverse communication;
//   no_mpi_message_passing (:551-748): nodes = the local atoms, then the ghosts within
//     r_cut of a local atom in ascending index order (found on the device each call);
//     layer 0 runs over all of them and layer 1, ZBL and the readouts over the local
//     ones (smx_compute_halo's evaluation); forces land on the atoms of each edge,
//     ghosts included.
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.hpp"

using smx::fail;

namespace {

// in-cut-off candidates of each node: num_neigh[ii] for the atom nodes[ii]
__global__ void k_pair_count(int n_nodes, const int* __restrict__ nodes, const int* __restrict__ aoff,
                             const int* __restrict__ cand_j, const double* __restrict__ x, double rc2,
                             int* __restrict__ num_neigh) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= n_nodes) return;
  const int i = nodes[ii];
  const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  int n = 0;
  for (int c = aoff[i]; c < aoff[i + 1]; ++c) {
    const int j = cand_j[c];
    const double dx = x[3 * j] - xi, dy = x[3 * j + 1] - yi, dz = x[3 * j + 2] - zi;
    const double r2 = dx * dx + dy * dy + dz * dz;
    n += (r2 < rc2 && r2 > 0.0) ? 1 : 0;
  }
  num_neigh[ii] = n;
}

// The edges: neighbour node node_map[owner ? owner[j] : j] (a node whose H1 row is read;
// -1 is an error for the first n_local nodes and 0 for a halo node's edge, whose index
// is never read, as the reference's map lookup gives), force target owner[j] when
// scatter_owner, else j.
__global__ void k_pair_fill(int n_nodes, int n_local, const int* __restrict__ nodes, const int* __restrict__ aoff,
                            const int* __restrict__ cand_j, const double* __restrict__ x, double rc2,
                            const int* __restrict__ first, const int* __restrict__ mtype,
                            const int* __restrict__ owner, const int* __restrict__ node_map, int scatter_owner,
                            int* __restrict__ node_type, int* __restrict__ nidx, int* __restrict__ ntype_e,
                            double* __restrict__ xyz, double* __restrict__ r, int* __restrict__ nbr_atom,
                            unsigned* __restrict__ bad) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= n_nodes) return;
  const int i = nodes[ii];
  node_type[ii] = mtype[i];
  const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  int e = first[ii];
  for (int c = aoff[i]; c < aoff[i + 1]; ++c) {
    const int j = cand_j[c];
    const double dx = x[3 * j] - xi, dy = x[3 * j + 1] - yi, dz = x[3 * j + 2] - zi;
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (!(r2 < rc2 && r2 > 0.0)) continue;
    const int jo = owner ? owner[j] : j;
    const int node = node_map[jo];
    if (node < 0 && ii < n_local) atomicOr(bad, 1u);
    nidx[e] = node < 0 ? 0 : node;
    ntype_e[e] = mtype[j];
    xyz[3 * e] = dx;
    xyz[3 * e + 1] = dy;
    xyz[3 * e + 2] = dz;
    r[e] = sqrt(r2);
    nbr_atom[e] = scatter_owner ? jo : j;
    ++e;
  }
}

// no-MPI-message-passing mode: flag[j] = 1 for every non-local atom within r_cut of a
// local one (pair_symmetrix_mace.cpp:557-580)
__global__ void k_halo_mark(int inum, const int* __restrict__ nodes, const int* __restrict__ aoff,
                            const int* __restrict__ cand_j, const double* __restrict__ x, double rc2,
                            const int* __restrict__ node_of_local, int* __restrict__ flag) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= inum) return;
  const int i = nodes[ii];
  const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  for (int c = aoff[i]; c < aoff[i + 1]; ++c) {
    const int j = cand_j[c];
    const double dx = x[3 * j] - xi, dy = x[3 * j + 1] - yi, dz = x[3 * j + 2] - zi;
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < rc2 && r2 > 0.0 && node_of_local[j] < 0) flag[j] = 1;
  }
}

// halo nodes inum + gfirst[a] for the flagged atoms, in ascending atom order, and the
// atom -> node map of this call; bad |= 2 for a halo atom without a neighbour list
__global__ void k_halo_nodes(int nall, int inum, const int* __restrict__ flag, const int* __restrict__ gfirst,
                             const int* __restrict__ node_of_local, const int* __restrict__ has_list,
                             int* __restrict__ nodes, int* __restrict__ node_of_atom, unsigned* __restrict__ bad) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nall) return;
  if (flag[a]) {
    const int n = inum + gfirst[a];
    nodes[n] = a;
    node_of_atom[a] = n;
    if (!has_list[a]) atomicOr(bad, 2u);
  } else {
    node_of_atom[a] = node_of_local[a];
  }
}

__global__ void k_pair_scatter(int n_nodes, const int* __restrict__ first, const int* __restrict__ nodes,
                               const int* __restrict__ nbr_atom, const double* __restrict__ fe,
                               double* __restrict__ f) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= n_nodes) return;
  double sx = 0.0, sy = 0.0, sz = 0.0;
  for (int e = first[ii]; e < first[ii + 1]; ++e) {
    const double fx = fe[3 * e], fy = fe[3 * e + 1], fz = fe[3 * e + 2];
    sx += fx;
    sy += fy;
    sz += fz;
    const int j = nbr_atom[e];
    atomicAdd(f + 3 * j, fx);
    atomicAdd(f + 3 * j + 1, fy);
    atomicAdd(f + 3 * j + 2, fz);
  }
  const int i = nodes[ii];
  atomicAdd(f + 3 * i, -sx);
  atomicAdd(f + 3 * i + 1, -sy);
  atomicAdd(f + 3 * i + 2, -sz);
}

constexpr int kReduceBlocks = 64;

}  // namespace

struct smx_pair {
  smx_engine* eng = nullptr;
  int mode = -1, inum = 0, gnum = 0, nall = 0, ncand = 0;
  // topology (uploaded on re-neighbouring): per-atom candidate ranges aoff[nall + 1] into
  // cand_j of the atoms with a list, nodes[0, inum) = ilist (the halo nodes follow per call)
  int *nodes = nullptr, *aoff = nullptr, *cand_j = nullptr, *mtype = nullptr, *local_of = nullptr;
  int *node_of_local = nullptr, *has_list = nullptr, *num_neigh = nullptr, *nbr_atom = nullptr;
  int *flag = nullptr, *gfirst = nullptr, *node_of_atom = nullptr;  // halo search (no-MPI-message-passing)
  double *x = nullptr, *f = nullptr, *partial = nullptr, *out = nullptr;
  unsigned* bad = nullptr;
  int* count_host = nullptr;  // pinned: the halo node count read back each call
  long cap_nall = 0, cap_cand = 0;
  std::vector<double> h_out = std::vector<double>(10);

  void free_all() {
    void* ps[] = {nodes, aoff, cand_j, mtype, local_of, node_of_local, has_list, num_neigh, nbr_atom, flag,
                  gfirst, node_of_atom, x, f, partial, out, bad};
    for (void* p : ps)
      if (p) cudaFree(p);
    nodes = aoff = cand_j = mtype = local_of = node_of_local = has_list = num_neigh = nbr_atom = nullptr;
    flag = gfirst = node_of_atom = nullptr;
    x = f = partial = out = nullptr;
    bad = nullptr;
    cap_nall = cap_cand = 0;
  }

  // nodes never outnumber the atoms: buffers per node are sized by nall
  void reserve(int na, int nc) {
    if (na <= cap_nall && nc <= cap_cand && x) return;
    free_all();
    cap_nall = std::max(na, 1);
    cap_cand = std::max(nc, 1);
    nodes = dalloc<int>(cap_nall);
    aoff = dalloc<int>(cap_nall + 1);
    num_neigh = dalloc<int>(cap_nall);
    cand_j = dalloc<int>(cap_cand);
    nbr_atom = dalloc<int>(cap_cand);
    mtype = dalloc<int>(cap_nall);
    local_of = dalloc<int>(cap_nall);
    node_of_local = dalloc<int>(cap_nall);
    has_list = dalloc<int>(cap_nall);
    flag = dalloc<int>(cap_nall);
    gfirst = dalloc<int>(cap_nall + 1);
    node_of_atom = dalloc<int>(cap_nall);
    x = dalloc<double>(3 * cap_nall);
    f = dalloc<double>(3 * cap_nall);
    partial = dalloc<double>(10 * kReduceBlocks);
    out = dalloc<double>(10);
    bad = dalloc<unsigned>(1);
  }
};

extern "C" {

smx_pair* smx_pair_create(smx_engine* eng) {
  if (!eng) {
    fail(SMX_ERR_INVALID, "engine is NULL");
    return nullptr;
  }
  auto* p = new smx_pair;
  p->eng = eng;
  return p;
}

void smx_pair_destroy(smx_pair* p) {
  if (!p) return;
  cudaSetDevice(p->eng->device);
  cudaStreamSynchronize(p->eng->stream);
  p->free_all();
  if (p->count_host) cudaFreeHost(p->count_host);
  delete p;
}

int smx_pair_compute_mode(smx_pair* p, int mode, int inum, int gnum, int nall, const int* ilist,
                          const int* numneigh, const int* const* firstneigh, int neighmask, int neigh_changed,
                          const double* x, const int* type, const int* local_of, const int* mace_types, int ntypes,
                          int eflag_global, int eflag_atom, int vflag_global, double* f, double* eng_vdwl,
                          double* eatom, double* virial) {
  if (!p) return fail(SMX_ERR_INVALID, "pair adapter is NULL");
  if (mode != SMX_PAIR_NO_DOMAIN_DECOMPOSITION && mode != SMX_PAIR_MPI_MESSAGE_PASSING &&
      mode != SMX_PAIR_NO_MPI_MESSAGE_PASSING)
    return fail(SMX_ERR_INVALID, "unknown pair-style mode");
  const bool halo = mode == SMX_PAIR_NO_MPI_MESSAGE_PASSING;
  if (!halo) gnum = 0;  // the other modes read the local atoms' lists only
  if (inum < 0 || gnum < 0 || nall < inum + gnum) return fail(SMX_ERR_INVALID, "need 0 <= inum, gnum and inum + gnum <= nall");
  if (nall > 0 && (!x || !f)) return fail(SMX_ERR_INVALID, "NULL x or f");
  smx_engine* eng = p->eng;
  const int S = eng->hm.S;
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    cudaStream_t s = eng->stream;
    if (neigh_changed || mode != p->mode || inum != p->inum || gnum != p->gnum || nall != p->nall) {
      const int nlist = inum + gnum;
      if (nlist > 0 && (!ilist || !numneigh || !firstneigh)) return fail(SMX_ERR_INVALID, "NULL neighbour-list array");
      if (nall > 0 && (!type || !mace_types)) return fail(SMX_ERR_INVALID, "NULL atom array");
      if (!halo && inum > 0 && !local_of) return fail(SMX_ERR_INVALID, "NULL local_of");
      std::vector<int> cnt(nall, 0), listed(nall, 0), mt(nall), nol(nall, -1), lo;
      for (int ii = 0; ii < nlist; ++ii) {
        const int i = ilist[ii];
        if (i < 0 || i >= nall) return fail(SMX_ERR_INVALID, "ilist entry out of range");
        if (numneigh[i] < 0) return fail(SMX_ERR_INVALID, "negative numneigh");
        if (listed[i]) return fail(SMX_ERR_INVALID, "atom listed twice in ilist");
        listed[i] = 1;
        cnt[i] = numneigh[i];
        if (ii < inum) nol[i] = ii;
      }
      std::vector<int> aoff(static_cast<size_t>(nall) + 1, 0);
      for (int a = 0; a < nall; ++a) aoff[a + 1] = aoff[a] + cnt[a];
      std::vector<int> cj(aoff[nall]);
      for (int ii = 0; ii < nlist; ++ii) {
        const int i = ilist[ii];
        for (int jj = 0; jj < numneigh[i]; ++jj) {
          const int j = firstneigh[i][jj] & neighmask;
          if (j < 0 || j >= nall) return fail(SMX_ERR_INVALID, "neighbour index out of range");
          cj[aoff[i] + jj] = j;
        }
      }
      for (int a = 0; a < nall; ++a) {
        if (type[a] < 1 || type[a] > ntypes) return fail(SMX_ERR_INVALID, "atom type out of range");
        mt[a] = mace_types[type[a] - 1];
        if (mt[a] < 0 || mt[a] >= S) return fail(SMX_ERR_INVALID, "mace_types entry out of range");
        if (!halo && (local_of[a] < 0 || local_of[a] >= nall))
          return fail(SMX_ERR_INVALID, "local_of entry out of range");
      }
      p->reserve(nall, aoff[nall]);
      if (!p->count_host) check(cudaMallocHost(&p->count_host, sizeof(int)), "cudaMallocHost");
      if (inum > 0) check(cudaMemcpyAsync(p->nodes, ilist, sizeof(int) * inum, cudaMemcpyHostToDevice, s), "H2D");
      if (nall > 0) {
        check(cudaMemcpyAsync(p->aoff, aoff.data(), sizeof(int) * (nall + 1), cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(p->mtype, mt.data(), sizeof(int) * nall, cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(p->node_of_local, nol.data(), sizeof(int) * nall, cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(p->has_list, listed.data(), sizeof(int) * nall, cudaMemcpyHostToDevice, s), "H2D");
        if (!halo)
          check(cudaMemcpyAsync(p->local_of, local_of, sizeof(int) * nall, cudaMemcpyHostToDevice, s), "H2D");
      }
      if (!cj.empty())
        check(cudaMemcpyAsync(p->cand_j, cj.data(), sizeof(int) * cj.size(), cudaMemcpyHostToDevice, s), "H2D");
      check(cudaStreamSynchronize(s), "topology upload");  // host vectors go out of scope
      p->mode = mode;
      p->inum = inum;
      p->gnum = gnum;
      p->nall = nall;
      p->ncand = aoff[nall];
    }
    if (inum == 0) return SMX_OK;
    const double rc = eng->hm.r_cut;
    check(cudaMemcpyAsync(p->x, x, sizeof(double) * 3 * nall, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemsetAsync(p->f, 0, sizeof(double) * 3 * nall, s), "memset");
    check(cudaMemsetAsync(p->bad, 0, sizeof(unsigned), s), "memset");
    int n_nodes = inum;
    const int* node_map = p->node_of_local;
    if (halo) {  // the ghosts within r_cut of a local atom become halo nodes
      check(cudaMemsetAsync(p->flag, 0, sizeof(int) * nall, s), "memset");
      k_halo_mark<<<smx::ceil_div(inum, 128), 128, 0, s>>>(inum, p->nodes, p->aoff, p->cand_j, p->x, rc * rc,
                                                           p->node_of_local, p->flag);
      smx::launch_scan_first(p->flag, nall, p->gfirst, s);
      check(cudaMemcpyAsync(p->count_host, p->gfirst + nall, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
      check(cudaStreamSynchronize(s), "halo count");
      n_nodes = inum + *p->count_host;
      k_halo_nodes<<<smx::ceil_div(nall, 128), 128, 0, s>>>(nall, inum, p->flag, p->gfirst, p->node_of_local,
                                                            p->has_list, p->nodes, p->node_of_atom, p->bad);
      node_map = p->node_of_atom;
    }
    eng->reserve(n_nodes, p->ncand);  // edges are a subset of the listed candidates
    const int nb = smx::ceil_div(n_nodes, 128);
    k_pair_count<<<nb, 128, 0, s>>>(n_nodes, p->nodes, p->aoff, p->cand_j, p->x, rc * rc, p->num_neigh);
    smx::launch_scan_first(p->num_neigh, n_nodes, eng->first, s);
    if (n_nodes > inum)  // the halo nodes' energy slots stay zero for the reduction below
      check(cudaMemsetAsync(eng->energies + inum, 0, sizeof(double) * (n_nodes - inum), s), "memset");
    k_pair_fill<<<nb, 128, 0, s>>>(n_nodes, inum, p->nodes, p->aoff, p->cand_j, p->x, rc * rc, eng->first,
                                   p->mtype, halo ? nullptr : p->local_of, node_map,
                                   mode == SMX_PAIR_NO_DOMAIN_DECOMPOSITION ? 1 : 0, eng->ntype, eng->nidx,
                                   eng->ntype_e, eng->xyz, eng->r, p->nbr_atom, p->bad);
    smx::EdgeIn in{eng->first, eng->ntype, eng->nidx, eng->ntype_e, eng->xyz, eng->r, n_nodes};
    eng->run(in, eng->energies, eng->forces, s, inum);
    k_pair_scatter<<<nb, 128, 0, s>>>(n_nodes, eng->first, p->nodes, p->nbr_atom, eng->forces, p->f);
    smx::launch_reduce(n_nodes, eng->first, eng->energies, eng->xyz, eng->forces, p->partial, kReduceBlocks, p->out,
                       s);
    std::vector<double> hf(static_cast<size_t>(3) * nall);
    unsigned hbad = 0;
    check(cudaMemcpyAsync(hf.data(), p->f, sizeof(double) * 3 * nall, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaMemcpyAsync(p->h_out.data(), p->out, sizeof(double) * 10, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaMemcpyAsync(&hbad, p->bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "D2H");
    if (eflag_atom && eatom)
      check(cudaMemcpyAsync(eatom, eng->energies, sizeof(double) * inum, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "pair compute");
    if (eng->take_status() != SMX_OK) return fail(SMX_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
    if (hbad & 2u)
      return fail(SMX_ERR_INVALID,
                  "a ghost within r_cut of a local atom has no neighbour list (no_mpi_message_passing needs the "
                  "ghost neighbour list)");
    if (hbad & 1u) return fail(SMX_ERR_INVALID, "a neighbour's local owner is not in ilist");
    for (long q = 0; q < 3L * nall; ++q) f[q] += hf[q];
    const double* o = p->h_out.data();
    if (eflag_global && eng_vdwl) *eng_vdwl += o[0];
    if (vflag_global && virial) {
      const double* W = o + 1;  // W_ab = sum_e xyz_a f_b, row-major
      virial[0] += W[0];
      virial[1] += W[4];
      virial[2] += W[8];
      virial[3] += 0.5 * (W[1] + W[3]);
      virial[4] += 0.5 * (W[2] + W[6]);
      virial[5] += 0.5 * (W[5] + W[7]);
    }
  } catch (const std::exception& e) {
    return fail(SMX_ERR_CUDA, e.what());
  }
  return SMX_OK;
}

int smx_pair_compute(smx_pair* p, int inum, int nall, const int* ilist, const int* numneigh,
                     const int* const* firstneigh, int neighmask, int neigh_changed, const double* x, const int* type,
                     const int* local_of, const int* mace_types, int ntypes, int eflag_global, int eflag_atom,
                     int vflag_global, double* f, double* eng_vdwl, double* eatom, double* virial) {
  return smx_pair_compute_mode(p, SMX_PAIR_NO_DOMAIN_DECOMPOSITION, inum, 0, nall, ilist, numneigh, firstneigh,
                               neighmask, neigh_changed, x, type, local_of, mace_types, ntypes, eflag_global,
                               eflag_atom, vflag_global, f, eng_vdwl, eatom, virial);
}

}  // extern "C"
