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

// The per-node kernels below run one warp per node (blocks of kWarpsPerBlock whole warps,
// a warp exits as one) and walk the node's candidates 32 at a time in list order, so a
// ballot keeps the edges in that order.  Candidate j of centre i is an edge when
// 0 < r^2 < r_cut^2, r^2 formed by explicit FMAs so that every kernel takes the same
// decision for the same pair.
constexpr int kWarpsPerBlock = 8;

__device__ __forceinline__ double pair_r2(const double* __restrict__ x, double xi, double yi, double zi, int j,
                                          double& dx, double& dy, double& dz) {
  dx = x[3 * j] - xi;
  dy = x[3 * j + 1] - yi;
  dz = x[3 * j + 2] - zi;
  return fma(dz, dz, fma(dy, dy, dx * dx));
}

__device__ __forceinline__ int node_warp() {
  return static_cast<int>((blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x) >> 5);
}

// in-cut-off candidates of each node: num_neigh[w] for the atom nodes[w]
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    k_pair_count(int n_nodes, const int* __restrict__ nodes, const int* __restrict__ aoff,
                 const int* __restrict__ cand_j, const double* __restrict__ x, double rc2,
                 int* __restrict__ num_neigh) {
  const int w = node_warp(), lane = threadIdx.x & 31;
  if (w >= n_nodes) return;
  const int i = nodes[w];
  const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  const int c1 = aoff[i + 1];
  int n = 0;
  for (int c0 = aoff[i]; c0 < c1; c0 += 32) {
    const int c = c0 + lane;
    bool in = false;
    if (c < c1) {
      double dx, dy, dz;
      const double r2 = pair_r2(x, xi, yi, zi, cand_j[c], dx, dy, dz);
      in = r2 < rc2 && r2 > 0.0;
    }
    n += __popc(__ballot_sync(0xffffffffu, in));
  }
  if (lane == 0) num_neigh[w] = n;
}

// The edges: neighbour node node_map[owner ? owner[j] : j] (a node whose H1 row is read;
// -1 is an error for the first n_local nodes and 0 for a halo node's edge, whose index
// is never read, as the reference's map lookup gives), force target owner[j] when
// scatter_owner, else j.
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    k_pair_fill(int n_nodes, int n_local, const int* __restrict__ nodes, const int* __restrict__ aoff,
                const int* __restrict__ cand_j, const double* __restrict__ x, double rc2,
                const int* __restrict__ first, const int* __restrict__ mtype, const int* __restrict__ owner,
                const int* __restrict__ node_map, int scatter_owner, int* __restrict__ node_type,
                int* __restrict__ nidx, int* __restrict__ ntype_e, double* __restrict__ xyz, double* __restrict__ r,
                int* __restrict__ nbr_atom, unsigned* __restrict__ bad) {
  const int w = node_warp(), lane = threadIdx.x & 31;
  if (w >= n_nodes) return;
  const int i = nodes[w];
  if (lane == 0) node_type[w] = mtype[i];
  const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  const int c1 = aoff[i + 1];
  const int e_end = first[w + 1];
  int e = first[w];
  for (int c0 = aoff[i]; c0 < c1; c0 += 32) {
    const int c = c0 + lane;
    bool in = false;
    int j = 0;
    double dx = 0.0, dy = 0.0, dz = 0.0, r2 = 0.0;
    if (c < c1) {
      j = cand_j[c];
      r2 = pair_r2(x, xi, yi, zi, j, dx, dy, dz);
      in = r2 < rc2 && r2 > 0.0;
    }
    const unsigned ball = __ballot_sync(0xffffffffu, in);
    const int slot = e + __popc(ball & ((1u << lane) - 1u));
    if (in && slot < e_end) {  // (the count pass took the same decisions: slot < e_end)
      const int jo = owner ? owner[j] : j;
      const int node = node_map[jo];
      if (node < 0 && w < n_local) atomicOr(bad, 1u);
      nidx[slot] = node < 0 ? 0 : node;
      ntype_e[slot] = mtype[j];
      xyz[3 * slot] = dx;
      xyz[3 * slot + 1] = dy;
      xyz[3 * slot + 2] = dz;
      r[slot] = sqrt(r2);
      nbr_atom[slot] = scatter_owner ? jo : j;
    }
    e += __popc(ball);
  }
}

// no-MPI-message-passing mode: flag[j] = 1 for every non-local atom within r_cut of a
// local one (pair_symmetrix_mace.cpp:557-580)
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    k_halo_mark(int inum, const int* __restrict__ nodes, const int* __restrict__ aoff,
                const int* __restrict__ cand_j, const double* __restrict__ x, double rc2,
                const int* __restrict__ node_of_local, int* __restrict__ flag) {
  const int w = node_warp(), lane = threadIdx.x & 31;
  if (w >= inum) return;
  const int i = nodes[w];
  const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  const int c1 = aoff[i + 1];
  for (int c = aoff[i] + lane; c < c1; c += 32) {
    const int j = cand_j[c];
    double dx, dy, dz;
    const double r2 = pair_r2(x, xi, yi, zi, j, dx, dy, dz);
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

// F_i -= sum_e f_e over the node's edges (a warp sum), F_target(e) += f_e
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    k_pair_scatter(int n_nodes, const int* __restrict__ first, const int* __restrict__ nodes,
                   const int* __restrict__ nbr_atom, const double* __restrict__ fe, double* __restrict__ f) {
  const int w = node_warp(), lane = threadIdx.x & 31;
  if (w >= n_nodes) return;
  double sx = 0.0, sy = 0.0, sz = 0.0;
  for (int e = first[w] + lane; e < first[w + 1]; e += 32) {
    const double fx = fe[3 * e], fy = fe[3 * e + 1], fz = fe[3 * e + 2];
    sx += fx;
    sy += fy;
    sz += fz;
    const int j = nbr_atom[e];
    atomicAdd(f + 3 * j, fx);
    atomicAdd(f + 3 * j + 1, fy);
    atomicAdd(f + 3 * j + 2, fz);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
    sz += __shfl_xor_sync(0xffffffffu, sz, o);
  }
  if (lane == 0) {
    const int i = nodes[w];
    atomicAdd(f + 3 * i, -sx);
    atomicAdd(f + 3 * i + 1, -sy);
    atomicAdd(f + 3 * i + 2, -sz);
  }
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
  // pinned host staging: positions in, forces / node energies / sums / flags out
  double *hx = nullptr, *hf = nullptr, *he = nullptr, *hout = nullptr;
  unsigned* hbad = nullptr;
  int* count_host = nullptr;  // pinned: the halo node count read back each call
  long cap_nall = 0, cap_cand = 0;

  void free_all() {
    void* ps[] = {nodes, aoff, cand_j, mtype, local_of, node_of_local, has_list, num_neigh, nbr_atom, flag,
                  gfirst, node_of_atom, x, f, partial, out, bad};
    for (void* p : ps)
      if (p) cudaFree(p);
    nodes = aoff = cand_j = mtype = local_of = node_of_local = has_list = num_neigh = nbr_atom = nullptr;
    flag = gfirst = node_of_atom = nullptr;
    x = f = partial = out = nullptr;
    bad = nullptr;
    void* hs[] = {hx, hf, he, hout, hbad};
    for (void* h : hs)
      if (h) cudaFreeHost(h);
    hx = hf = he = hout = nullptr;
    hbad = nullptr;
    cap_nall = cap_cand = 0;
  }

  template <typename T>
  static T* host_alloc(long n) {
    void* h = nullptr;
    smx::check(cudaMallocHost(&h, sizeof(T) * static_cast<size_t>(n)), "cudaMallocHost");
    return static_cast<T*>(h);
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
    hx = host_alloc<double>(3 * cap_nall);
    hf = host_alloc<double>(3 * cap_nall);
    he = host_alloc<double>(cap_nall);
    hout = host_alloc<double>(10);
    hbad = host_alloc<unsigned>(1);
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
    std::memcpy(p->hx, x, sizeof(double) * 3 * nall);
    check(cudaMemcpyAsync(p->x, p->hx, sizeof(double) * 3 * nall, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemsetAsync(p->f, 0, sizeof(double) * 3 * nall, s), "memset");
    check(cudaMemsetAsync(p->bad, 0, sizeof(unsigned), s), "memset");
    int n_nodes = inum;
    const int* node_map = p->node_of_local;
    if (halo) {  // the ghosts within r_cut of a local atom become halo nodes
      check(cudaMemsetAsync(p->flag, 0, sizeof(int) * nall, s), "memset");
      k_halo_mark<<<smx::ceil_div(inum, kWarpsPerBlock), 32 * kWarpsPerBlock, 0, s>>>(
          inum, p->nodes, p->aoff, p->cand_j, p->x, rc * rc, p->node_of_local, p->flag);
      smx::launch_scan_first(p->flag, nall, p->gfirst, s);
      check(cudaMemcpyAsync(p->count_host, p->gfirst + nall, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
      check(cudaStreamSynchronize(s), "halo count");
      n_nodes = inum + *p->count_host;
      k_halo_nodes<<<smx::ceil_div(nall, 128), 128, 0, s>>>(nall, inum, p->flag, p->gfirst, p->node_of_local,
                                                            p->has_list, p->nodes, p->node_of_atom, p->bad);
      node_map = p->node_of_atom;
    }
    eng->reserve(n_nodes, p->ncand);  // edges are a subset of the listed candidates
    const int nb = smx::ceil_div(n_nodes, kWarpsPerBlock), bt = 32 * kWarpsPerBlock;
    k_pair_count<<<nb, bt, 0, s>>>(n_nodes, p->nodes, p->aoff, p->cand_j, p->x, rc * rc, p->num_neigh);
    smx::launch_scan_first(p->num_neigh, n_nodes, eng->first, s);
    if (n_nodes > inum)  // the halo nodes' energy slots stay zero for the reduction below
      check(cudaMemsetAsync(eng->energies + inum, 0, sizeof(double) * (n_nodes - inum), s), "memset");
    k_pair_fill<<<nb, bt, 0, s>>>(n_nodes, inum, p->nodes, p->aoff, p->cand_j, p->x, rc * rc, eng->first,
                                   p->mtype, halo ? nullptr : p->local_of, node_map,
                                   mode == SMX_PAIR_NO_DOMAIN_DECOMPOSITION ? 1 : 0, eng->ntype, eng->nidx,
                                   eng->ntype_e, eng->xyz, eng->r, p->nbr_atom, p->bad);
    smx::EdgeIn in{eng->first, eng->ntype, eng->nidx, eng->ntype_e, eng->xyz, eng->r, n_nodes};
    eng->run(in, eng->energies, eng->forces, s, inum);
    k_pair_scatter<<<nb, bt, 0, s>>>(n_nodes, eng->first, p->nodes, p->nbr_atom, eng->forces, p->f);
    smx::launch_reduce(n_nodes, eng->first, eng->energies, eng->xyz, eng->forces, p->partial, kReduceBlocks, p->out,
                       s);
    check(cudaMemcpyAsync(p->hf, p->f, sizeof(double) * 3 * nall, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaMemcpyAsync(p->hout, p->out, sizeof(double) * 10, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaMemcpyAsync(p->hbad, p->bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "D2H");
    const bool want_eatom = eflag_atom && eatom;
    if (want_eatom)
      check(cudaMemcpyAsync(p->he, eng->energies, sizeof(double) * inum, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "pair compute");
    const unsigned hbad = *p->hbad;
    const double* hf = p->hf;
    if (eng->take_status() != SMX_OK) return fail(SMX_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
    if (hbad & 2u)
      return fail(SMX_ERR_INVALID,
                  "a ghost within r_cut of a local atom has no neighbour list (no_mpi_message_passing needs the "
                  "ghost neighbour list)");
    if (hbad & 1u) return fail(SMX_ERR_INVALID, "a neighbour's local owner is not in ilist");
    for (long q = 0; q < 3L * nall; ++q) f[q] += hf[q];
    if (want_eatom) std::memcpy(eatom, p->he, sizeof(double) * inum);
    const double* o = p->hout;
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
