// LAMMPS pair-style adapter: one compute() of pair_style symmetrix/mace in its
// no-domain-decomposition mode (pair_symmetrix/pair_symmetrix_mace.cpp:242-372), with
// the neighbour filtering, the evaluation and the force scatter on the GPU.
//
// The caller passes LAMMPS's own arrays: the full neighbour list (inum, ilist,
// numneigh, firstneigh, NEIGHMASK), positions x[nall][3] of local and ghost atoms,
// atom types, local_of[j] = atom->map(atom->tag[j]) (the local owner of a ghost) and
// the LAMMPS type -> model species map.  The list topology is uploaded when the
// caller says it changed (LAMMPS re-neighbouring); every call uploads only x.
//
// Per call on the device: candidates with 0 < r^2 < r_cut^2 become the engine's CSR
// edges (centre = node ii, neighbour = node of local_of[j], xyz = x_j - x_i), the
// engine evaluates, forces are scattered F_i -= f_e, F_local_of[j] += f_e (float64
// atomics: the summation order, hence the last bits, may differ between runs), and
// energy and virial sum_e xyz_a f_b are reduced on the device.
#include <cuda_runtime.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.hpp"

using smx::fail;

namespace {

__global__ void k_pair_count(int inum, const int* __restrict__ cand_off, const int* __restrict__ cand_j,
                             const int* __restrict__ ilist, const double* __restrict__ x, double rc2,
                             int* __restrict__ num_neigh) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= inum) return;
  const int i = ilist[ii];
  const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  int n = 0;
  for (int c = cand_off[ii]; c < cand_off[ii + 1]; ++c) {
    const int j = cand_j[c];
    const double dx = x[3 * j] - xi, dy = x[3 * j + 1] - yi, dz = x[3 * j + 2] - zi;
    const double r2 = dx * dx + dy * dy + dz * dz;
    n += (r2 < rc2 && r2 > 0.0) ? 1 : 0;
  }
  num_neigh[ii] = n;
}

__global__ void k_pair_fill(int inum, const int* __restrict__ cand_off, const int* __restrict__ cand_j,
                            const int* __restrict__ ilist, const double* __restrict__ x, double rc2,
                            const int* __restrict__ first, const int* __restrict__ mtype,
                            const int* __restrict__ local_of, const int* __restrict__ node_of_local,
                            int* __restrict__ node_type, int* __restrict__ nidx, int* __restrict__ ntype_e,
                            double* __restrict__ xyz, double* __restrict__ r, int* __restrict__ nbr_local,
                            unsigned* __restrict__ bad) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= inum) return;
  const int i = ilist[ii];
  node_type[ii] = mtype[i];
  const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  int e = first[ii];
  for (int c = cand_off[ii]; c < cand_off[ii + 1]; ++c) {
    const int j = cand_j[c];
    const double dx = x[3 * j] - xi, dy = x[3 * j + 1] - yi, dz = x[3 * j + 2] - zi;
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (!(r2 < rc2 && r2 > 0.0)) continue;
    const int jl = local_of[j];
    const int node = node_of_local[jl];
    if (node < 0) atomicOr(bad, 1u);
    nidx[e] = node < 0 ? 0 : node;
    ntype_e[e] = mtype[j];
    xyz[3 * e] = dx;
    xyz[3 * e + 1] = dy;
    xyz[3 * e + 2] = dz;
    r[e] = sqrt(r2);
    nbr_local[e] = jl;
    ++e;
  }
}

__global__ void k_pair_scatter(int inum, const int* __restrict__ first, const int* __restrict__ ilist,
                               const int* __restrict__ nbr_local, const double* __restrict__ fe,
                               double* __restrict__ f) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= inum) return;
  double sx = 0.0, sy = 0.0, sz = 0.0;
  for (int e = first[ii]; e < first[ii + 1]; ++e) {
    const double fx = fe[3 * e], fy = fe[3 * e + 1], fz = fe[3 * e + 2];
    sx += fx;
    sy += fy;
    sz += fz;
    const int j = nbr_local[e];
    atomicAdd(f + 3 * j, fx);
    atomicAdd(f + 3 * j + 1, fy);
    atomicAdd(f + 3 * j + 2, fz);
  }
  const int i = ilist[ii];
  atomicAdd(f + 3 * i, -sx);
  atomicAdd(f + 3 * i + 1, -sy);
  atomicAdd(f + 3 * i + 2, -sz);
}

constexpr int kReduceBlocks = 64;

}  // namespace

struct smx_pair {
  smx_engine* eng = nullptr;
  int inum = 0, nall = 0, ncand = 0;
  // topology (uploaded on re-neighbouring)
  int *ilist = nullptr, *cand_off = nullptr, *cand_j = nullptr, *mtype = nullptr, *local_of = nullptr;
  int *node_of_local = nullptr, *num_neigh = nullptr, *nbr_local = nullptr;
  double *x = nullptr, *f = nullptr, *partial = nullptr, *out = nullptr;
  unsigned* bad = nullptr;
  long cap_nall = 0, cap_inum = 0, cap_cand = 0;
  std::vector<double> h_out = std::vector<double>(10);

  void free_all() {
    void* ps[] = {ilist, cand_off, cand_j, mtype, local_of, node_of_local, num_neigh, nbr_local, x, f, partial, out,
                  bad};
    for (void* p : ps)
      if (p) cudaFree(p);
    ilist = cand_off = cand_j = mtype = local_of = node_of_local = num_neigh = nbr_local = nullptr;
    x = f = partial = out = nullptr;
    bad = nullptr;
    cap_nall = cap_inum = cap_cand = 0;
  }

  void reserve(int ni, int na, int nc) {
    if (ni <= cap_inum && na <= cap_nall && nc <= cap_cand && x) return;
    free_all();
    cap_inum = std::max(ni, 1);
    cap_nall = std::max(na, 1);
    cap_cand = std::max(nc, 1);
    ilist = dalloc<int>(cap_inum);
    cand_off = dalloc<int>(cap_inum + 1);
    num_neigh = dalloc<int>(cap_inum);
    cand_j = dalloc<int>(cap_cand);
    nbr_local = dalloc<int>(cap_cand);
    mtype = dalloc<int>(cap_nall);
    local_of = dalloc<int>(cap_nall);
    node_of_local = dalloc<int>(cap_nall);
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
  delete p;
}

int smx_pair_compute(smx_pair* p, int inum, int nall, const int* ilist, const int* numneigh,
                     const int* const* firstneigh, int neighmask, int neigh_changed, const double* x, const int* type,
                     const int* local_of, const int* mace_types, int ntypes, int eflag_global, int eflag_atom,
                     int vflag_global, double* f, double* eng_vdwl, double* eatom, double* virial) {
  if (!p) return fail(SMX_ERR_INVALID, "pair adapter is NULL");
  if (inum < 0 || nall < inum) return fail(SMX_ERR_INVALID, "need 0 <= inum <= nall");
  if (nall > 0 && (!x || !f)) return fail(SMX_ERR_INVALID, "NULL x or f");
  smx_engine* eng = p->eng;
  const int S = eng->hm.S;
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    cudaStream_t s = eng->stream;
    if (neigh_changed || inum != p->inum || nall != p->nall) {
      if (inum > 0 && (!ilist || !numneigh || !firstneigh || !type || !local_of || !mace_types))
        return fail(SMX_ERR_INVALID, "NULL neighbour-list or atom array");
      std::vector<int> off(static_cast<size_t>(inum) + 1, 0), cj, mt(nall), nol(nall, -1);
      for (int ii = 0; ii < inum; ++ii) {
        if (ilist[ii] < 0 || ilist[ii] >= nall) return fail(SMX_ERR_INVALID, "ilist entry out of range");
        if (numneigh[ilist[ii]] < 0) return fail(SMX_ERR_INVALID, "negative numneigh");
        off[ii + 1] = off[ii] + numneigh[ilist[ii]];
        nol[ilist[ii]] = ii;
      }
      cj.resize(off[inum]);
      for (int ii = 0; ii < inum; ++ii) {
        const int i = ilist[ii];
        for (int jj = 0; jj < numneigh[i]; ++jj) {
          const int j = firstneigh[i][jj] & neighmask;
          if (j < 0 || j >= nall) return fail(SMX_ERR_INVALID, "neighbour index out of range");
          cj[off[ii] + jj] = j;
        }
      }
      for (int a = 0; a < nall; ++a) {
        if (type[a] < 1 || type[a] > ntypes) return fail(SMX_ERR_INVALID, "atom type out of range");
        mt[a] = mace_types[type[a] - 1];
        if (mt[a] < 0 || mt[a] >= S) return fail(SMX_ERR_INVALID, "mace_types entry out of range");
        if (local_of[a] < 0 || local_of[a] >= nall) return fail(SMX_ERR_INVALID, "local_of entry out of range");
      }
      p->reserve(inum, nall, off[inum]);
      eng->reserve(inum, off[inum]);
      if (inum > 0) {
        check(cudaMemcpyAsync(p->ilist, ilist, sizeof(int) * inum, cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(p->cand_off, off.data(), sizeof(int) * (inum + 1), cudaMemcpyHostToDevice, s), "H2D");
      }
      if (!cj.empty())
        check(cudaMemcpyAsync(p->cand_j, cj.data(), sizeof(int) * cj.size(), cudaMemcpyHostToDevice, s), "H2D");
      if (nall > 0) {
        check(cudaMemcpyAsync(p->mtype, mt.data(), sizeof(int) * nall, cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(p->local_of, local_of, sizeof(int) * nall, cudaMemcpyHostToDevice, s), "H2D");
        check(cudaMemcpyAsync(p->node_of_local, nol.data(), sizeof(int) * nall, cudaMemcpyHostToDevice, s), "H2D");
      }
      check(cudaStreamSynchronize(s), "topology upload");  // host vectors go out of scope
      p->inum = inum;
      p->nall = nall;
      p->ncand = off[inum];
    }
    if (inum == 0) return SMX_OK;
    const double rc = eng->hm.r_cut;
    check(cudaMemcpyAsync(p->x, x, sizeof(double) * 3 * nall, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemsetAsync(p->f, 0, sizeof(double) * 3 * nall, s), "memset");
    check(cudaMemsetAsync(p->bad, 0, sizeof(unsigned), s), "memset");
    const int nb = smx::ceil_div(inum, 128);
    k_pair_count<<<nb, 128, 0, s>>>(inum, p->cand_off, p->cand_j, p->ilist, p->x, rc * rc, p->num_neigh);
    smx::launch_scan_first(p->num_neigh, inum, eng->first, s);
    k_pair_fill<<<nb, 128, 0, s>>>(inum, p->cand_off, p->cand_j, p->ilist, p->x, rc * rc, eng->first, p->mtype,
                                   p->local_of, p->node_of_local, eng->ntype, eng->nidx, eng->ntype_e, eng->xyz,
                                   eng->r, p->nbr_local, p->bad);
    smx::EdgeIn in{eng->first, eng->ntype, eng->nidx, eng->ntype_e, eng->xyz, eng->r, inum};
    eng->run(in, eng->energies, eng->forces, s);
    k_pair_scatter<<<nb, 128, 0, s>>>(inum, eng->first, p->ilist, p->nbr_local, eng->forces, p->f);
    smx::launch_reduce(inum, eng->first, eng->energies, eng->xyz, eng->forces, p->partial, kReduceBlocks, p->out, s);
    std::vector<double> hf(static_cast<size_t>(3) * nall);
    unsigned hbad = 0;
    check(cudaMemcpyAsync(hf.data(), p->f, sizeof(double) * 3 * nall, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaMemcpyAsync(p->h_out.data(), p->out, sizeof(double) * 10, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaMemcpyAsync(&hbad, p->bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "D2H");
    if (eflag_atom && eatom)
      check(cudaMemcpyAsync(eatom, eng->energies, sizeof(double) * inum, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "pair compute");
    if (eng->take_status() != SMX_OK) return fail(SMX_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
    if (hbad) return fail(SMX_ERR_INVALID, "a neighbour's local owner is not in ilist");
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

}  // extern "C"
