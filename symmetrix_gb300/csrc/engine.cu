// Engine object and C ABI (include/smx_gb300.h).
//
// Evaluation order follows MACE::compute_node_energies_forces
// (libsymmetrix/source/mace.cpp:17-64) with stages fused into GB300 kernels:
//   layer0_fwd (Y, R0, A0, M0) -> gemm H1 -> layer1_fwd (R1, Phi1) -> gemm A1 ->
//   node_tail (M1, H2, readouts, energy, seeds, reverse M1/H2) -> gemm Phi1_adj ->
//   layer1_rev (edge forces, H1_adj) -> gemm M0_adj -> layer0_rev (A0_adj, forces).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/smx_gb300.h"
#include "device.cuh"
#include "kernels.h"
#include "model.hpp"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
T* dalloc(size_t n) {
  void* p = nullptr;
  if (n == 0) n = 1;
  check(cudaMalloc(&p, n * sizeof(T)), "cudaMalloc");
  return static_cast<T*>(p);
}

}  // namespace

struct smx_engine {
  int device = 0;
  int precision = SMX_PRECISION_FP32;
  smx::HostModel hm;
  smx::DevModel dm{};
  std::vector<void*> model_mem;
  cudaStream_t stream = nullptr;
  bool keep_stages = false;

  // workspace (grow-only)
  long capN = 0, capE = 0;
  float *A0 = nullptr, *M0 = nullptr, *H1 = nullptr, *Phi1 = nullptr, *A1 = nullptr, *M1 = nullptr, *H2 = nullptr;
  float *A0_adj = nullptr, *M0_adj = nullptr, *H1_adj = nullptr, *Phi1_adj = nullptr, *A1_adj = nullptr;
  float *M1_adj = nullptr, *H2_adj = nullptr, *f1 = nullptr;
  int *first = nullptr, *ntype = nullptr, *nidx = nullptr, *ntype_e = nullptr;
  double *xyz = nullptr, *r = nullptr, *energies = nullptr, *forces = nullptr;
  int lastN = 0;

  template <typename T>
  const T* upload(const std::vector<T>& v) {
    T* p = dalloc<T>(v.size());
    if (!v.empty()) check(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
    model_mem.push_back(p);
    return p;
  }

  void load(const std::string& path) {
    hm.load_json(path);
    smx::PackedModel pm = smx::pack_model(hm);
    auto& m = dm;
    m.S = pm.S;
    m.C = pm.C;
    m.L_max = pm.L_max;
    m.nLM = pm.nLM;
    m.n_lme = pm.n_lme;
    m.n_instr = pm.n_instr;
    m.n_p = pm.n_p;
    m.nint = pm.nint;
    m.T0 = pm.T0;
    m.T1 = pm.T1;
    m.n_hidden = pm.n_hidden;
    m.h = pm.h;
    m.inv_h = static_cast<float>(1.0 / hm.spl_h);
    m.r_cut = pm.r_cut;
    m.ro2_scale = pm.ro2_scale;
    m.spl0 = reinterpret_cast<const float4*>(upload(pm.spl0));
    m.spl1 = reinterpret_cast<const float4*>(upload(pm.spl1));
    m.mono0 = upload(pm.mono0);
    for (int q = 0; q < 10; ++q) m.mono0_off[q] = q < static_cast<int>(pm.mono0_off.size()) ? pm.mono0_off[q] : pm.mono0_off.back();
    m.coef0 = upload(pm.coef0);
    m.mono1 = upload(pm.mono1);
    m.coef1 = upload(pm.coef1);
    m.H1W = upload(pm.H1W);
    m.H1W_T = upload(pm.H1W_T);
    m.cg_fwd_off = upload(pm.cg_fwd_off);
    m.cg_fwd_p = upload(pm.cg_fwd_p);
    m.cg_fwd_v = upload(pm.cg_fwd_v);
    m.cg_rev_off = upload(pm.cg_rev_off);
    m.cg_rev_lme = upload(pm.cg_rev_lme);
    m.cg_rev_v = upload(pm.cg_rev_v);
    for (int l = 0; l < 4; ++l) {
      m.lme_off[l] = pm.lme_off[l];
      m.num_e[l] = pm.num_e[l];
      m.A1W[l] = upload(pm.A1W[l]);
      m.A1W_T[l] = upload(pm.A1W_T[l]);
    }
    m.H2W_H1 = upload(pm.H2W_H1);
    m.H2W_H1_T = upload(pm.H2W_H1_T);
    m.H2W_M1 = upload(pm.H2W_M1);
    m.H2W_M1_T = upload(pm.H2W_M1_T);
    m.ro1 = upload(pm.ro1);
    m.ro2_w1 = upload(pm.ro2_w1);
    m.ro2_w2 = upload(pm.ro2_w2);
    m.e0 = upload(pm.e0);
    if (hm.has_zbl) throw std::invalid_argument("model file: ZBL pair repulsion is not supported by this build");
    if (hm.L_max != 1) throw std::invalid_argument("model file: this build supports L_max = 1 (hidden irreps 0e + 1o)");
    if (hm.A0_scaled || hm.A1_scaled)
      throw std::invalid_argument("model file: density-scaled interaction blocks are not supported by this build");
  }

  void free_workspace() {
    void* ps[] = {A0, M0, H1, Phi1, A1, M1, H2, A0_adj, M0_adj, H1_adj, Phi1_adj, A1_adj, M1_adj, H2_adj, f1,
                  first, ntype, nidx, ntype_e, xyz, r, energies, forces};
    for (void* p : ps)
      if (p) cudaFree(p);
    A0 = M0 = H1 = Phi1 = A1 = M1 = H2 = A0_adj = M0_adj = H1_adj = Phi1_adj = A1_adj = M1_adj = H2_adj = f1 = nullptr;
    first = ntype = nidx = ntype_e = nullptr;
    xyz = r = energies = forces = nullptr;
    capN = capE = 0;
  }

  void reserve(long N, long E) {
    if (N <= capN && E <= capE) return;
    const long nN = std::max(N, capN), nE = std::max(E, capE);
    free_workspace();
    const long C = dm.C;
    A0 = dalloc<float>(nN * 16 * C);
    M0 = dalloc<float>(nN * dm.nLM * C);
    H1 = dalloc<float>(nN * dm.nLM * C);
    Phi1 = dalloc<float>(nN * dm.n_lme * C);
    A1 = dalloc<float>(nN * 16 * C);
    M1 = dalloc<float>(nN * C);
    H2 = dalloc<float>(nN * C);
    A0_adj = dalloc<float>(nN * 16 * C);
    M0_adj = dalloc<float>(nN * dm.nLM * C);
    H1_adj = dalloc<float>(nN * dm.nLM * C);
    Phi1_adj = dalloc<float>(nN * dm.n_lme * C);
    A1_adj = dalloc<float>(nN * 16 * C);
    M1_adj = dalloc<float>(nN * C);
    H2_adj = dalloc<float>(nN * C);
    f1 = dalloc<float>(3 * nE);
    first = dalloc<int>(nN + 1);
    ntype = dalloc<int>(nN);
    nidx = dalloc<int>(nE);
    ntype_e = dalloc<int>(nE);
    xyz = dalloc<double>(3 * nE);
    r = dalloc<double>(nE);
    energies = dalloc<double>(nN);
    forces = dalloc<double>(3 * nE);
    capN = nN;
    capE = nE;
  }

  // x_off / y_off: float offset of the segment's first row inside a node's block
  smx::GemmSeg seg_rows(const float* X, float* Y, const float* B, int N, int rpn, int K, int ncols, long x_ns,
                        int x_off, int x_rs, long y_ns, int y_off, int y_rs) const {
    smx::GemmSeg g;
    g.X = X;
    g.Y = Y;
    g.B = B;
    g.rows = N * rpn;
    g.K = K;
    g.ncols = ncols;
    g.rpn = rpn;
    g.x_ns = x_ns;
    g.x_off = x_off;
    g.x_rs = x_rs;
    g.y_ns = y_ns;
    g.y_off = y_off;
    g.y_rs = y_rs;
    return g;
  }

  // The full forward + adjoint pass on device-resident inputs.
  void run(const smx::EdgeIn& in, double* out_e, double* out_f, cudaStream_t s) {
    const int N = in.N;
    const int C = dm.C;
    lastN = N;
    if (N == 0) return;
    smx::launch_layer0_fwd(dm, in, A0, M0, s);
    {  // H1 = M0 @ H1W[L]  (mace.cpp:397-423)
      smx::GemmBatch b{};
      for (int L = 0; L <= dm.L_max; ++L)
        b.s[b.n++] = seg_rows(M0, H1, dm.H1W + static_cast<size_t>(L) * C * C, N, 2 * L + 1, C, C,
                              static_cast<long>(dm.nLM) * C, L * L * C, C, static_cast<long>(dm.nLM) * C, L * L * C, C);
      smx::launch_gemm(b, s);
    }
    smx::launch_layer1_fwd(dm, in, H1, Phi1, s);
    {  // A1 = Phi1 @ A1W[l]  (mace.cpp:607-642)
      smx::GemmBatch b{};
      for (int l = 0; l < 4; ++l)
        if (dm.num_e[l] > 0)
          b.s[b.n++] = seg_rows(Phi1, A1, dm.A1W[l], N, 2 * l + 1, dm.num_e[l] * C, C,
                                static_cast<long>(dm.n_lme) * C, dm.lme_off[l] * C, dm.num_e[l] * C,
                                16L * C, l * l * C, C);
      smx::launch_gemm(b, s);
    }
    smx::launch_node_tail(dm, in.node_type, N, A1, H1, M1, H2, A1_adj, H1_adj, M1_adj, H2_adj, out_e, s);
    {  // Phi1_adj = A1_adj @ A1W[l]^T  (mace.cpp:644-679)
      smx::GemmBatch b{};
      for (int l = 0; l < 4; ++l)
        if (dm.num_e[l] > 0)
          b.s[b.n++] = seg_rows(A1_adj, Phi1_adj, dm.A1W_T[l], N, 2 * l + 1, C, dm.num_e[l] * C, 16L * C, l * l * C,
                                C, static_cast<long>(dm.n_lme) * C, dm.lme_off[l] * C, dm.num_e[l] * C);
      smx::launch_gemm(b, s);
    }
    smx::launch_layer1_rev(dm, in, H1, Phi1_adj, H1_adj, f1, s);
    {  // M0_adj = H1_adj @ H1W[L]^T  (mace.cpp:425-451)
      smx::GemmBatch b{};
      for (int L = 0; L <= dm.L_max; ++L)
        b.s[b.n++] = seg_rows(H1_adj, M0_adj, dm.H1W_T + static_cast<size_t>(L) * C * C, N, 2 * L + 1, C, C,
                              static_cast<long>(dm.nLM) * C, L * L * C, C, static_cast<long>(dm.nLM) * C, L * L * C, C);
      smx::launch_gemm(b, s);
    }
    smx::launch_layer0_rev(dm, in, A0, M0_adj, f1, keep_stages ? A0_adj : nullptr, out_f, s);
    check(cudaGetLastError(), "kernel launch");
  }
};

namespace {

bool is_finite_d(double v) { return std::isfinite(v); }

}  // namespace

extern "C" {

const char* smx_last_error(void) { return g_last_error.c_str(); }

smx_engine* smx_create(const char* model_path, int precision, int device) {
  if (!model_path) {
    fail(SMX_ERR_INVALID, "model_path is NULL");
    return nullptr;
  }
  if (precision != SMX_PRECISION_FP32) {
    fail(SMX_ERR_INVALID, "unsupported precision mode");
    return nullptr;
  }
  auto eng = std::make_unique<smx_engine>();
  try {
    int ndev = 0;
    check(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) throw std::invalid_argument("CUDA device index out of range");
    check(cudaSetDevice(device), "cudaSetDevice");
    eng->device = device;
    eng->precision = precision;
    check(cudaStreamCreateWithFlags(&eng->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    eng->load(model_path);
    check(cudaDeviceSynchronize(), "model upload");
  } catch (const CudaError& e) {
    fail(SMX_ERR_CUDA, e.what());
    smx_destroy(eng.release());
    return nullptr;
  } catch (const std::exception& e) {
    fail(SMX_ERR_MODEL, e.what());
    smx_destroy(eng.release());
    return nullptr;
  }
  return eng.release();
}

void smx_destroy(smx_engine* eng) {
  if (!eng) return;
  cudaSetDevice(eng->device);
  if (eng->stream) cudaStreamSynchronize(eng->stream);
  eng->free_workspace();
  for (void* p : eng->model_mem) cudaFree(p);
  if (eng->stream) cudaStreamDestroy(eng->stream);
  delete eng;
}

int smx_num_elements(const smx_engine* eng) { return eng ? eng->hm.S : -1; }
int smx_num_channels(const smx_engine* eng) { return eng ? eng->hm.C : -1; }
double smx_r_cut(const smx_engine* eng) { return eng ? eng->hm.r_cut : -1.0; }
int smx_l_max(const smx_engine* eng) { return eng ? eng->hm.l_max : -1; }
int smx_L_max(const smx_engine* eng) { return eng ? eng->hm.L_max : -1; }
int smx_num_LM(const smx_engine* eng) { return eng ? eng->hm.nLM : -1; }
int smx_atomic_numbers(const smx_engine* eng, int* out, int cap) {
  if (!eng) return -1;
  for (int q = 0; q < eng->hm.S && q < cap; ++q) out[q] = eng->hm.Z[q];
  return eng->hm.S;
}

int smx_set_option(smx_engine* eng, const char* key, long value) {
  if (!eng || !key) return fail(SMX_ERR_INVALID, "NULL argument");
  if (std::strcmp(key, "keep_stages") == 0) {
    eng->keep_stages = value != 0;
    return SMX_OK;
  }
  return fail(SMX_ERR_INVALID, std::string("unknown option '") + key + "'");
}

int smx_compute_node_energies_forces(smx_engine* eng, int num_nodes, const int* node_types, const int* num_neigh,
                                     const int* neigh_indices, const int* neigh_types, long num_edges,
                                     const double* xyz, const double* r, double* node_energies,
                                     double* node_forces) {
  if (!eng) return fail(SMX_ERR_INVALID, "engine is NULL");
  if (num_nodes < 0 || num_edges < 0) return fail(SMX_ERR_INVALID, "negative size");
  if (num_nodes > 0 && (!node_types || !num_neigh || !node_energies))
    return fail(SMX_ERR_INVALID, "NULL node array");
  if (num_edges > 0 && (!neigh_indices || !neigh_types || !xyz || !r || !node_forces))
    return fail(SMX_ERR_INVALID, "NULL edge array");
  const int S = eng->hm.S;
  const double rc = eng->hm.r_cut;
  // host-side validation and CSR offsets (the reference trusts its caller here)
  std::vector<int> first(static_cast<size_t>(num_nodes) + 1, 0);
  for (int i = 0; i < num_nodes; ++i) {
    if (node_types[i] < 0 || node_types[i] >= S) return fail(SMX_ERR_INVALID, "node_types out of range");
    if (num_neigh[i] < 0) return fail(SMX_ERR_INVALID, "negative num_neigh");
    first[i + 1] = first[i] + num_neigh[i];
  }
  if (first[num_nodes] != num_edges) return fail(SMX_ERR_INVALID, "sum(num_neigh) != num_edges");
  for (long e = 0; e < num_edges; ++e) {
    if (neigh_indices[e] < 0 || neigh_indices[e] >= num_nodes)
      return fail(SMX_ERR_INVALID, "neigh_indices out of range (must be < num_nodes)");
    if (neigh_types[e] < 0 || neigh_types[e] >= S) return fail(SMX_ERR_INVALID, "neigh_types out of range");
    if (!(r[e] > 0.0 && r[e] < rc) || !is_finite_d(xyz[3 * e]) || !is_finite_d(xyz[3 * e + 1]) || !is_finite_d(xyz[3 * e + 2]))
      return fail(SMX_ERR_INVALID, "edge length outside (0, r_cut) or non-finite edge vector");
  }
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    eng->reserve(num_nodes, num_edges);
    cudaStream_t s = eng->stream;
    check(cudaMemcpyAsync(eng->first, first.data(), sizeof(int) * (num_nodes + 1), cudaMemcpyHostToDevice, s), "H2D");
    if (num_nodes > 0)
      check(cudaMemcpyAsync(eng->ntype, node_types, sizeof(int) * num_nodes, cudaMemcpyHostToDevice, s), "H2D");
    if (num_edges > 0) {
      check(cudaMemcpyAsync(eng->nidx, neigh_indices, sizeof(int) * num_edges, cudaMemcpyHostToDevice, s), "H2D");
      check(cudaMemcpyAsync(eng->ntype_e, neigh_types, sizeof(int) * num_edges, cudaMemcpyHostToDevice, s), "H2D");
      check(cudaMemcpyAsync(eng->xyz, xyz, sizeof(double) * 3 * num_edges, cudaMemcpyHostToDevice, s), "H2D");
      check(cudaMemcpyAsync(eng->r, r, sizeof(double) * num_edges, cudaMemcpyHostToDevice, s), "H2D");
    }
    smx::EdgeIn in{eng->first, eng->ntype, eng->nidx, eng->ntype_e, eng->xyz, eng->r, num_nodes};
    eng->run(in, eng->energies, eng->forces, s);
    if (num_nodes > 0)
      check(cudaMemcpyAsync(node_energies, eng->energies, sizeof(double) * num_nodes, cudaMemcpyDeviceToHost, s), "D2H");
    if (num_edges > 0)
      check(cudaMemcpyAsync(node_forces, eng->forces, sizeof(double) * 3 * num_edges, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "evaluation");
  } catch (const std::exception& e) {
    return fail(SMX_ERR_CUDA, e.what());
  }
  return SMX_OK;
}

int smx_compute_node_energies_forces_device(smx_engine* eng, int num_nodes, const int* node_types,
                                            const int* num_neigh, const int* neigh_indices, const int* neigh_types,
                                            long num_edges, const double* xyz, const double* r,
                                            double* node_energies, double* node_forces, void* stream) {
  if (!eng) return fail(SMX_ERR_INVALID, "engine is NULL");
  if (num_nodes < 0 || num_edges < 0) return fail(SMX_ERR_INVALID, "negative size");
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    eng->reserve(num_nodes, num_edges);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : eng->stream;
    if (num_nodes > 0) smx::launch_scan_first(num_neigh, num_nodes, eng->first, s);
    smx::EdgeIn in{eng->first, node_types, neigh_indices, neigh_types, xyz, r, num_nodes};
    eng->run(in, node_energies, node_forces, s);
  } catch (const std::exception& e) {
    return fail(SMX_ERR_CUDA, e.what());
  }
  return SMX_OK;
}

long smx_get_stage(smx_engine* eng, const char* name, double* out, long cap) {
  if (!eng || !name) return -1;
  const long N = eng->lastN, C = eng->dm.C;
  const float* src = nullptr;
  long n = 0;
  const std::string s(name);
  if (s == "A0") { src = eng->A0; n = N * 16 * C; }
  else if (s == "M0") { src = eng->M0; n = N * eng->dm.nLM * C; }
  else if (s == "H1") { src = eng->H1; n = N * eng->dm.nLM * C; }
  else if (s == "Phi1") { src = eng->Phi1; n = N * eng->dm.n_lme * C; }
  else if (s == "A1") { src = eng->A1; n = N * 16 * C; }
  else if (s == "M1") { src = eng->M1; n = N * C; }
  else if (s == "H2") { src = eng->H2; n = N * C; }
  else if (s == "A0_adj") { src = eng->keep_stages ? eng->A0_adj : nullptr; n = N * 16 * C; }
  else if (s == "M0_adj") { src = eng->M0_adj; n = N * eng->dm.nLM * C; }
  else if (s == "H1_adj") { src = eng->H1_adj; n = N * eng->dm.nLM * C; }
  else if (s == "Phi1_adj") { src = eng->Phi1_adj; n = N * eng->dm.n_lme * C; }
  else if (s == "A1_adj") { src = eng->A1_adj; n = N * 16 * C; }
  else if (s == "M1_adj") { src = eng->M1_adj; n = N * C; }
  else if (s == "H2_adj") { src = eng->H2_adj; n = N * C; }
  else return -1;
  if (!src) return fail(SMX_ERR_INVALID, "stage not kept (set keep_stages)") ? -1 : -1;
  if (out && cap > 0 && n > 0) {
    std::vector<float> tmp(static_cast<size_t>(n));
    cudaSetDevice(eng->device);
    cudaStreamSynchronize(eng->stream);
    if (cudaMemcpy(tmp.data(), src, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    for (long q = 0; q < n && q < cap; ++q) out[q] = tmp[q];
  }
  return n;
}

}  // extern "C"
