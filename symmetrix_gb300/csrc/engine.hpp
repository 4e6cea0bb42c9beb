// Engine object shared by the C ABI translation units (engine.cu, md.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/smx_gb300.h"
#include "device.cuh"
#include "kernels.h"
#include "model.hpp"

namespace smx {
int fail(int code, const std::string& msg);
struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
inline void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}
template <typename T>
T* dalloc(size_t n) {
  void* p = nullptr;
  if (n == 0) n = 1;
  check(cudaMalloc(&p, n * sizeof(T)), "cudaMalloc");
  return static_cast<T*>(p);
}
}  // namespace smx

using smx::check;
using smx::dalloc;
using smx::CudaError;

struct smx_engine {
  int device = 0;
  int precision = SMX_PRECISION_FP32;
  smx::HostModel hm;
  smx::DevModel dm{};
  std::vector<void*> model_mem;
  cudaStream_t stream = nullptr;
  bool keep_stages = false;
  // optional per-stage CUDA-event timing of the last evaluation
  static constexpr int kStages = 9;
  bool profile = false;
  cudaEvent_t ev[kStages + 1] = {};
  float stage_ms[kStages] = {};
  cudaStream_t prof_stream = nullptr;

  // workspace (grow-only)
  long capN = 0, capE = 0;
  float *A0 = nullptr, *M0 = nullptr, *H1 = nullptr, *Phi1 = nullptr, *A1 = nullptr, *M1 = nullptr, *H2 = nullptr;
  float *A0_adj = nullptr, *M0_adj = nullptr, *H1_adj = nullptr, *Phi1_adj = nullptr, *A1_adj = nullptr;
  float *M1_adj = nullptr, *H2_adj = nullptr;
  double* f1 = nullptr;  // layer-1 edge forces (float64 accumulation)
  float* zbl_e = nullptr;  // per-node ZBL energy
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
    m.poly_canon = pm.poly_canon;
    m.n_hidden = pm.n_hidden;
    m.h = pm.h;
    m.inv_h = static_cast<float>(1.0 / hm.spl_h);
    m.r_cut = pm.r_cut;
    m.ro2_scale = pm.ro2_scale;
    m.spl0 = reinterpret_cast<const float4*>(upload(pm.spl0));
    m.spl1 = reinterpret_cast<const float4*>(upload(pm.spl1));
    m.spl1_fwd = reinterpret_cast<const float4*>(upload(pm.spl1_fwd));
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
    m.has_zbl = pm.has_zbl;
    m.zbl_p = pm.zbl_p;
    for (int q = 0; q < 4; ++q) m.zbl_c[q] = pm.zbl_c[q];
    m.zbl_pair = pm.has_zbl ? reinterpret_cast<const float4*>(upload(pm.zbl_pair)) : nullptr;
    check(smx::init_edge_kernels(dm), "cudaFuncSetAttribute");
    if (hm.L_max != 1) throw std::invalid_argument("model file: this build supports L_max = 1 (hidden irreps 0e + 1o)");
    if (hm.A0_scaled || hm.A1_scaled)
      throw std::invalid_argument("model file: density-scaled interaction blocks are not supported by this build");
  }

  void free_workspace() {
    void* ps[] = {A0, M0, H1, Phi1, A1, M1, H2, A0_adj, M0_adj, H1_adj, Phi1_adj, A1_adj, M1_adj, H2_adj, f1,
                  first, ntype, nidx, ntype_e, xyz, r, energies, forces};
    for (void* p : ps)
      if (p) cudaFree(p);
    A0 = M0 = H1 = Phi1 = A1 = M1 = H2 = A0_adj = M0_adj = H1_adj = Phi1_adj = A1_adj = M1_adj = H2_adj = nullptr;
    f1 = nullptr;
    if (zbl_e) cudaFree(zbl_e);
    zbl_e = nullptr;
    first = ntype = nidx = ntype_e = nullptr;
    xyz = r = energies = forces = nullptr;
    capN = capE = 0;
  }

  void reserve(long N, long E) {
    if (first && N <= capN && E <= capE) return;
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
    f1 = dalloc<double>(3 * nE);
    zbl_e = dalloc<float>(nN);
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

  void mark(int q, cudaStream_t s) {
    if (profile) check(cudaEventRecord(ev[q], s), "cudaEventRecord");
  }

  // The full forward + adjoint pass on device-resident inputs.
  void run(const smx::EdgeIn& in, double* out_e, double* out_f, cudaStream_t s) {
    const int N = in.N;
    const int C = dm.C;
    lastN = N;
    if (N == 0) return;
    if (profile && !ev[0])
      for (auto& e : ev) check(cudaEventCreate(&e), "cudaEventCreate");
    prof_stream = s;
    mark(0, s);
    smx::launch_layer0_fwd(dm, in, A0, M0, dm.has_zbl ? zbl_e : nullptr, s);
    mark(1, s);
    {  // H1 = M0 @ H1W[L]  (mace.cpp:397-423)
      smx::GemmBatch b{};
      for (int L = 0; L <= dm.L_max; ++L)
        b.s[b.n++] = seg_rows(M0, H1, dm.H1W + static_cast<size_t>(L) * C * C, N, 2 * L + 1, C, C,
                              static_cast<long>(dm.nLM) * C, L * L * C, C, static_cast<long>(dm.nLM) * C, L * L * C, C);
      smx::launch_gemm(b, s);
    }
    mark(2, s);
    smx::launch_layer1_fwd(dm, in, H1, Phi1, s);
    mark(3, s);
    {  // A1 = Phi1 @ A1W[l]  (mace.cpp:607-642)
      smx::GemmBatch b{};
      for (int l = 0; l < 4; ++l)
        if (dm.num_e[l] > 0)
          b.s[b.n++] = seg_rows(Phi1, A1, dm.A1W[l], N, 2 * l + 1, dm.num_e[l] * C, C,
                                static_cast<long>(dm.n_lme) * C, dm.lme_off[l] * C, dm.num_e[l] * C,
                                16L * C, l * l * C, C);
      smx::launch_gemm(b, s);
    }
    mark(4, s);
    smx::launch_node_tail(dm, in.node_type, N, A1, H1, M1, H2, A1_adj, H1_adj, M1_adj, H2_adj,
                          dm.has_zbl ? zbl_e : nullptr, out_e, s);
    mark(5, s);
    {  // Phi1_adj = A1_adj @ A1W[l]^T  (mace.cpp:644-679)
      smx::GemmBatch b{};
      for (int l = 0; l < 4; ++l)
        if (dm.num_e[l] > 0)
          b.s[b.n++] = seg_rows(A1_adj, Phi1_adj, dm.A1W_T[l], N, 2 * l + 1, C, dm.num_e[l] * C, 16L * C, l * l * C,
                                C, static_cast<long>(dm.n_lme) * C, dm.lme_off[l] * C, dm.num_e[l] * C);
      smx::launch_gemm(b, s);
    }
    mark(6, s);
    smx::launch_layer1_rev(dm, in, H1, Phi1_adj, H1_adj, f1, s);
    mark(7, s);
    {  // M0_adj = H1_adj @ H1W[L]^T  (mace.cpp:425-451)
      smx::GemmBatch b{};
      for (int L = 0; L <= dm.L_max; ++L)
        b.s[b.n++] = seg_rows(H1_adj, M0_adj, dm.H1W_T + static_cast<size_t>(L) * C * C, N, 2 * L + 1, C, C,
                              static_cast<long>(dm.nLM) * C, L * L * C, C, static_cast<long>(dm.nLM) * C, L * L * C, C);
      smx::launch_gemm(b, s);
    }
    mark(8, s);
    smx::launch_layer0_rev(dm, in, A0, M0_adj, f1, A0_adj, out_f, s);
    mark(9, s);
    check(cudaGetLastError(), "kernel launch");
  }
};

