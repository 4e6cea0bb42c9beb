// Engine object shared by the C ABI translation units (engine.cu, md.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
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
// float -> bf16 bit pattern, round to nearest even (NaN kept quiet)
inline uint16_t bf16_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
  u += 0x7fffu + ((u >> 16) & 1u);
  return static_cast<uint16_t>(u >> 16);
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
  // status word of the bounded device waits (mapped pinned host memory: the host
  // reads it after a synchronisation without a copy)
  unsigned* status_host = nullptr;
  unsigned* status_dev = nullptr;
  // flags of the device-side input check of the host-pointer call (mapped, as above)
  unsigned* check_host = nullptr;
  unsigned* check_dev = nullptr;
  // precision form: bf16 B operands (K contiguous) of the tensor-core GEMMs
  // (K contiguous, split_wterms(tc_terms) bf16 split terms concatenated along K: see tc_operand)
  const __nv_bfloat16 *W_H1 = nullptr, *W_M0adj = nullptr, *W_A1[4] = {}, *W_Phi1adj[4] = {};
  bool tc_H1 = false, tc_A1[4] = {}, tc_Phi1adj[4] = {};
  // 1: bf16 operands; 2: weights split hi + lo (x_hi W_hi + x_hi W_lo); 3: both
  // split (x_hi W_hi + x_lo W_hi + x_hi W_lo: close to float32 operand precision)
  int tc_terms = 3;
  std::vector<float> hw_H1W, hw_H1W_T, hw_A1W[4], hw_A1W_T[4];  // float32 host copies
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
  smx::fix64* H1_adj_fx = nullptr;  // H1_adj accumulator (fixed point: order-independent sums)
  // precision form: bf16 GEMM operands (M0 and H1_adj as [N*nLM][C]; Phi1 and A1_adj
  // regrouped per l as [N*(2l+1)][n_eta*C] and [N*(2l+1)][C])
  __nv_bfloat16 *M0_bf = nullptr, *Phi1_bf = nullptr, *A1adj_bf = nullptr, *H1adj_bf = nullptr;
  float* zbl_e = nullptr;  // per-node ZBL energy
  int *first = nullptr, *ntype = nullptr, *nidx = nullptr, *ntype_e = nullptr;
  int* atom_order = nullptr;  // centre atoms sorted by species (when species_order is on), [2][capN]
  int* nneigh = nullptr;      // num_neigh of the host-pointer call
  double *xyz = nullptr, *r = nullptr, *energies = nullptr, *forces = nullptr;
  // nodes of the last evaluation: all of them (layer 0) and the layer-1 ones (fewer when
  // the trailing nodes were a halo)
  int lastN = 0, lastN1 = 0;
  long lastE = 0;                  // edges of the last host- or device-pointer call or stage call
  bool evaluated = false;          // the workspace holds the stages of an evaluation
  bool M0_kept = false, Phi1_kept = false, A1adj_kept = false;  // float32 rows written by it

  // B operand of a tensor-core GEMM from a row-major float [nrows][K] matrix: row n
  // holds (W_hi) for 1 split product, (W_hi | W_lo) for 2 or 3, W_lo = bf16(W - W_hi)
  // (see write_split).
  const __nv_bfloat16* tc_operand(const std::vector<float>& W, int nrows, int K) {
    const int WT = smx::split_wterms(tc_terms);
    std::vector<uint16_t> b(static_cast<size_t>(nrows) * K * WT);
    for (int n = 0; n < nrows; ++n)
      for (int k = 0; k < K; ++k) {
        const float w = W[static_cast<size_t>(n) * K + k];
        const uint16_t hi = smx::bf16_bits(w);
        uint32_t hu = static_cast<uint32_t>(hi) << 16;
        float hf;
        std::memcpy(&hf, &hu, 4);
        const uint16_t lo = smx::bf16_bits(w - hf);
        for (int t = 0; t < WT; ++t) b[(static_cast<size_t>(n) * WT + t) * K + k] = t == 0 ? hi : lo;
      }
    return reinterpret_cast<const __nv_bfloat16*>(upload(b));
  }

  void setup_tc_weights() {
    const int C = dm.C;
    if (tc_H1) {
      W_H1 = tc_operand(hw_H1W_T, 2 * C, C);   // [L][k'][k]: B of H1 = M0 . H1W[L]
      W_M0adj = tc_operand(hw_H1W, 2 * C, C);  // [L][k][k']: B of M0_adj = H1_adj . H1W[L]^T
    }
    for (int l = 0; l < 4; ++l) {
      if (tc_A1[l]) W_A1[l] = tc_operand(hw_A1W_T[l], C, dm.num_e[l] * C);             // [k'][e k]
      if (tc_Phi1adj[l]) W_Phi1adj[l] = tc_operand(hw_A1W[l], dm.num_e[l] * C, C);     // [e k][k']
    }
  }

  template <typename T>
  const T* upload(const std::vector<T>& v) {
    T* p = dalloc<T>(v.size());
    if (!v.empty()) check(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
    model_mem.push_back(p);
    return p;
  }

  void load(const std::string& path) {
    smx::PackedModel pm;
    smx::load_model(path, hm, pm);
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
    {  // forward table padded to its longest row (up to 8 terms): independent loads
      const int nr = static_cast<int>(pm.cg_fwd_off.size()) - 1;
      int kp = 0;
      for (int r = 0; r < nr; ++r) kp = std::max(kp, pm.cg_fwd_off[r + 1] - pm.cg_fwd_off[r]);
      m.cg_fwd_pad = nullptr;
      m.cg_fwd_kp = 0;
      if (nr > 0 && kp >= 1 && kp <= 8) {
        std::vector<int> pad(static_cast<size_t>(2) * kp * nr, 0);
        for (int r = 0; r < nr; ++r)
          for (int q = pm.cg_fwd_off[r], t = 0; q < pm.cg_fwd_off[r + 1]; ++q, ++t) {
            float v = pm.cg_fwd_v[q];
            int bits;
            std::memcpy(&bits, &v, sizeof(bits));
            pad[2 * (static_cast<size_t>(r) * kp + t)] = pm.cg_fwd_p[q];
            pad[2 * (static_cast<size_t>(r) * kp + t) + 1] = bits;
          }
        m.cg_fwd_pad = reinterpret_cast<const int2*>(upload(pad));
        m.cg_fwd_kp = kp;
      }
      cg_fwd_pad_keep = m.cg_fwd_pad;
      cg_fwd_kp_keep = m.cg_fwd_kp;
    }
    {  // two-term padded copy: the adjoint kernels then gather g with independent loads
      const int np = static_cast<int>(pm.cg_rev_off.size()) - 1;
      bool fits = np > 0;
      for (int p = 0; p < np && fits; ++p) fits = pm.cg_rev_off[p + 1] - pm.cg_rev_off[p] <= 2;
      m.cg_rev_pad = nullptr;
      if (fits) {
        std::vector<int> pad(static_cast<size_t>(4) * np, 0);
        for (int p = 0; p < np; ++p)
          for (int q = pm.cg_rev_off[p], t = 0; q < pm.cg_rev_off[p + 1]; ++q, ++t) {
            float v = pm.cg_rev_v[q];
            int bits;
            std::memcpy(&bits, &v, sizeof(bits));
            pad[4 * p + 2 * t] = pm.cg_rev_lme[q];
            pad[4 * p + 2 * t + 1] = bits;
          }
        m.cg_rev_pad = reinterpret_cast<const int2*>(upload(pad));
      }
      cg_rev_pad_keep = m.cg_rev_pad;
    }
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
    m.op_m0 = m.op_phi1 = m.op_a1adj = nullptr;
    m.tc_terms = tc_terms;
    // two blocks per node (half the channels each) let two L_max = 2 layer-1 blocks share
    // an SM: one computes while the other waits at a barrier
    l2_split_max = (pm.L_max == 2 && pm.C >= 64) ? 2 : 1;
    m.l2_split = l2_split_max;
    m.f1_stride = 0;
    m.zbl_p = pm.zbl_p;
    for (int q = 0; q < 4; ++q) m.zbl_c[q] = pm.zbl_c[q];
    m.zbl_pair = pm.has_zbl ? reinterpret_cast<const float4*>(upload(pm.zbl_pair)) : nullptr;
    for (int layer = 0; layer < 2; ++layer) {  // density-normalised interaction blocks
      m.dens_spl[layer] =
          pm.dens_scaled[layer] ? reinterpret_cast<const float4*>(upload(pm.dens_spl[layer])) : nullptr;
      m.dens_nint[layer] = pm.dens_nint[layer];
      m.dens_h[layer] = pm.dens_h[layer];
      m.dens_inv_h[layer] = pm.dens_scaled[layer] ? 1.0f / pm.dens_h[layer] : 0.0f;
      m.dens_s[layer] = m.dens_c[layer] = nullptr;
    }
    check(smx::init_edge_kernels(dm), "cudaFuncSetAttribute");
    {  // persistent grids of the per-atom kernels: resident blocks per SM x SMs
      int* sc = dalloc<int>(2);
      model_mem.push_back(sc);
      check(cudaMemset(sc, 0, 2 * sizeof(int)), "cudaMemset");
      m.sched = sc;
      m.status = status_dev;  // bounded waits inside the edge kernels report here
      int nsm = 0, per_sm[smx::kAkCount] = {};
      check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");
      smx::layer0_residency(m, per_sm);
      smx::layer1_residency(m, per_sm);
      smx::node_tail_residency(m, per_sm);
      check(cudaGetLastError(), "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
      for (int k = 0; k < smx::kAkCount; ++k) {
        pfull[k] = per_sm[k] * nsm;
        m.pgrid[k] = sched_force == 1 ? pfull[k] : 0;
      }
    }
    if (precision == SMX_PRECISION_BF16) {
      check(smx::init_umma_kernels(), "cudaFuncSetAttribute");
      const int C = pm.C;
      // (three split products, the most the tc_terms option allows)
      tc_H1 = smx::umma_supported(C, C, 3) && pm.L_max == 1;
      for (int l = 0; l < 4; ++l) {
        if (pm.num_e[l] == 0) continue;
        tc_A1[l] = smx::umma_supported(pm.num_e[l] * C, C, 3);
        tc_Phi1adj[l] = smx::umma_supported(C, C, 3);
      }
      hw_H1W = pm.H1W;
      hw_H1W_T = pm.H1W_T;
      for (int l = 0; l < 4; ++l) {
        hw_A1W[l] = pm.A1W[l];
        hw_A1W_T[l] = pm.A1W_T[l];
      }
      setup_tc_weights();
    }
    if (hm.L_max == 2 && hm.C > 128)
      throw std::invalid_argument("model file: L_max = 2 models are supported up to 128 channels");

  }

  void free_workspace() {
    void* ps[] = {A0, M0, H1, Phi1, A1, M1, H2, A0_adj, M0_adj, H1_adj, Phi1_adj, A1_adj, M1_adj, H2_adj, f1,
                  first, ntype, nidx, ntype_e, xyz, r, energies, forces, M0_bf, Phi1_bf, A1adj_bf, H1adj_bf,
                  atom_order, nneigh};
    for (void* p : ps)
      if (p) cudaFree(p);
    A0 = M0 = H1 = Phi1 = A1 = M1 = H2 = A0_adj = M0_adj = H1_adj = Phi1_adj = A1_adj = M1_adj = H2_adj = nullptr;
    M0_bf = Phi1_bf = A1adj_bf = H1adj_bf = nullptr;
    dm.op_m0 = dm.op_phi1 = dm.op_a1adj = nullptr;
    for (int layer = 0; layer < 2; ++layer) {
      if (dm.dens_s[layer]) cudaFree(dm.dens_s[layer]);
      if (dm.dens_c[layer]) cudaFree(dm.dens_c[layer]);
      dm.dens_s[layer] = dm.dens_c[layer] = nullptr;
    }
    f1 = nullptr;
    if (H1_adj_fx) cudaFree(H1_adj_fx);
    H1_adj_fx = nullptr;
    if (zbl_e) cudaFree(zbl_e);
    zbl_e = nullptr;
    first = ntype = nidx = ntype_e = atom_order = nneigh = nullptr;
    xyz = r = energies = forces = nullptr;
    capN = capE = 0;
    evaluated = false;
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
    H1_adj_fx = dalloc<smx::fix64>(nN * dm.nLM * C);
    Phi1_adj = dalloc<float>(nN * dm.n_lme * C);
    A1_adj = dalloc<float>(nN * 16 * C);
    M1_adj = dalloc<float>(nN * C);
    H2_adj = dalloc<float>(nN * C);
    // L_max = 2 with two channel slices: one f1 slice each
    dm.f1_stride = l2_split_max > 1 ? 3 * nE : 0;
    f1 = dalloc<double>(3 * nE * l2_split_max);
    zbl_e = dalloc<float>(nN);
    first = dalloc<int>(nN + 1);
    ntype = dalloc<int>(nN);
    nidx = dalloc<int>(nE);
    ntype_e = dalloc<int>(nE);
    xyz = dalloc<double>(3 * nE);
    r = dalloc<double>(nE);
    energies = dalloc<double>(nN);
    forces = dalloc<double>(3 * nE);
    atom_order = dalloc<int>(2 * nN);  // all nodes, then the layer-1 nodes of a halo pass
    nneigh = dalloc<int>(nN);
    if (precision == SMX_PRECISION_BF16) {
      const long T = smx::split_xterms(tc_terms);  // stored X terms
      M0_bf = dalloc<__nv_bfloat16>(T * nN * dm.nLM * C);
      Phi1_bf = dalloc<__nv_bfloat16>(T * nN * dm.n_lme * C);
      A1adj_bf = dalloc<__nv_bfloat16>(T * nN * 16 * C);
      H1adj_bf = dalloc<__nv_bfloat16>(T * nN * dm.nLM * C);
      dm.op_m0 = tc_H1 ? M0_bf : nullptr;
      dm.op_phi1 = Phi1_bf;
      dm.op_a1adj = A1adj_bf;
    }
    for (int layer = 0; layer < 2; ++layer)
      if (dm.dens_spl[layer]) {
        dm.dens_s[layer] = dalloc<float>(nN);
        dm.dens_c[layer] = dalloc<float>(nN);
      }
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

  // ---- tensor-core GEMM schedule (BF16 form) and its autotuner ----
  // Groups: 0 H1, 1 A1 (one launch for all l), 2 Phi1_adj (ditto), 3 M0_adj.  The N-tile
  // width (A1, Phi1_adj; the H1/M0_adj tiles are the two L blocks, so N-tile = C) and the
  // TMA ring depth are picked by timing the candidates on the first evaluation's own
  // operands (CUDA events, one warm-up and three timed launches each), then kept.
  struct TcCfg {
    int NT = 0;  // 0: C; -1: each GEMM's whole B width (one N-tile: X is read once)
    int stages = 4;
  };
  TcCfg tc_cfg[4];
  bool tc_tuned[4] = {false, false, false, false};
  bool autotune = true;
  float tc_tuned_us[4] = {0, 0, 0, 0};
  // test of the timeout path: this many of the next tensor-core GEMM launches issue no
  // load, so their bounded wait gives up (option "test_gemm_timeout")
  int test_gemm_timeout = 0;

  void tc_apply(const TcCfg& c, smx::UmmaGemm* g, int ng, bool tile_n) const {
    for (int q = 0; q < ng; ++q) {
      if (tile_n) g[q].NT = c.NT > 0 ? c.NT : (c.NT < 0 ? g[q].nb_rows : dm.C);
      g[q].stages = c.stages;
    }
  }

  void tc_tune(int gid, smx::UmmaGemm* g, int ng, bool tile_n, cudaStream_t s) {
    const int C = dm.C;
    std::vector<TcCfg> cand;
    for (int nt : {C, C / 2, 2 * C}) {
      if (!tile_n && nt != C) continue;
      bool ok = nt >= 64 && nt <= 256;
      for (int q = 0; q < ng && ok; ++q) ok = g[q].nb_rows % nt == 0 && smx::umma_supported(g[q].K, nt, g[q].terms);
      if (!ok) continue;
      for (int st : {1, 2, 3, 4}) cand.push_back(TcCfg{nt == C ? 0 : nt, st});
    }
    if (tile_n) {  // one N-tile per GEMM where some B is wider than C and all fit a tile
      bool ok = true, wider = false;
      for (int q = 0; q < ng && ok; ++q) {
        ok = g[q].nb_rows <= 256 && smx::umma_supported(g[q].K, g[q].nb_rows, g[q].terms);
        wider = wider || g[q].nb_rows != C;
      }
      if (ok && wider)
        for (int st : {1, 2, 3, 4}) cand.push_back(TcCfg{-1, st});
    }
    cudaEvent_t a, b;
    check(cudaEventCreate(&a), "cudaEventCreate");
    check(cudaEventCreate(&b), "cudaEventCreate");
    float best = 1e30f;
    TcCfg bestc = tc_cfg[gid];
    smx::UmmaGemm w[4];
    for (const TcCfg& c : cand) {
      std::copy(g, g + ng, w);
      tc_apply(c, w, ng, tile_n);
      smx::launch_umma_gemms(w, ng, status_dev, s);  // warm-up
      check(cudaEventRecord(a, s), "cudaEventRecord");
      for (int r = 0; r < 3; ++r) smx::launch_umma_gemms(w, ng, status_dev, s);
      check(cudaEventRecord(b, s), "cudaEventRecord");
      check(cudaEventSynchronize(b), "autotune");
      float ms = 0.0f;
      check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
      if (ms < best) {
        best = ms;
        bestc = c;
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    tc_cfg[gid] = bestc;
    tc_tuned[gid] = true;
    tc_tuned_us[gid] = best * 1000.0f / 3.0f;
  }

  // The M0_adj GEMM (L_max 1) as two segments, one per L block: X rows grouped by L
  // (lgroup_row), B = the block's C x C weights, output rows (node, LM) of Y [N][4][C].
  void lblock_gemms(const __nv_bfloat16* X, const __nv_bfloat16* W, float* Y, int N, smx::UmmaGemm* g) const {
    const int C = dm.C, T = tc_terms;
    const long XT = smx::split_xterms(T), WT = smx::split_wterms(T), ns = static_cast<long>(dm.nLM) * C;
    g[0] = smx::UmmaGemm{X, N, C, W, C, C, smx::UmmaOut{Y, N, 1, ns, 0, 0, 0}};
    g[1] = smx::UmmaGemm{X + XT * N * C, 3L * N, C, W + WT * C * C, C, C, smx::UmmaOut{Y, 3L * N, 3, ns, C, C, 0}};
    g[0].terms = g[1].terms = T;
  }

  // launch one GEMM group with its tuned schedule (tuning it first if due)
  void run_tc(int gid, smx::UmmaGemm* g, int ng, bool tile_n, cudaStream_t s) {
    if (ng == 0) return;
    if (autotune && !tc_tuned[gid]) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      check(cudaStreamIsCapturing(s, &cs), "cudaStreamIsCapturing");
      if (cs == cudaStreamCaptureStatusNone) tc_tune(gid, g, ng, tile_n, s);
    }
    tc_apply(tc_cfg[gid], g, ng, tile_n);
    const bool test = test_gemm_timeout > 0;
    if (test) --test_gemm_timeout;
    smx::launch_umma_gemms(g, ng, status_dev, s, test);
  }

  // padded Clebsch-Gordan tables (option "cg_padded" 0 switches the kernels to the
  // compressed-row walk, which models with longer rows always use)
  const int2 *cg_fwd_pad_keep = nullptr, *cg_rev_pad_keep = nullptr;
  int cg_fwd_kp_keep = 0;
  void use_cg_padded(bool on) {
    dm.cg_fwd_pad = on ? cg_fwd_pad_keep : nullptr;
    dm.cg_fwd_kp = on ? cg_fwd_kp_keep : 0;
    dm.cg_rev_pad = on ? cg_rev_pad_keep : nullptr;
  }

  // ---- centre-atom order of the edge kernels ----
  // -1: species-sorted when a layer's spline table exceeds kOrderTableBytes (then the
  // rows of all pairs do not stay in L2, the rows of one centre species do); 0: input
  // order; 1: species-sorted.
  static constexpr double kOrderTableBytes = 64.0 * 1024 * 1024;
  int species_order = -1;
  bool order_species() const {
    if (species_order >= 0) return species_order == 1;
    const double npairs = 0.5 * dm.S * (dm.S + 1);
    const double fwd = npairs * dm.nint * dm.n_instr * dm.C * 16.0;
    const double l0 = static_cast<double>(dm.S) * dm.S * dm.nint * 4 * dm.C * 16.0;
    return dm.S > 1 && (fwd > kOrderTableBytes || l0 > kOrderTableBytes);
  }

  // ---- centre-atom schedule of the per-atom kernels and its autotuner ----
  // Each per-atom kernel runs either one block per atom or as a persistent grid (its
  // resident blocks on every SM) claiming atoms from a counter (smx::AtomCursor).  The
  // first evaluation outside a stream capture times whole passes in both schedules
  // (alternating, two passes each, per-stage CUDA events) and keeps the faster per
  // kernel; the two layer-0 adjoint kernels share one stage and are switched together.
  int pfull[smx::kAkCount] = {};
  // L_max = 2 layer-1 kernels: channel slices per node, 1 or (from 64 channels) 2, tuned
  int l2_split_max = 1;
  int sched_force = -1;  // -1: tune; 0: one block per atom; 1: persistent
  bool sched_tuned = false;

  void sched_set(int mode) {
    for (int k = 0; k < smx::kAkCount; ++k) dm.pgrid[k] = mode ? pfull[k] : 0;
  }

  // the persistent grids of the layer-1 kernels follow their block shape
  void set_l2_split(int ns) {
    dm.l2_split = ns;
    int nsm = 0, per_sm[smx::kAkCount] = {};
    check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");
    smx::layer1_residency(dm, per_sm);
    for (int k : {smx::kAkLayer1Fwd, smx::kAkLayer1Rev}) {
      const bool on = dm.pgrid[k] > 0;
      pfull[k] = per_sm[k] * nsm;
      if (on) dm.pgrid[k] = pfull[k];
    }
  }

  void tune_sched(const smx::EdgeIn& in, double* out_e, double* out_f, cudaStream_t s, int n1) {
    static constexpr int kStageOf[smx::kAkCount] = {0, 8, 8, 2, 6, 4};  // stage index of each kernel
    const bool prof = profile;
    profile = true;
    float best[2][kStages];
    for (auto& b : best)
      for (float& v : b) v = 1e30f;
    for (int rep = 0; rep < 2; ++rep)
      for (int mode = 0; mode < 2; ++mode) {
        sched_set(mode);
        run_pass(in, out_e, out_f, s, n1);
        check(cudaEventSynchronize(ev[kStages]), "autotune");
        for (int q = 0; q < kStages; ++q) {
          float ms = 0.0f;
          check(cudaEventElapsedTime(&ms, ev[q], ev[q + 1]), "cudaEventElapsedTime");
          best[mode][q] = std::min(best[mode][q], ms);
        }
      }
    for (int k = 0; k < smx::kAkCount; ++k) {
      const int q = kStageOf[k];
      dm.pgrid[k] = best[1][q] < best[0][q] ? pfull[k] : 0;
    }
    if (l2_split_max > 1) {  // channel slices of the L_max = 2 layer-1 kernels: stages 2 and 6
      float t[3] = {1e30f, 1e30f, 1e30f};
      for (int rep = 0; rep < 2; ++rep)
        for (int ns = 1; ns <= l2_split_max; ++ns) {
          set_l2_split(ns);
          run_pass(in, out_e, out_f, s, n1);
          check(cudaEventSynchronize(ev[kStages]), "autotune");
          float a = 0.0f, b = 0.0f;
          check(cudaEventElapsedTime(&a, ev[2], ev[3]), "cudaEventElapsedTime");
          check(cudaEventElapsedTime(&b, ev[6], ev[7]), "cudaEventElapsedTime");
          t[ns] = std::min(t[ns], a + b);
        }
      set_l2_split(t[1] <= t[2] ? 1 : 2);
    }
    profile = prof;
    sched_tuned = true;
  }

  long sched_mask() const {
    long mask = 0;
    for (int k = 0; k < smx::kAkCount; ++k)
      if (dm.pgrid[k] > 0) mask |= 1L << k;
    return mask;
  }

  // SMX_ERR_TIMEOUT if a bounded device wait gave up since the last check (call after
  // synchronising the work in question); clears the word.
  int take_status() {
    if (!status_host) return SMX_OK;
    const unsigned v = *reinterpret_cast<volatile unsigned*>(status_host);
    if (v == 0) return SMX_OK;
    *reinterpret_cast<volatile unsigned*>(status_host) = 0;
    return SMX_ERR_TIMEOUT;
  }

  // ---- single stages (the reference binding's compute_* / reverse_*, symmetrix/source/
  // cpp/mace.cpp:152-179) on the workspace of the last evaluation.  The channel-mixing
  // GEMMs run on the float32 SIMT kernel in both precision forms; compute_Phi1 also
  // evaluates R1 and Y (one fused kernel, as in the full pass); the layer-1 kernels run
  // without the density-normalisation terms, which belong to compute_A1_scaled and
  // reverse_A1_scaled (fused into the node tail).
  smx::GemmBatch node_gemm(const float* X, float* Y, const float* const* W, int nb, bool per_l, bool trans) const {
    // per_l false: the L blocks of [N][nLM][C] (H1 and its adjoint); true: the l blocks of
    // Phi1 [N][n_lme][C] against A1 [N][16][C] (trans: A1_adj -> Phi1_adj)
    const int C = dm.C, N = per_l ? lastN1 : lastN;
    smx::GemmBatch b{};
    if (!per_l) {
      for (int L = 0; L < nb; ++L)
        b.s[b.n++] = seg_rows(X, Y, W[L], N, 2 * L + 1, C, C, static_cast<long>(dm.nLM) * C, L * L * C, C,
                              static_cast<long>(dm.nLM) * C, L * L * C, C);
      return b;
    }
    for (int l = 0; l < 4; ++l) {
      if (dm.num_e[l] == 0) continue;
      const int K = dm.num_e[l] * C;
      if (!trans)
        b.s[b.n++] = seg_rows(X, Y, W[l], N, 2 * l + 1, K, C, static_cast<long>(dm.n_lme) * C, dm.lme_off[l] * C, K,
                              16L * C, l * l * C, C);
      else
        b.s[b.n++] = seg_rows(X, Y, W[l], N, 2 * l + 1, C, K, 16L * C, l * l * C, C,
                              static_cast<long>(dm.n_lme) * C, dm.lme_off[l] * C, K);
    }
    return b;
  }

  // "compute_H1", "reverse_H1", "compute_A1", "reverse_A1": node stages of the last N
  bool run_node_stage(const std::string& st, cudaStream_t s) {
    const int C = dm.C;
    const float* WH[3] = {dm.H1W, dm.H1W + static_cast<size_t>(C) * C, dm.H1W + 2 * static_cast<size_t>(C) * C};
    const float* WHT[3] = {dm.H1W_T, dm.H1W_T + static_cast<size_t>(C) * C, dm.H1W_T + 2 * static_cast<size_t>(C) * C};
    if (st == "compute_H1") {
      smx::launch_gemm(node_gemm(M0, H1, WH, dm.L_max + 1, false, false), s);
    } else if (st == "reverse_H1") {
      smx::launch_gemm(node_gemm(H1_adj, M0_adj, WHT, dm.L_max + 1, false, false), s);
    } else if (st == "compute_A1") {
      smx::launch_gemm(node_gemm(Phi1, A1, dm.A1W, 4, true, false), s);
    } else if (st == "reverse_A1") {
      smx::launch_gemm(node_gemm(A1_adj, Phi1_adj, dm.A1W_T, 4, true, true), s);
      A1adj_kept = true;
    } else {
      return false;
    }
    return true;
  }

  // "compute_Phi1" (with R1 and Y) and "reverse_Phi1" on the edges `in` (E edges): the
  // forward writes Phi1; the adjoint adds dPhi1-contracted terms to H1_adj (from zero with
  // zero_h1adj) and sets node_forces to its per-edge forces (added to the current ones
  // unless zero_dxyz), as mace.cpp:504-605 with its two flags
  void run_edge_stage(bool reverse, const smx::EdgeIn& in, long E, bool zero_dxyz, bool zero_h1adj,
                      cudaStream_t s) {
    smx::DevModel m = dm;
    m.dens_spl[0] = m.dens_spl[1] = nullptr;
    m.op_phi1 = nullptr;
    const long nh = static_cast<long>(in.N) * dm.nLM * dm.C;
    if (!reverse) {
      smx::launch_layer1_fwd(m, in, H1, Phi1, s);
      Phi1_kept = true;
      return;
    }
    smx::launch_rows_to_fixed(H1_adj, H1_adj_fx, nh, zero_h1adj, s);
    smx::launch_layer1_rev(m, in, H1, Phi1_adj, H1_adj_fx, f1, s);
    smx::launch_fixed_rows(H1_adj_fx, H1_adj, nullptr, in.N * static_cast<long>(dm.nLM), dm.C, 1, dm.nLM, s);
    smx::launch_forces_from_f1(forces, f1, dm.f1_stride, dm.l2_split, 3 * E, zero_dxyz, s);
  }

  // The full forward + adjoint pass on device-resident inputs (tuning the atom schedule
  // first when due).  n1 (0 < n1 <= in.N; -1: in.N): layer 1, the readouts and ZBL run
  // over the first n1 nodes only and the rest form a halo that layer 0 evaluates for the
  // H1 rows the first n1 nodes' edges read (the pair style's no-MPI-message-passing
  // form, pair_symmetrix/pair_symmetrix_mace.cpp:672-698); out_e then receives n1 values.
  void run(const smx::EdgeIn& in, double* out_e, double* out_f, cudaStream_t s, int n1 = -1) {
    if (autotune && sched_force < 0 && !sched_tuned && in.N > 0) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      check(cudaStreamIsCapturing(s, &cs), "cudaStreamIsCapturing");
      if (cs == cudaStreamCaptureStatusNone) tune_sched(in, out_e, out_f, s, n1);
    }
    run_pass(in, out_e, out_f, s, n1);
  }

  void run_pass(const smx::EdgeIn& in_, double* out_e, double* out_f, cudaStream_t s, int n1 = -1) {
    smx::EdgeIn in = in_;  // layer 0: all N nodes
    const int N = in.N;
    const int N1 = n1 < 0 ? N : n1;
    if (N1 > N || (N > 0 && N1 == 0)) throw std::invalid_argument("layer-1 node count outside (0, num_nodes]");
    const bool halo = N1 < N;
    if (N > 0 && order_species()) {
      smx::launch_species_order(in.node_type, N, dm.S, atom_order, s);
      in.order = atom_order;
    }
    smx::EdgeIn in1 = in;  // layer 1: the first N1 nodes (a prefix of the edge list)
    in1.N = N1;
    if (halo && in.order) {  // the layer-1 kernels visit the first N1 nodes, in their own order
      smx::launch_species_order(in.node_type, N1, dm.S, atom_order + capN, s);
      in1.order = atom_order + capN;
    }
    if (halo) in.n_local = N1;
    const int C = dm.C;
    const int T = tc_terms, XT = smx::split_xterms(T);
    lastN = N;
    lastN1 = N1;
    if (N == 0) {
      evaluated = true;
      return;
    }
    if (profile && !ev[0])
      for (auto& e : ev) check(cudaEventCreate(&e), "cudaEventCreate");
    prof_stream = s;
    mark(0, s);
    // the halo's H1_adj rows receive only the local nodes' layer-1 scatter (the node tail
    // seeds the first N1 rows)
    if (halo)
      smx::launch_rows_to_fixed(nullptr, H1_adj_fx + static_cast<size_t>(N1) * dm.nLM * C,
                                static_cast<long>(N - N1) * dm.nLM * C, true, s);
    // The BF16 form's GEMMs read the producers' split bf16 rows; the float32 copies of
    // M0, Phi1 and A1_adj are then written only for inspection or a SIMT fallback.
    bool all_A1 = true, all_Phi1adj = true;
    for (int l = 0; l < 4; ++l)
      if (dm.num_e[l] > 0) {
        all_A1 = all_A1 && tc_A1[l];
        all_Phi1adj = all_Phi1adj && tc_Phi1adj[l];
      }
    const bool f32_rows = keep_stages || precision != SMX_PRECISION_BF16;
    float* M0_out = (f32_rows || !tc_H1) ? M0 : nullptr;
    float* Phi1_out = (f32_rows || !all_A1) ? Phi1 : nullptr;
    float* A1adj_out = (f32_rows || !all_Phi1adj) ? A1_adj : nullptr;
    M0_kept = M0_out != nullptr;
    Phi1_kept = Phi1_out != nullptr;
    A1adj_kept = A1adj_out != nullptr;
    evaluated = true;
    smx::launch_layer0_fwd(dm, in, A0, M0_out, dm.has_zbl ? zbl_e : nullptr, s);
    mark(1, s);
    if (tc_H1) {  // H1 = M0 @ H1W[L]  (mace.cpp:397-423), tensor cores
      // (layer0_fwd wrote M0 as split bf16 rows into M0_bf)
      smx::UmmaGemm g{M0_bf, static_cast<long>(N) * dm.nLM, C, W_H1, 2 * C, C,
                       smx::UmmaOut{H1, static_cast<long>(N) * dm.nLM, dm.nLM, static_cast<long>(dm.nLM) * C, 0, C,
                                    1}};
      g.terms = T;
      run_tc(0, &g, 1, false, s);
    } else {  // H1 = M0 @ H1W[L]  (mace.cpp:397-423)
      smx::GemmBatch b{};
      for (int L = 0; L <= dm.L_max; ++L)
        b.s[b.n++] = seg_rows(M0, H1, dm.H1W + static_cast<size_t>(L) * C * C, N, 2 * L + 1, C, C,
                              static_cast<long>(dm.nLM) * C, L * L * C, C, static_cast<long>(dm.nLM) * C, L * L * C, C);
      smx::launch_gemm(b, s);
    }
    mark(2, s);
    smx::launch_layer1_fwd(dm, in1, H1, Phi1_out, s);
    mark(3, s);
    {  // A1 = Phi1 @ A1W[l]  (mace.cpp:607-642)
      // tensor cores on the per-l regrouped split bf16 rows layer1_fwd wrote, one launch
      smx::UmmaGemm g[4];
      int ng = 0;
      for (int l = 0; l < 4; ++l)
        if (dm.num_e[l] > 0 && tc_A1[l]) {
          const long rows = static_cast<long>(N1) * (2 * l + 1);
          const int K = dm.num_e[l] * C;
          g[ng] = smx::UmmaGemm{Phi1_bf + static_cast<size_t>(XT) * N1 * dm.lme_off[l] * C, rows, K, W_A1[l], C, C,
                                smx::UmmaOut{A1, rows, 2 * l + 1, 16L * C, l * l * C, C, 0}};
          g[ng++].terms = T;
        }
      run_tc(1, g, ng, true, s);
      smx::GemmBatch b{};
      for (int l = 0; l < 4; ++l)
        if (dm.num_e[l] > 0 && !tc_A1[l])
          b.s[b.n++] = seg_rows(Phi1, A1, dm.A1W[l], N1, 2 * l + 1, dm.num_e[l] * C, C,
                                static_cast<long>(dm.n_lme) * C, dm.lme_off[l] * C, dm.num_e[l] * C,
                                16L * C, l * l * C, C);
      smx::launch_gemm(b, s);
    }
    mark(4, s);
    smx::launch_node_tail(dm, in.node_type, N1, A1, H1, M1, H2, A1adj_out, H1_adj_fx, M1_adj, H2_adj,
                          dm.has_zbl ? zbl_e : nullptr, out_e, s);
    mark(5, s);
    {  // Phi1_adj = A1_adj @ A1W[l]^T  (mace.cpp:644-679)
      // tensor cores on the split rows node_tail wrote, one N-tile per eta, one launch
      smx::UmmaGemm g[4];
      int ng = 0;
      for (int l = 0; l < 4; ++l)
        if (dm.num_e[l] > 0 && tc_Phi1adj[l]) {
          const long rows = static_cast<long>(N1) * (2 * l + 1);
          g[ng] = smx::UmmaGemm{A1adj_bf + static_cast<size_t>(XT) * N1 * l * l * C, rows, C, W_Phi1adj[l],
                                dm.num_e[l] * C, C,
                                smx::UmmaOut{Phi1_adj, rows, 2 * l + 1, static_cast<long>(dm.n_lme) * C,
                                             dm.lme_off[l] * C, dm.num_e[l] * C, 0}};
          g[ng++].terms = T;
        }
      run_tc(2, g, ng, true, s);
      smx::GemmBatch b{};
      for (int l = 0; l < 4; ++l)
        if (dm.num_e[l] > 0 && !tc_Phi1adj[l])
          b.s[b.n++] = seg_rows(A1_adj, Phi1_adj, dm.A1W_T[l], N1, 2 * l + 1, C, dm.num_e[l] * C, 16L * C, l * l * C,
                                C, static_cast<long>(dm.n_lme) * C, dm.lme_off[l] * C, dm.num_e[l] * C);
      smx::launch_gemm(b, s);
    }
    mark(6, s);
    smx::launch_layer1_rev(dm, in1, H1, Phi1_adj, H1_adj_fx, f1, s);
    mark(7, s);
    // the float H1_adj rows (and the BF16 form's split operand) from the fixed-point sums
    smx::launch_fixed_rows(H1_adj_fx, H1_adj, tc_H1 ? H1adj_bf : nullptr, static_cast<long>(N) * dm.nLM, C, T, dm.nLM,
                           s);
    if (tc_H1) {  // M0_adj = H1_adj @ H1W[L]^T  (mace.cpp:425-451), tensor cores
      smx::UmmaGemm g[2];
      lblock_gemms(H1adj_bf, W_M0adj, M0_adj, N, g);
      run_tc(3, g, 2, false, s);
    } else {  // M0_adj = H1_adj @ H1W[L]^T  (mace.cpp:425-451)
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

