// MACE model: host-side parse of the libsymmetrix JSON format and the device
// layout the GB300 kernels read.
//
// The JSON keys and their meaning are those of MACE::load_from_json
// (libsymmetrix/source/mace.cpp:905-1030).  Load-time transforms (all exact in
// float64, rounded to float32 once):
//   * layer-0 radial splines are folded with H0_weights[type_j] and the
//     per-species channel mixing A0_weights[type_i][l] into one spline set per
//     ORDERED species pair, so A0 = sum_j Y_lm(x_ij) R0'_{ti,tj,l}(r_ij) needs no
//     GEMM (a spline is linear in its nodal data);
//   * layer-1 radial splines are reordered into the canonical tensor-product
//     instruction order the kernels are specialised for;
//   * the symmetric-contraction polynomials keep the JSON monomials (shared by
//     every species and channel of one output) with coefficients laid out
//     channel-fastest;
//   * every channel-mixing matrix is stored as given and transposed for the
//     adjoint pass.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

namespace smx {

constexpr int kNumLm = 16;  // (l_max + 1)^2 with l_max = 3
constexpr int kMaxLM = 9;   // (L_max + 1)^2 with L_max <= 2

struct HostModel {
  int S = 0, C = 0, l_max = 0, L_max = 0, nLM = 0;
  double r_cut = 0.0;
  std::vector<int> Z;
  std::vector<double> e0;
  bool has_zbl = false;
  double zbl_a_exp = 0, zbl_a_pref = 0;
  std::vector<double> zbl_c, zbl_radii;
  int zbl_p = 0;
  // radial splines, nodal values/derivatives [pair][spline][knot]
  double spl_h = 0;
  int K = 0, npairs = 0, nspl0 = 0, nspl1 = 0;
  std::vector<double> v0, d0, v1, d1;
  std::vector<double> H0;   // [S][C]
  std::vector<double> A0W;  // [S][4][C][C]
  bool A0_scaled = false, A1_scaled = false;
  double A0_h = 0, A1_h = 0;
  int A0_K = 0, A1_K = 0;
  std::vector<double> A0_sv, A0_sd, A1_sv, A1_sd;  // [pair][knot]
  std::vector<std::vector<std::vector<int>>> M0_mono;  // [LM][t] -> variable indices
  std::vector<std::vector<double>> M0_coef;            // [(s*nLM+LM)*C + k][t]
  std::vector<std::vector<int>> M1_mono;
  std::vector<std::vector<double>> M1_coef;  // [s*C + k][t]
  std::vector<double> H1W;                   // [L][C][C]
  std::vector<int> phi_l, phi_l1, phi_l2, phi_lme, phi_p;
  std::vector<double> phi_cg;
  int n_lme = 0, n_p = 0, n_instr = 0;
  int num_e[4] = {0, 0, 0, 0};
  std::vector<std::vector<double>> A1W;  // [l][n_e*C*C]
  std::vector<double> H2W_H1;            // [S][C][C]
  std::vector<double> H2W_M1;            // [C][C]
  std::vector<double> ro1, ro2_w1, ro2_w2;
  double ro2_scale = 1.0;
  int n_hidden = 16;

  void load_json(const std::string& path);
  int pair_index(int a, int b) const {
    if (a > b) std::swap(a, b);
    return a * (2 * S - a - 1) / 2 + b;
  }
};

// Canonical layer-1 instruction list (l1 from Y, l2 from H1, l_out) for L_max,
// sorted by l_out with the creation order (l2 outer, l1 inner) inside each l_out.
std::vector<std::array<int, 3>> canonical_instructions(int L_max);

// Host-side float32 arrays in the exact layout the device kernels read.
struct PackedModel {
  int S, C, L_max, nLM, n_lme, n_instr, n_p, nint, npairs;
  float h, r_cut;
  // folded, ordered pair ti*S+tj: [S*S][nint][4 (l)][2][C/2][4], channel pairs (2c, 2c+1):
  // plane 0 = (c0, c0', c1, c1'), plane 1 = (c2, c2', c3, c3')
  std::vector<float> spl0;
  // [npairs][nint][n_instr][2][C/2][4], canonical instruction order; channel pairs
  // (2c, 2c+1): plane 0 = (c0, c0', c1, c1'), plane 1 = (c2, c2', c3, c3')
  std::vector<float> spl1;
  std::vector<float> spl1_fwd;  // [npairs][nint][n_instr][C][4]: one float4 cubic per channel
  std::vector<int> mono0;      // packed a | b<<8 | c<<16 (16 = constant one), per LM contiguous
  std::vector<int> mono0_off;  // [nLM + 1]
  int T0 = 0;                  // max monomials per LM (coefficient stride)
  std::vector<float> coef0;    // [S][nLM][T0][C]
  std::vector<int> mono1;
  int T1 = 0;
  std::vector<float> coef1;  // [S][T1][C]
  // 1 when every monomial of the model is in the canonical sets of poly_canon.h; the
  // coefficients are then stored in canonical order (zero for absent monomials) and
  // the kernels use the generated straight-line polynomials
  int poly_canon = 0;
  std::vector<float> H1W, H1W_T;  // [L][C][C]
  // CG table: sorted by lme (forward) and by canonical p (adjoint)
  std::vector<int> cg_fwd_off;  // [n_lme + 1]
  std::vector<int> cg_fwd_p;
  std::vector<float> cg_fwd_v;
  std::vector<int> cg_rev_off;  // [n_p + 1]
  std::vector<int> cg_rev_lme;
  std::vector<float> cg_rev_v;
  int lme_off[4], num_e[4];
  std::vector<float> A1W[4], A1W_T[4];  // [n_e C][C] and [C][n_e C]
  std::vector<float> H2W_H1, H2W_H1_T;  // [S][C][C]
  std::vector<float> H2W_M1, H2W_M1_T;  // [C][C]
  std::vector<float> ro1, ro2_w1, ro2_w2;
  float ro2_scale;
  int n_hidden;
  std::vector<float> e0;
  std::vector<int> Z;
  // density-normalised blocks (mace.cpp:273-346, :681-757): per unordered species pair
  // one cubic per interval, [npairs][nint][4], on knots of spacing dens_h[layer]
  int dens_scaled[2] = {0, 0}, dens_nint[2] = {0, 0};
  float dens_h[2] = {0, 0};
  std::vector<float> dens_spl[2];
  // ZBL pair repulsion (zbl.cpp): per ordered species pair (1/a, 0.5 * 14.3996 Zu Zv, r_max, 0)
  int has_zbl = 0, zbl_p = 0;
  float zbl_c[4] = {0, 0, 0, 0};
  std::vector<float> zbl_pair;  // [S*S][4]
};

PackedModel pack_model(const HostModel& hm);

// Binary model cache (model_cache.cpp): the packed model plus the HostModel scalars
// the engine reads; load fills only those HostModel fields.
bool is_model_cache(const std::string& path);
void save_model_cache(const std::string& path, const HostModel& hm, const PackedModel& pm);
void load_model_cache(const std::string& path, HostModel& hm, PackedModel& pm);

// JSON or cache file -> (hm, pm)
inline void load_model(const std::string& path, HostModel& hm, PackedModel& pm) {
  if (is_model_cache(path)) {
    load_model_cache(path, hm, pm);
  } else {
    hm.load_json(path);
    pm = pack_model(hm);
  }
}

}  // namespace smx
