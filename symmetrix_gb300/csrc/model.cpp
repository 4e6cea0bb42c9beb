// Model loading and packing for the GB300 engine (see model.hpp).
#include "model.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>

#include "json_reader.hpp"
#include "poly_canon_tables.h"

namespace smx {

namespace {

std::string read_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open model file '" + path + "'");
  std::ostringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

std::vector<double> numbers(const JsonDoc& d, uint32_t n, std::vector<uint32_t>* shape = nullptr) {
  std::vector<double> v;
  d.flatten(n, v, shape);
  return v;
}

std::vector<int> ints(const JsonDoc& d, uint32_t n) {
  std::vector<double> v = numbers(d, n);
  std::vector<int> out(v.size());
  for (size_t i = 0; i < v.size(); ++i) out[i] = static_cast<int>(v[i]);
  return out;
}

std::vector<std::vector<int>> int_lists(const JsonDoc& d, uint32_t n) {
  std::vector<std::vector<int>> out(d.size(n));
  for (uint32_t q = 0; q < out.size(); ++q) out[q] = ints(d, d.elem(n, q));
  return out;
}

void require(bool ok, const std::string& what) {
  if (!ok) throw std::invalid_argument("model file: " + what);
}

}  // namespace

void HostModel::load_json(const std::string& path) {
  JsonDoc d(read_file(path));
  const uint32_t R = d.root();
  auto get = [&](const char* k) { return d.at(R, k); };
  S = static_cast<int>(d.num(get("num_elements")));
  C = static_cast<int>(d.num(get("num_channels")));
  r_cut = d.num(get("r_cut"));
  l_max = static_cast<int>(d.num(get("l_max")));
  L_max = static_cast<int>(d.num(get("L_max")));
  require(S >= 1, "num_elements must be positive");
  require(std::isfinite(r_cut) && r_cut > 0.0, "r_cut must be positive and finite");
  require(l_max == 3, "l_max must be 3");
  require(L_max >= 1 && L_max <= 2, "L_max must be 1 or 2");
  require(C >= 32 && C <= 256 && C % 32 == 0, "num_channels must be a multiple of 32 in [32, 256]");
  nLM = (L_max + 1) * (L_max + 1);
  Z = ints(d, get("atomic_numbers"));
  e0 = numbers(d, get("atomic_energies"));
  require(static_cast<int>(Z.size()) == S && static_cast<int>(e0.size()) == S, "species table sizes");

  has_zbl = d.boolean(get("has_zbl"));
  if (has_zbl) {
    zbl_a_exp = d.num(get("zbl_a_exp"));
    zbl_a_pref = d.num(get("zbl_a_prefactor"));
    zbl_c = numbers(d, get("zbl_c"));
    zbl_radii = numbers(d, get("zbl_covalent_radii"));
    zbl_p = static_cast<int>(d.num(get("zbl_p")));
    require(zbl_c.size() == 4, "zbl_c must have 4 entries");
  }

  // radial splines [pair][spline][knot]
  spl_h = d.num(get("radial_spline_h"));
  std::vector<uint32_t> sh;
  v0 = numbers(d, get("radial_spline_values_0"), &sh);
  require(sh.size() == 3, "radial_spline_values_0 must be 3-d");
  npairs = static_cast<int>(sh[0]);
  nspl0 = static_cast<int>(sh[1]);
  K = static_cast<int>(sh[2]);
  d0 = numbers(d, get("radial_spline_derivs_0"), &sh);
  require(sh.size() == 3 && (int)sh[0] == npairs && (int)sh[1] == nspl0 && (int)sh[2] == K, "radial_spline_derivs_0 shape");
  v1 = numbers(d, get("radial_spline_values_1"), &sh);
  require(sh.size() == 3 && (int)sh[0] == npairs && (int)sh[2] == K, "radial_spline_values_1 shape");
  nspl1 = static_cast<int>(sh[1]);
  d1 = numbers(d, get("radial_spline_derivs_1"), &sh);
  require(sh.size() == 3 && (int)sh[0] == npairs && (int)sh[1] == nspl1 && (int)sh[2] == K, "radial_spline_derivs_1 shape");
  require(npairs == S * (S + 1) / 2, "one spline set per unordered species pair");
  require(nspl0 == (l_max + 1) * C, "layer-0 radial set must have (l_max+1)*C splines");
  require(K >= 2, "at least two spline knots");
  // the knots must reach r_cut: the reference reads past its table otherwise
  // (cubic_spline_set.cpp:54 does no bounds check)
  require(std::isfinite(spl_h) && spl_h > 0.0 && (K - 1) * spl_h >= r_cut * (1.0 - 1e-6),
          "radial_spline_h must be positive, with (knots - 1) * h >= r_cut");

  H0 = numbers(d, get("H0_weights"));
  require(static_cast<int>(H0.size()) == S * C, "H0_weights size");
  A0W = numbers(d, get("A0_weights"), &sh);
  require(sh.size() == 3 && (int)sh[0] == S && (int)sh[1] == l_max + 1 && (int)sh[2] == C * C, "A0_weights shape");

  A0_scaled = d.boolean(get("A0_scaled"));
  if (A0_scaled) {
    A0_h = d.num(get("A0_spline_h"));
    A0_sv = numbers(d, get("A0_spline_values"), &sh);
    A0_K = static_cast<int>(sh[1]);
    A0_sd = numbers(d, get("A0_spline_derivs"));
    require((int)sh[0] == npairs && A0_sd.size() == A0_sv.size(), "A0 density splines shape");
  }

  // symmetric contraction, layer 0 (mace.cpp:956-973): {species: {LM: {k: [coef]}}}, {LM: [[idx..]]}
  const uint32_t m0w = get("M0_weights"), m0m = get("M0_monomials");
  M0_mono.assign(nLM, {});
  for (int LM = 0; LM < nLM; ++LM) M0_mono[LM] = int_lists(d, d.at(m0m, std::to_string(LM)));
  M0_coef.assign(static_cast<size_t>(S) * nLM * C, {});
  for (int s = 0; s < S; ++s) {
    const uint32_t ws = d.at(m0w, std::to_string(s));
    for (int LM = 0; LM < nLM; ++LM) {
      const uint32_t wl = d.at(ws, std::to_string(LM));
      for (int k = 0; k < C; ++k) {
        auto& v = M0_coef[(static_cast<size_t>(s) * nLM + LM) * C + k];
        v = numbers(d, d.at(wl, std::to_string(k)));
        require(v.size() == M0_mono[LM].size(), "M0 coefficient count != monomial count");
      }
    }
  }

  H1W = numbers(d, get("H1_weights"));
  require(static_cast<int>(H1W.size()) == (L_max + 1) * C * C, "H1_weights size");

  phi_l = ints(d, get("Phi1_l"));
  phi_l1 = ints(d, get("Phi1_l1"));
  phi_l2 = ints(d, get("Phi1_l2"));
  phi_lme = ints(d, get("Phi1_lme"));
  phi_cg = numbers(d, get("Phi1_clebsch_gordan"));
  phi_p = ints(d, get("Phi1_lelm1lm2"));
  n_instr = static_cast<int>(phi_l.size());
  require(phi_l1.size() == phi_l.size() && phi_l2.size() == phi_l.size(), "Phi1 instruction tables");
  require(phi_lme.size() == phi_cg.size() && phi_p.size() == phi_cg.size(), "Phi1 coupling tables");
  require(nspl1 == n_instr * C, "layer-1 radial set must have n_instr*C splines");
  n_lme = 0;
  n_p = 0;
  for (int q = 0; q < 4; ++q) num_e[q] = 0;
  for (int q = 0; q < n_instr; ++q) {
    require(phi_l[q] >= 0 && phi_l[q] <= l_max, "Phi1_l out of range");
    n_lme += 2 * phi_l[q] + 1;
    n_p += (2 * phi_l1[q] + 1) * (2 * phi_l2[q] + 1);
    num_e[phi_l[q]] += 1;
  }

  // layer-1 channel mixing [l][n_e*C*C]
  const uint32_t a1 = get("A1_weights");
  require(static_cast<int>(d.size(a1)) == l_max + 1, "A1_weights must have l_max+1 blocks");
  A1W.assign(l_max + 1, {});
  for (int l = 0; l <= l_max; ++l) {
    A1W[l] = numbers(d, d.elem(a1, l));
    require(static_cast<int>(A1W[l].size()) == num_e[l] * C * C, "A1_weights block size");
  }
  A1_scaled = d.boolean(get("A1_scaled"));
  if (A1_scaled) {
    A1_h = d.num(get("A1_spline_h"));
    A1_sv = numbers(d, get("A1_spline_values"), &sh);
    A1_K = static_cast<int>(sh[1]);
    A1_sd = numbers(d, get("A1_spline_derivs"));
    require((int)sh[0] == npairs && A1_sd.size() == A1_sv.size(), "A1 density splines shape");
  }

  const uint32_t m1w = get("M1_weights");
  M1_mono = int_lists(d, get("M1_monomials"));
  M1_coef.assign(static_cast<size_t>(S) * C, {});
  for (int s = 0; s < S; ++s) {
    const uint32_t ws = d.at(m1w, std::to_string(s));
    for (int k = 0; k < C; ++k) {
      auto& v = M1_coef[static_cast<size_t>(s) * C + k];
      v = numbers(d, d.at(ws, std::to_string(k)));
      require(v.size() == M1_mono.size(), "M1 coefficient count != monomial count");
    }
  }

  H2W_H1 = numbers(d, get("H2_weights_for_H1"), &sh);
  require(sh.size() == 2 && (int)sh[0] == S && (int)sh[1] == C * C, "H2_weights_for_H1 shape");
  H2W_M1 = numbers(d, get("H2_weights_for_M1"));
  require(static_cast<int>(H2W_M1.size()) == C * C, "H2_weights_for_M1 size");
  ro1 = numbers(d, get("readout_1_weights"));
  ro2_w1 = numbers(d, get("readout_2_weights_1"));
  ro2_w2 = numbers(d, get("readout_2_weights_2"));
  ro2_scale = d.num(get("readout_2_scale_factor"));
  n_hidden = static_cast<int>(ro2_w2.size());
  require(static_cast<int>(ro1.size()) == C, "readout_1_weights size");
  require(n_hidden >= 1 && n_hidden <= 32 && static_cast<int>(ro2_w1.size()) == n_hidden * C,
          "readout_2 weights sizes");
}

std::vector<std::array<int, 3>> canonical_instructions(int L_max) {
  std::vector<std::array<int, 3>> ins;
  for (int l2 = 0; l2 <= L_max; ++l2)
    for (int l1 = 0; l1 <= 3; ++l1)
      for (int l = std::abs(l1 - l2); l <= std::min(l1 + l2, 3); ++l)
        if ((l1 + l2 + l) % 2 == 0) ins.push_back({l1, l2, l});
  std::stable_sort(ins.begin(), ins.end(), [](const auto& a, const auto& b) { return a[2] < b[2]; });
  return ins;
}

namespace {

// Hermite coefficients (c0..c3) of interval i for nodal (v, d) with spacing h
inline void hermite(double h, double v0, double v1, double g0, double g1, double* c) {
  c[0] = v0;
  c[1] = g0;
  c[2] = (3.0 * (v1 - v0) - h * (2.0 * g0 + g1)) / (h * h);
  c[3] = (2.0 * (v0 - v1) + h * (g0 + g1)) / (h * h * h);
}

int pack_mono(const std::vector<int>& m) {
  if (m.size() > 3) throw std::invalid_argument("model file: monomials of degree > 3 are not supported");
  int idx[3] = {16, 16, 16};
  for (size_t q = 0; q < m.size(); ++q) {
    if (m[q] < 0 || m[q] >= kNumLm) throw std::invalid_argument("model file: monomial variable out of range");
    idx[q] = m[q];
  }
  return idx[0] | (idx[1] << 8) | (idx[2] << 16);
}

}  // namespace

PackedModel pack_model(const HostModel& hm) {
  PackedModel pm;
  const int S = hm.S, C = hm.C, nint = hm.K - 1;
  pm.S = S;
  pm.C = C;
  pm.L_max = hm.L_max;
  pm.nLM = hm.nLM;
  pm.n_lme = hm.n_lme;
  pm.n_instr = hm.n_instr;
  pm.n_p = hm.n_p;
  pm.nint = nint;
  pm.npairs = hm.npairs;
  pm.h = static_cast<float>(hm.spl_h);
  pm.r_cut = static_cast<float>(hm.r_cut);
  const double h = hm.spl_h;
  const int K = hm.K;

  // ---- layer 0: fold H0[tj] and A0W[ti][l] into ordered-pair splines ----
  pm.spl0.assign(static_cast<size_t>(S) * S * nint * 4 * C * 4, 0.0f);
  {
    std::vector<double> U(static_cast<size_t>(nint) * 4 * C);  // [iv][p][k'] for one (pair, l, tj)
    std::vector<double> out(static_cast<size_t>(nint) * 4 * C);
    for (int ti = 0; ti < S; ++ti)
      for (int tj = 0; tj < S; ++tj) {
        const int pr = hm.pair_index(ti, tj);
        for (int l = 0; l <= 3; ++l) {
          for (int iv = 0; iv < nint; ++iv)
            for (int kk = 0; kk < C; ++kk) {
              const size_t base = (static_cast<size_t>(pr) * hm.nspl0 + l * C + kk) * K;
              double c[4];
              hermite(h, hm.v0[base + iv], hm.v0[base + iv + 1], hm.d0[base + iv], hm.d0[base + iv + 1], c);
              for (int p = 0; p < 4; ++p) U[(static_cast<size_t>(iv) * 4 + p) * C + kk] = c[p] * hm.H0[tj * C + kk];
            }
          const double* W = &hm.A0W[(static_cast<size_t>(ti) * 4 + l) * C * C];
          std::fill(out.begin(), out.end(), 0.0);
          for (size_t row = 0; row < static_cast<size_t>(nint) * 4; ++row) {
            double* o = &out[row * C];
            const double* u = &U[row * C];
            for (int kk = 0; kk < C; ++kk) {
              const double a = u[kk];
              const double* w = W + static_cast<size_t>(kk) * C;
              for (int k = 0; k < C; ++k) o[k] += a * w[k];
            }
          }
          for (int iv = 0; iv < nint; ++iv)
            for (int k = 0; k < C; ++k)
              for (int p = 0; p < 4; ++p)
                pm.spl0[(((((static_cast<size_t>(ti) * S + tj) * nint + iv) * 4 + l) * 2 + p / 2) * (C / 2) + k / 2) * 4 +
                        (p % 2) * 2 + k % 2] = static_cast<float>(out[(static_cast<size_t>(iv) * 4 + p) * C + k]);
        }
      }
  }

  // ---- layer 1: canonical instruction order ----
  const auto canon = canonical_instructions(hm.L_max);
  if (static_cast<int>(canon.size()) != hm.n_instr)
    throw std::invalid_argument("model file: layer-1 instruction set differs from the MACE selection rules");
  std::vector<int> json_of_canon(hm.n_instr, -1), canon_of_json(hm.n_instr, -1);
  for (int q = 0; q < hm.n_instr; ++q) {
    for (int c = 0; c < hm.n_instr; ++c)
      if (json_of_canon[c] < 0 && canon[c][0] == hm.phi_l1[q] && canon[c][1] == hm.phi_l2[q] &&
          canon[c][2] == hm.phi_l[q]) {
        json_of_canon[c] = q;
        canon_of_json[q] = c;
        break;
      }
    if (canon_of_json[q] < 0)
      throw std::invalid_argument("model file: unsupported layer-1 instruction");
  }
  // instructions must be grouped by output l (Phi1 rows are [l][m][e])
  for (int q = 1; q < hm.n_instr; ++q)
    if (hm.phi_l[q] < hm.phi_l[q - 1]) throw std::invalid_argument("model file: Phi1_l must be sorted");
  pm.spl1.assign(static_cast<size_t>(hm.npairs) * nint * hm.n_instr * C * 4, 0.0f);
  pm.spl1_fwd.assign(pm.spl1.size(), 0.0f);
  for (int pr = 0; pr < hm.npairs; ++pr)
    for (int c = 0; c < hm.n_instr; ++c) {
      const int q = json_of_canon[c];
      for (int k = 0; k < C; ++k) {
        const size_t base = (static_cast<size_t>(pr) * hm.nspl1 + q * C + k) * K;
        for (int iv = 0; iv < nint; ++iv) {
          double cc[4];
          hermite(h, hm.v1[base + iv], hm.v1[base + iv + 1], hm.d1[base + iv], hm.d1[base + iv + 1], cc);
          for (int p = 0; p < 4; ++p)
            pm.spl1[((((static_cast<size_t>(pr) * nint + iv) * hm.n_instr + c) * 2 + p / 2) * (C / 2) + k / 2) * 4 +
                    (p % 2) * 2 + k % 2] = static_cast<float>(cc[p]);
          for (int p = 0; p < 4; ++p)
            pm.spl1_fwd[(((static_cast<size_t>(pr) * nint + iv) * hm.n_instr + c) * C + k) * 4 + p] =
                static_cast<float>(cc[p]);
        }
      }
    }

  // CG table: json p -> (instruction, m1, m2) -> canonical p
  std::vector<int> off_json(hm.n_instr + 1, 0), off_canon(hm.n_instr + 1, 0);
  for (int q = 0; q < hm.n_instr; ++q)
    off_json[q + 1] = off_json[q] + (2 * hm.phi_l1[q] + 1) * (2 * hm.phi_l2[q] + 1);
  for (int c = 0; c < hm.n_instr; ++c)
    off_canon[c + 1] = off_canon[c] + (2 * canon[c][0] + 1) * (2 * canon[c][1] + 1);
  std::vector<int> canon_p(hm.n_p, -1);
  for (int q = 0; q < hm.n_instr; ++q) {
    const int n2 = 2 * hm.phi_l2[q] + 1;
    for (int w = off_json[q]; w < off_json[q + 1]; ++w) {
      const int local = w - off_json[q];
      canon_p[w] = off_canon[canon_of_json[q]] + (local / n2) * n2 + local % n2;
    }
  }
  const int G = static_cast<int>(hm.phi_cg.size());
  std::vector<int> ord(G);
  for (int g = 0; g < G; ++g) {
    ord[g] = g;
    if (hm.phi_p[g] < 0 || hm.phi_p[g] >= hm.n_p || hm.phi_lme[g] < 0 || hm.phi_lme[g] >= hm.n_lme)
      throw std::invalid_argument("model file: Phi1 coupling index out of range");
  }
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return hm.phi_lme[a] < hm.phi_lme[b]; });
  pm.cg_fwd_off.assign(hm.n_lme + 1, 0);
  for (int g : ord) {
    pm.cg_fwd_p.push_back(canon_p[hm.phi_p[g]]);
    pm.cg_fwd_v.push_back(static_cast<float>(hm.phi_cg[g]));
    pm.cg_fwd_off[hm.phi_lme[g] + 1] += 1;
  }
  for (int q = 0; q < hm.n_lme; ++q) pm.cg_fwd_off[q + 1] += pm.cg_fwd_off[q];
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return canon_p[hm.phi_p[a]] < canon_p[hm.phi_p[b]]; });
  pm.cg_rev_off.assign(hm.n_p + 1, 0);
  for (int g : ord) {
    pm.cg_rev_lme.push_back(hm.phi_lme[g]);
    pm.cg_rev_v.push_back(static_cast<float>(hm.phi_cg[g]));
    pm.cg_rev_off[canon_p[hm.phi_p[g]] + 1] += 1;
  }
  for (int q = 0; q < hm.n_p; ++q) pm.cg_rev_off[q + 1] += pm.cg_rev_off[q];
  int acc = 0;
  for (int l = 0; l < 4; ++l) {
    pm.lme_off[l] = acc;
    pm.num_e[l] = hm.num_e[l];
    acc += (2 * l + 1) * hm.num_e[l];
  }

  // ---- polynomials ----
  // Canonical layout when the model's monomials are a subset of the generated sets.
  // Monomial factors commute, so each is matched by its sorted index tuple; an exact
  // repeat of an earlier monomial is dropped, as MultivariatePolynomial's ordered map
  // does (multivariate_polynomial.cpp:34-44).
  auto sorted_pack = [](std::vector<int> m) {
    std::sort(m.begin(), m.end());
    return pack_mono(m);
  };
  auto canon_index = [&](int LM, int packed) {
    for (int t = poly::kOffset[LM]; t < poly::kOffset[LM + 1]; ++t)
      if (poly::kMono[t] == packed) return t - poly::kOffset[LM];
    return -1;
  };
  auto map_list = [&](int LM, const std::vector<std::vector<int>>& monos, std::vector<int>& dst) {
    dst.assign(monos.size(), -1);
    for (size_t t = 0; t < monos.size(); ++t) {
      bool repeat = false;
      for (size_t u = 0; u < t; ++u) repeat = repeat || monos[u] == monos[t];
      if (repeat) continue;
      const int c = canon_index(LM, sorted_pack(monos[t]));
      if (c < 0) return false;
      dst[t] = c;
    }
    return true;
  };
  pm.poly_canon =
      ((hm.L_max == 1 || hm.L_max == 2) && hm.nLM == (hm.L_max + 1) * (hm.L_max + 1) && hm.nLM <= poly::kNumLM) ? 1
                                                                                                            : 0;
  std::vector<std::vector<int>> cmap0(hm.nLM);
  std::vector<int> cmap1;
  if (pm.poly_canon) {
    for (int LM = 0; LM < hm.nLM && pm.poly_canon; ++LM)
      if (!map_list(LM, hm.M0_mono[LM], cmap0[LM])) pm.poly_canon = 0;
    if (pm.poly_canon && !map_list(0, hm.M1_mono, cmap1)) pm.poly_canon = 0;
  }
  pm.mono0_off.assign(hm.nLM + 1, 0);
  pm.T0 = 0;
  for (int LM = 0; LM < hm.nLM; ++LM) {
    for (const auto& m : hm.M0_mono[LM]) pm.mono0.push_back(pack_mono(m));
    pm.mono0_off[LM + 1] = static_cast<int>(pm.mono0.size());
    pm.T0 = std::max<int>(pm.T0, hm.M0_mono[LM].size());
  }
  if (pm.poly_canon) {  // coefficient slots: the longest canonical list among the model's LM
    pm.T0 = 0;
    for (int LM = 0; LM < hm.nLM; ++LM) pm.T0 = std::max(pm.T0, poly::kOffset[LM + 1] - poly::kOffset[LM]);
  }
  pm.coef0.assign(static_cast<size_t>(S) * hm.nLM * std::max(pm.T0, 1) * C, 0.0f);
  for (int s = 0; s < S; ++s)
    for (int LM = 0; LM < hm.nLM; ++LM)
      for (int k = 0; k < C; ++k) {
        const auto& v = hm.M0_coef[(static_cast<size_t>(s) * hm.nLM + LM) * C + k];
        for (size_t t = 0; t < v.size(); ++t) {
          const int slot = pm.poly_canon ? cmap0[LM][t] : static_cast<int>(t);
          if (slot < 0) continue;
          float& dst = pm.coef0[((static_cast<size_t>(s) * hm.nLM + LM) * pm.T0 + slot) * C + k];
          dst = pm.poly_canon ? dst + static_cast<float>(v[t]) : static_cast<float>(v[t]);
        }
      }
  for (const auto& m : hm.M1_mono) pm.mono1.push_back(pack_mono(m));
  pm.T1 = pm.poly_canon ? poly::kOffset[1] : static_cast<int>(hm.M1_mono.size());
  pm.coef1.assign(static_cast<size_t>(S) * std::max(pm.T1, 1) * C, 0.0f);
  for (int s = 0; s < S; ++s)
    for (int k = 0; k < C; ++k) {
      const auto& v = hm.M1_coef[static_cast<size_t>(s) * C + k];
      for (size_t t = 0; t < v.size(); ++t) {
        const int slot = pm.poly_canon ? cmap1[t] : static_cast<int>(t);
        if (slot < 0) continue;
        float& dst = pm.coef1[(static_cast<size_t>(s) * pm.T1 + slot) * C + k];
        dst = pm.poly_canon ? dst + static_cast<float>(v[t]) : static_cast<float>(v[t]);
      }
    }

  // ---- channel mixing ----
  auto f32 = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
  auto transpose = [](const std::vector<double>& v, size_t off, int rows, int cols) {
    std::vector<float> t(static_cast<size_t>(rows) * cols);
    for (int a = 0; a < rows; ++a)
      for (int b = 0; b < cols; ++b) t[static_cast<size_t>(b) * rows + a] = static_cast<float>(v[off + static_cast<size_t>(a) * cols + b]);
    return t;
  };
  pm.H1W = f32(hm.H1W);
  pm.H1W_T.clear();
  for (int L = 0; L <= hm.L_max; ++L) {
    auto t = transpose(hm.H1W, static_cast<size_t>(L) * C * C, C, C);
    pm.H1W_T.insert(pm.H1W_T.end(), t.begin(), t.end());
  }
  for (int l = 0; l < 4; ++l) {
    pm.A1W[l] = f32(hm.A1W[l]);
    pm.A1W_T[l] = transpose(hm.A1W[l], 0, hm.num_e[l] * C, C);
  }
  pm.H2W_H1 = f32(hm.H2W_H1);
  pm.H2W_H1_T.clear();
  for (int s = 0; s < S; ++s) {
    auto t = transpose(hm.H2W_H1, static_cast<size_t>(s) * C * C, C, C);
    pm.H2W_H1_T.insert(pm.H2W_H1_T.end(), t.begin(), t.end());
  }
  pm.H2W_M1 = f32(hm.H2W_M1);
  pm.H2W_M1_T = transpose(hm.H2W_M1, 0, C, C);
  pm.ro1 = f32(hm.ro1);
  pm.ro2_w1 = f32(hm.ro2_w1);
  pm.ro2_w2 = f32(hm.ro2_w2);
  pm.ro2_scale = static_cast<float>(hm.ro2_scale);
  pm.n_hidden = hm.n_hidden;
  pm.e0 = f32(hm.e0);
  pm.Z = hm.Z;
  // density-normalisation splines
  for (int layer = 0; layer < 2; ++layer) {
    const bool on = layer == 0 ? hm.A0_scaled : hm.A1_scaled;
    if (!on) continue;
    const double dh = layer == 0 ? hm.A0_h : hm.A1_h;
    const int dK = layer == 0 ? hm.A0_K : hm.A1_K;
    const std::vector<double>& sv = layer == 0 ? hm.A0_sv : hm.A1_sv;
    const std::vector<double>& sd = layer == 0 ? hm.A0_sd : hm.A1_sd;
    require(dK >= 2 && dh > 0.0, "density spline knots");
    pm.dens_scaled[layer] = 1;
    pm.dens_nint[layer] = dK - 1;
    pm.dens_h[layer] = static_cast<float>(dh);
    pm.dens_spl[layer].assign(static_cast<size_t>(hm.npairs) * (dK - 1) * 4, 0.0f);
    for (int pr = 0; pr < hm.npairs; ++pr)
      for (int iv = 0; iv < dK - 1; ++iv) {
        const size_t b = static_cast<size_t>(pr) * dK + iv;
        double c[4];
        hermite(dh, sv[b], sv[b + 1], sd[b], sd[b + 1], c);
        for (int q = 0; q < 4; ++q)
          pm.dens_spl[layer][(static_cast<size_t>(pr) * (dK - 1) + iv) * 4 + q] = static_cast<float>(c[q]);
      }
  }
  if (hm.has_zbl) {
    pm.has_zbl = 1;
    pm.zbl_p = hm.zbl_p;
    for (int q = 0; q < 4; ++q) pm.zbl_c[q] = static_cast<float>(hm.zbl_c[q]);
    pm.zbl_pair.assign(static_cast<size_t>(S) * S * 4, 0.0f);
    for (int a = 0; a < S; ++a)
      for (int b = 0; b < S; ++b) {
        const int Zu = hm.Z[a], Zv = hm.Z[b];
        if (Zu < 0 || Zv < 0 || Zu >= static_cast<int>(hm.zbl_radii.size()) ||
            Zv >= static_cast<int>(hm.zbl_radii.size()))
          throw std::invalid_argument("model file: zbl_covalent_radii does not cover the model's atomic numbers");
        // zbl.cpp:22-40: a = a_prefactor * 0.529 / (Zu^a_exp + Zv^a_exp), r_max = rcov_u + rcov_v
        const double a_len = hm.zbl_a_pref * 0.529 / (std::pow(double(Zu), hm.zbl_a_exp) + std::pow(double(Zv), hm.zbl_a_exp));
        float* q = &pm.zbl_pair[(static_cast<size_t>(a) * S + b) * 4];
        q[0] = static_cast<float>(1.0 / a_len);
        q[1] = static_cast<float>(0.5 * 14.3996 * Zu * Zv);
        q[2] = static_cast<float>(hm.zbl_radii[Zu] + hm.zbl_radii[Zv]);
        q[3] = 0.0f;
      }
  }
  return pm;
}

}  // namespace smx
