// ORACLE — test infrastructure only.  A float64 CPU restatement of libsymmetrix's
// MACE evaluator (libsymmetrix/source/mace.cpp) that the GPU engine is checked
// against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// load this library; the GPU engine never links or calls it.
//
// Parity is pinned two ways: against the reference's own evaluator compiled from
// its unchanged sources (oracle/_ref, built by oracle/build.py where the reference
// tree is present), and against committed golden outputs of that build
// (tests/golden).  Each stage below cites the reference function it restates.
//
// Layouts are the reference's: Y[E][16], Y_grad[E][3][16], R0[E][(l_max+1)C],
// R1[E][n_instr C], A0/A1[N][16][C], M0/H1[N][LM][C], Phi1r[N][P][C],
// Phi1[N][num_lme][C], M1/H2[N][C], node_energies[N], node_forces[3E]
// (node_forces = -dE/dxyz per directed edge).
//
// Thread safety: one Oracle object per thread; objects share nothing.  One object may
// itself split each stage over node ranges (orc_set_threads); its results are the same
// bits whatever the thread count.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <exception>
#include <thread>
#include <vector>

#include "nlohmann/json.hpp"

namespace {

using vecd = std::vector<double>;
using veci = std::vector<int>;

thread_local std::string g_err;

// Hermite cubic spline set on uniform knots r_n = n h, coefficients per
// interval c[(4 i + p) * ns + s] (cubic_spline_set.cpp:5-25).
struct SplineSet {
  double h = 0;
  int ns = 0, nint = 0;
  vecd c;
  void build(double h_, const std::vector<vecd>& v, const std::vector<vecd>& d) {
    h = h_;
    ns = static_cast<int>(v.size());
    nint = static_cast<int>(v[0].size()) - 1;
    c.assign(4 * static_cast<size_t>(nint) * ns, 0.0);
    for (int i = 0; i < nint; ++i)
      for (int s = 0; s < ns; ++s) {
        const double y0 = v[s][i], y1 = v[s][i + 1], d0 = d[s][i], d1 = d[s][i + 1];
        c[(4 * i + 0) * ns + s] = y0;
        c[(4 * i + 1) * ns + s] = d0;
        c[(4 * i + 2) * ns + s] = (3 * (y1 - y0) - h * (2 * d0 + d1)) / (h * h);
        c[(4 * i + 3) * ns + s] = (2 * (y0 - y1) + h * (d0 + d1)) / (h * h * h);
      }
  }
  // value and derivative of every spline at r (cubic_spline_set.cpp:50-84)
  void eval(double r, double* val, double* der) const {
    const int i = static_cast<int>(r / h);
    if (i < 0 || i >= nint) throw std::invalid_argument("radial spline evaluated outside [0, r_cut)");
    const double x = r - h * i;
    const double* c0 = c.data() + 4 * static_cast<size_t>(i) * ns;
    const double *c1 = c0 + ns, *c2 = c1 + ns, *c3 = c2 + ns;
    for (int s = 0; s < ns; ++s) {
      val[s] = c0[s] + x * (c1[s] + x * (c2[s] + x * c3[s]));
      der[s] = c1[s] + x * (2 * c2[s] + 3 * x * c3[s]);
    }
  }
};

// Scalar spline with the bounds check of cubic_spline.cpp:15-41.
struct Spline1 {
  SplineSet s;
  void build(double h, const vecd& v, const vecd& d) { s.build(h, {v}, {d}); }
  void eval(double r, double& f, double& g) const {
    const int i = static_cast<int>(r / s.h);
    if (i < 0 || i >= s.nint) throw std::invalid_argument("Out of bounds in CubicSpline::evaluate.");
    s.eval(r, &f, &g);
  }
};

// Sum of c_t * prod(x[m_t]) over monomials with its gradient; the reference
// evaluates the same polynomial through a product DAG
// (multivariate_polynomial.cpp:10-127).
struct Poly {
  std::vector<veci> mono;  // shared by all channels/species of one output
};

double poly_eval(const Poly& P, const double* coef, const double* x, double* g, int nv) {
  double f = 0.0;
  for (int a = 0; a < nv; ++a) g[a] = 0.0;
  for (size_t t = 0; t < P.mono.size(); ++t) {
    const veci& m = P.mono[t];
    double prod = 1.0;
    for (int v : m) prod *= x[v];
    f += coef[t] * prod;
    for (size_t q = 0; q < m.size(); ++q) {
      double d = coef[t];
      for (size_t u = 0; u < m.size(); ++u)
        if (u != q) d *= x[m[u]];
      g[m[q]] += d;
    }
  }
  return f;
}

// Real spherical harmonics of the unit vector, e3nn ordering and normalisation
// (mace.cpp:118-148: axis shuffle (x,y,z)->(z,x,y), orthonormal real Y_lm,
// times 2 sqrt(pi)); gradient with respect to the raw edge vector.
void sph_harm(const double* v, double* Y, double* G /*[3][16]*/) {
  const double pi = 3.14159265358979323846;
  const double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  // shuffled unit vector (X, Y, Z) = (z, x, y)
  const double u[3] = {v[2] / r, v[0] / r, v[1] / r};
  const double X = u[0], Yv = u[1], Z = u[2];
  const double s = 2.0 * std::sqrt(pi);
  const double c0 = 0.5 / std::sqrt(pi), c1 = std::sqrt(3.0 / (4.0 * pi));
  const double c2a = 0.5 * std::sqrt(15.0 / pi), c2b = 0.25 * std::sqrt(5.0 / pi),
               c2c = 0.25 * std::sqrt(15.0 / pi);
  const double c3a = 0.25 * std::sqrt(35.0 / (2.0 * pi)), c3b = 0.5 * std::sqrt(105.0 / pi),
               c3c = 0.25 * std::sqrt(21.0 / (2.0 * pi)), c3d = 0.25 * std::sqrt(7.0 / pi),
               c3e = 0.25 * std::sqrt(105.0 / pi);
  double P[16], D[3][16] = {};
  const double XX = X * X, YY = Yv * Yv, ZZ = Z * Z;
  P[0] = c0;
  P[1] = c1 * Yv; D[1][1] = c1;
  P[2] = c1 * Z;  D[2][2] = c1;
  P[3] = c1 * X;  D[0][3] = c1;
  P[4] = c2a * X * Yv; D[0][4] = c2a * Yv; D[1][4] = c2a * X;
  P[5] = c2a * Yv * Z; D[1][5] = c2a * Z; D[2][5] = c2a * Yv;
  P[6] = c2b * (2 * ZZ - XX - YY); D[0][6] = -2 * c2b * X; D[1][6] = -2 * c2b * Yv; D[2][6] = 4 * c2b * Z;
  P[7] = c2a * X * Z; D[0][7] = c2a * Z; D[2][7] = c2a * X;
  P[8] = c2c * (XX - YY); D[0][8] = 2 * c2c * X; D[1][8] = -2 * c2c * Yv;
  P[9] = c3a * (3 * XX * Yv - YY * Yv); D[0][9] = 6 * c3a * X * Yv; D[1][9] = c3a * (3 * XX - 3 * YY);
  P[10] = c3b * X * Yv * Z; D[0][10] = c3b * Yv * Z; D[1][10] = c3b * X * Z; D[2][10] = c3b * X * Yv;
  P[11] = c3c * Yv * (4 * ZZ - XX - YY);
  D[0][11] = -2 * c3c * X * Yv; D[1][11] = c3c * (4 * ZZ - XX - 3 * YY); D[2][11] = 8 * c3c * Yv * Z;
  P[12] = c3d * Z * (2 * ZZ - 3 * XX - 3 * YY);
  D[0][12] = -6 * c3d * X * Z; D[1][12] = -6 * c3d * Yv * Z; D[2][12] = c3d * (6 * ZZ - 3 * XX - 3 * YY);
  P[13] = c3c * X * (4 * ZZ - XX - YY);
  D[0][13] = c3c * (4 * ZZ - 3 * XX - YY); D[1][13] = -2 * c3c * X * Yv; D[2][13] = 8 * c3c * X * Z;
  P[14] = c3e * Z * (XX - YY); D[0][14] = 2 * c3e * X * Z; D[1][14] = -2 * c3e * Yv * Z; D[2][14] = c3e * (XX - YY);
  P[15] = c3a * (XX * X - 3 * X * YY); D[0][15] = c3a * (3 * XX - 3 * YY); D[1][15] = -6 * c3a * X * Yv;
  for (int lm = 0; lm < 16; ++lm) Y[lm] = s * P[lm];
  // gradient in shuffled axes, then back to (x,y,z): d/dx = d/dY', d/dy = d/dZ', d/dz = d/dX'
  for (int l = 0; l <= 3; ++l)
    for (int lm = l * l; lm < (l + 1) * (l + 1); ++lm) {
      double gs[3];
      for (int a = 0; a < 3; ++a) gs[a] = s * (D[a][lm] - l * P[lm] * u[a]) / r;
      G[0 * 16 + lm] = gs[1];
      G[1 * 16 + lm] = gs[2];
      G[2 * 16 + lm] = gs[0];
    }
}

// ZBL pair repulsion (zbl.cpp:22-94).
struct Zbl {
  double a_exp = 0, a_pref = 0;
  vecd c, radii;
  int p = 6;
  static constexpr double ce[4] = {-3.2, -0.9423, -0.4028, -0.2016};
  static constexpr double vpref = 14.3996;
  static double envelope(double r, double rm, int p, double* dr) {
    if (r >= rm) {
      if (dr) *dr = 0.0;
      return 0.0;
    }
    const double x = r / rm;
    if (dr)
      *dr = (-(p + 1.0) * (p + 2.0) / 2.0 * p * std::pow(x, p - 1) + p * (p + 2.0) * (p + 1.0) * std::pow(x, p) -
             p * (p + 1.0) / 2.0 * (p + 2.0) * std::pow(x, p + 1)) / rm;
    return 1.0 - (p + 1.0) * (p + 2.0) / 2.0 * std::pow(x, p) + p * (p + 2.0) * std::pow(x, p + 1) -
           p * (p + 1.0) / 2.0 * std::pow(x, p + 2);
  }
  double energy(int Zu, int Zv, double r, double* dr) const {
    const double a = a_pref * 0.529 / (std::pow(double(Zu), a_exp) + std::pow(double(Zv), a_exp));
    double phi = 0, dphi = 0;
    for (int q = 0; q < 4; ++q) {
      const double e = c[q] * std::exp(ce[q] * r / a);
      phi += e;
      dphi += ce[q] * e / a;
    }
    const double v = vpref * Zu * Zv / r * phi;
    const double dv = vpref * Zu * Zv * (r * dphi - phi) / (r * r);
    double denv = 0;
    const double env = envelope(r, radii[Zu] + radii[Zv], p, &denv);
    if (dr) *dr = 0.5 * (v * denv + dv * env);
    return 0.5 * v * env;
  }
};

struct Oracle {
  // ----- model (mace.cpp:905-1030) -----
  int S = 0, C = 0, l_max = 0, nlm = 0, L_max = 0, nLM = 0;
  double r_cut = 0;
  veci Z;
  vecd e0;
  bool has_zbl = false;
  Zbl zbl;
  std::vector<SplineSet> spl0, spl1;
  vecd H0w;                      // [S][C]
  std::vector<std::vector<vecd>> A0w;  // [S][l][C*C]
  bool A0_scaled = false, A1_scaled = false;
  std::vector<Spline1> A0s, A1s;
  std::vector<Poly> P0;          // [LM]
  vecd P0c;                      // [S][LM][C][t_max0]
  int t_max0 = 0;
  vecd H1w;                      // [L][C*C]
  veci phi_l, phi_l1, phi_l2, phi_lme, phi_p;
  vecd phi_cg;
  int n_lme = 0, n_p = 0;
  veci num_e;
  std::vector<vecd> A1w;         // [l][n_e*C*C]
  Poly P1;
  vecd P1c;                      // [S][C][t_max1]
  int t_max1 = 0;
  std::vector<vecd> H2w_H1;      // [S][C*C]
  vecd H2w_M1, ro1, ro2_w1, ro2_w2;
  double ro2_scale = 1.0;

  // ----- per-call buffers (mace.hpp:27-145) -----
  vecd node_energies, node_forces, Y, Y_grad, R0, R0_deriv, R1, R1_deriv, A0, A0_adj, M0, M0_grad, M0_adj,
      H1, H1_adj, Phi1r, dPhi1r, Phi1, dPhi1, A1, A1_adj, M1, M1_grad, M1_adj, H2, H2_adj;

  int pair_index(int a, int b) const {
    if (a > b) std::swap(a, b);
    return a * (2 * S - a - 1) / 2 + b;
  }

  void load(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open model file " + path);
    nlohmann::json j = nlohmann::json::parse(f);
    S = j["num_elements"].get<int>();
    C = j["num_channels"].get<int>();
    r_cut = j["r_cut"].get<double>();
    l_max = j["l_max"].get<int>();
    L_max = j["L_max"].get<int>();
    if (l_max != 3) throw std::invalid_argument("l_max must be 3");
    nlm = (l_max + 1) * (l_max + 1);
    nLM = (L_max + 1) * (L_max + 1);
    Z = j["atomic_numbers"].get<veci>();
    e0 = j["atomic_energies"].get<vecd>();
    has_zbl = j["has_zbl"].get<bool>();
    if (has_zbl) {
      zbl.a_exp = j["zbl_a_exp"].get<double>();
      zbl.a_pref = j["zbl_a_prefactor"].get<double>();
      zbl.c = j["zbl_c"].get<vecd>();
      zbl.radii = j["zbl_covalent_radii"].get<vecd>();
      zbl.p = j["zbl_p"].get<int>();
    }
    const double h = j["radial_spline_h"].get<double>();
    auto v0 = j["radial_spline_values_0"].get<std::vector<std::vector<vecd>>>();
    auto d0 = j["radial_spline_derivs_0"].get<std::vector<std::vector<vecd>>>();
    auto v1 = j["radial_spline_values_1"].get<std::vector<std::vector<vecd>>>();
    auto d1 = j["radial_spline_derivs_1"].get<std::vector<std::vector<vecd>>>();
    spl0.resize(v0.size());
    spl1.resize(v1.size());
    for (size_t p = 0; p < v0.size(); ++p) spl0[p].build(h, v0[p], d0[p]);
    for (size_t p = 0; p < v1.size(); ++p) spl1[p].build(h, v1[p], d1[p]);
    H0w = j["H0_weights"].get<vecd>();
    A0w = j["A0_weights"].get<std::vector<std::vector<vecd>>>();
    A0_scaled = j["A0_scaled"].get<bool>();
    if (A0_scaled) {
      const double hh = j["A0_spline_h"].get<double>();
      auto vv = j["A0_spline_values"].get<std::vector<vecd>>();
      auto dd = j["A0_spline_derivs"].get<std::vector<vecd>>();
      A0s.resize(vv.size());
      for (size_t p = 0; p < vv.size(); ++p) A0s[p].build(hh, vv[p], dd[p]);
    }
    // polynomials (mace.cpp:956-973)
    auto m0w = j["M0_weights"].get<std::map<std::string, std::map<std::string, std::map<std::string, vecd>>>>();
    auto m0m = j["M0_monomials"].get<std::map<std::string, std::vector<veci>>>();
    P0.resize(nLM);
    t_max0 = 0;
    for (int LM = 0; LM < nLM; ++LM) {
      P0[LM].mono = m0m.at(std::to_string(LM));
      t_max0 = std::max<int>(t_max0, P0[LM].mono.size());
    }
    P0c.assign(static_cast<size_t>(S) * nLM * C * t_max0, 0.0);
    for (int s = 0; s < S; ++s)
      for (int LM = 0; LM < nLM; ++LM)
        for (int k = 0; k < C; ++k) {
          const vecd& cf = m0w.at(std::to_string(s)).at(std::to_string(LM)).at(std::to_string(k));
          if (cf.size() != P0[LM].mono.size()) throw std::invalid_argument("M0 coefficient/monomial mismatch");
          std::copy(cf.begin(), cf.end(), P0c.begin() + ((static_cast<size_t>(s) * nLM + LM) * C + k) * t_max0);
        }
    H1w = j["H1_weights"].get<vecd>();
    phi_l = j["Phi1_l"].get<veci>();
    phi_l1 = j["Phi1_l1"].get<veci>();
    phi_l2 = j["Phi1_l2"].get<veci>();
    phi_lme = j["Phi1_lme"].get<veci>();
    phi_cg = j["Phi1_clebsch_gordan"].get<vecd>();
    phi_p = j["Phi1_lelm1lm2"].get<veci>();
    n_lme = 0;
    n_p = 0;
    num_e.assign(l_max + 1, 0);
    for (size_t q = 0; q < phi_l.size(); ++q) {
      n_lme += 2 * phi_l[q] + 1;
      n_p += (2 * phi_l1[q] + 1) * (2 * phi_l2[q] + 1);
      num_e[phi_l[q]] += 1;
    }
    A1w = j["A1_weights"].get<std::vector<vecd>>();
    A1_scaled = j["A1_scaled"].get<bool>();
    if (A1_scaled) {
      const double hh = j["A1_spline_h"].get<double>();
      auto vv = j["A1_spline_values"].get<std::vector<vecd>>();
      auto dd = j["A1_spline_derivs"].get<std::vector<vecd>>();
      A1s.resize(vv.size());
      for (size_t p = 0; p < vv.size(); ++p) A1s[p].build(hh, vv[p], dd[p]);
    }
    auto m1w = j["M1_weights"].get<std::map<std::string, std::map<std::string, vecd>>>();
    P1.mono = j["M1_monomials"].get<std::vector<veci>>();
    t_max1 = static_cast<int>(P1.mono.size());
    P1c.assign(static_cast<size_t>(S) * C * t_max1, 0.0);
    for (int s = 0; s < S; ++s)
      for (int k = 0; k < C; ++k) {
        const vecd& cf = m1w.at(std::to_string(s)).at(std::to_string(k));
        if (static_cast<int>(cf.size()) != t_max1) throw std::invalid_argument("M1 coefficient/monomial mismatch");
        std::copy(cf.begin(), cf.end(), P1c.begin() + (static_cast<size_t>(s) * C + k) * t_max1);
      }
    H2w_H1 = j["H2_weights_for_H1"].get<std::vector<vecd>>();
    H2w_M1 = j["H2_weights_for_M1"].get<vecd>();
    ro1 = j["readout_1_weights"].get<vecd>();
    ro2_w1 = j["readout_2_weights_1"].get<vecd>();
    ro2_w2 = j["readout_2_weights_2"].get<vecd>();
    ro2_scale = j["readout_2_scale_factor"].get<double>();
  }

  // ----- parallel loops over node ranges -----
  // Every stage's work for node i (and its edges) is independent of the other nodes,
  // except the H1_adj scatter of reverse_Phi1, which is done as a gather over each
  // node's incoming edges in ascending edge order.  Each element is therefore computed
  // by the same operations in the same order as in a serial run: results do not
  // depend on the thread count, bit for bit.
  int nthreads = 1;
  std::vector<long> eoff;  // [N+1] first edge of each node
  // lean: the radials R0, R1 and their derivatives are not stored per edge (the
  // reference's layout, ~20 KB per edge) but evaluated where each stage needs them, by
  // the same spline code: the same numbers, in far less memory (large boxes)
  bool lean = false;
  // R, R' of edge e (centre type ti, neighbour type tj): the stored row, or (lean) the
  // spline evaluated into the caller's buffers
  void radial_row(const std::vector<SplineSet>& spl, const vecd& R, const vecd& Rd, int ti, int tj, long e, double r,
                  double* bR, double* bRd, const double*& pR, const double*& pRd) const {
    const size_t ns = spl[0].ns;
    if (!lean) {
      pR = &R[e * ns];
      pRd = &Rd[e * ns];
      return;
    }
    spl[pair_index(ti, tj)].eval(r, bR, bRd);
    pR = bR;
    pRd = bRd;
  }
  template <typename F>
  void par_nodes(int N, F&& f) {  // f(i0, i1) over disjoint node ranges
    const int T = std::max(1, std::min(nthreads, N / 4));
    if (T <= 1) {
      f(0, N);
      return;
    }
    std::vector<std::thread> th;
    std::vector<std::exception_ptr> err(T);
    for (int t = 0; t < T; ++t)
      th.emplace_back([&, t] {
        try {
          f(static_cast<int>(static_cast<long>(N) * t / T), static_cast<int>(static_cast<long>(N) * (t + 1) / T));
        } catch (...) {
          err[t] = std::current_exception();
        }
      });
    for (auto& x : th) x.join();
    for (auto& e : err)
      if (e) std::rethrow_exception(e);
  }

  // ----- forward + reverse (mace.cpp:17-64) -----
  // N1 < N: layer 0 over all N nodes, layer 1, the readouts and ZBL over the first N1
  // only, as the pair style's no-MPI-message-passing mode calls the stages
  // (pair_symmetrix/pair_symmetrix_mace.cpp:672-698): the trailing N - N1 nodes are a
  // halo whose H1 rows the first N1 nodes' layer-1 edges read; node_energies has N1
  // entries and node_forces one triple per edge of all N nodes.
  void compute(int N, const int* ntype, const int* nneigh, const int* nidx, const int* ntypes_e, long E,
               const double* xyz, const double* r, int N1 = -1) {
    if (N1 < 0) N1 = N;
    if (N1 > N) throw std::invalid_argument("more layer-1 nodes than nodes");
    long check = 0;
    for (int i = 0; i < N; ++i) check += nneigh[i];
    if (check != E) throw std::invalid_argument("sum(num_neigh) != number of edges");
    eoff.assign(N + 1, 0);
    for (int i = 0; i < N; ++i) eoff[i + 1] = eoff[i] + nneigh[i];
    for (long e = 0; e < eoff[N1]; ++e)  // the halo's own edges index nothing
      if (nidx[e] < 0 || nidx[e] >= N) throw std::invalid_argument("neighbor index out of range");
    node_energies.assign(N1, 0.0);
    node_forces.assign(3 * E, 0.0);
    if (has_zbl) zbl_stage(N1, ntype, ntypes_e, xyz, r);
    stage_Y(N, E, xyz);
    stage_R(N, ntype, ntypes_e, r, spl0, R0, R0_deriv);
    stage_A0(N, ntype, ntypes_e, r);
    scale_fwd(N, ntype, ntypes_e, r, A0_scaled, A0s, A0);
    stage_M0(N, ntype);
    stage_H1(N);
    stage_R(N1, ntype, ntypes_e, r, spl1, R1, R1_deriv);
    stage_Phi1(N1, ntype, nidx, ntypes_e, r);
    stage_A1(N1);
    scale_fwd(N1, ntype, ntypes_e, r, A1_scaled, A1s, A1);
    stage_M1(N1, ntype);
    stage_H2(N1, ntype);
    stage_readouts(N1, ntype);
    reverse_H2(N1, ntype);
    reverse_M1(N1);
    scale_rev(N1, ntype, ntypes_e, xyz, r, A1_scaled, A1s, A1, A1_adj);
    reverse_A1(N1);
    reverse_Phi1(N1, ntype, nidx, ntypes_e, xyz, r);
    reverse_H1(N);
    reverse_M0(N);
    scale_rev(N, ntype, ntypes_e, xyz, r, A0_scaled, A0s, A0, A0_adj);
    reverse_A0(N, ntype, ntypes_e, xyz, r);
  }

  // zbl.cpp:96-125
  void zbl_stage(int N, const int* ntype, const int* te, const double* xyz, const double* r) {
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i)
        for (long e = eoff[i]; e < eoff[i + 1]; ++e) {
          double g = 0;
          node_energies[i] += zbl.energy(Z[ntype[i]], Z[te[e]], r[e], &g);
          for (int a = 0; a < 3; ++a) node_forces[3 * e + a] -= xyz[3 * e + a] / r[e] * g;
        }
    });
  }

  // mace.cpp:118-148
  void stage_Y(int N, long E, const double* xyz) {
    Y.assign(E * nlm, 0.0);
    Y_grad.assign(3 * E * nlm, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      for (long e = eoff[i0]; e < eoff[i1]; ++e) sph_harm(xyz + 3 * e, &Y[e * nlm], &Y_grad[3 * e * nlm]);
    });
  }

  // mace.cpp:66-116
  void stage_R(int N, const int* ntype, const int* te, const double* r, const std::vector<SplineSet>& spl, vecd& R,
               vecd& Rd) {
    const int ns = spl[0].ns;
    const long E = eoff[N];
    if (lean) {
      R.clear();
      Rd.clear();
      return;
    }
    R.assign(E * ns, 0.0);
    Rd.assign(E * ns, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i)
        for (long e = eoff[i]; e < eoff[i + 1]; ++e)
          spl[pair_index(ntype[i], te[e])].eval(r[e], &R[e * ns], &Rd[e * ns]);
    });
  }

  // mace.cpp:150-201: Phi0 = sum_j R0 Y H0[type_j], then per-l channel mixing
  void stage_A0(int N, const int* ntype, const int* te, const double* r) {
    A0.assign(static_cast<size_t>(N) * nlm * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      vecd phi0(nlm * C), bR(spl0[0].ns), bRd(spl0[0].ns);
      for (int i = i0; i < i1; ++i) {
        std::fill(phi0.begin(), phi0.end(), 0.0);
        for (long e = eoff[i]; e < eoff[i + 1]; ++e) {
          const double* h0 = &H0w[te[e] * C];
          const double *R0e, *R0de;
          radial_row(spl0, R0, R0_deriv, ntype[i], te[e], e, r[e], bR.data(), bRd.data(), R0e, R0de);
          for (int l = 0; l <= l_max; ++l) {
            const double* rl = R0e + l * C;
            for (int lm = l * l; lm < (l + 1) * (l + 1); ++lm) {
              const double y = Y[e * nlm + lm];
              for (int k = 0; k < C; ++k) phi0[lm * C + k] += rl[k] * y * h0[k];
            }
          }
        }
        for (int l = 0; l <= l_max; ++l) {
          const double* W = A0w[ntype[i]][l].data();
          for (int lm = l * l; lm < (l + 1) * (l + 1); ++lm)
            for (int k = 0; k < C; ++k) {
              double s = 0;
              for (int kk = 0; kk < C; ++kk) s += phi0[lm * C + kk] * W[kk * C + k];
              A0[(static_cast<size_t>(i) * nlm + lm) * C + k] = s;
            }
        }
      }
    });
  }

  // mace.cpp:273-297 / :681-705
  void scale_fwd(int N, const int* ntype, const int* te, const double* r, bool on, const std::vector<Spline1>& sp,
                 vecd& A) {
    if (!on) return;
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i) {
        double s = 1.0;
        for (long e = eoff[i]; e < eoff[i + 1]; ++e) {
          double f, g;
          sp[pair_index(ntype[i], te[e])].eval(r[e], f, g);
          s += f;
        }
        for (int x = 0; x < nlm * C; ++x) A[static_cast<size_t>(i) * nlm * C + x] /= s;
      }
    });
  }

  // mace.cpp:299-346 / :707-757
  void scale_rev(int N, const int* ntype, const int* te, const double* xyz, const double* r, bool on,
                 const std::vector<Spline1>& sp, const vecd& A, vecd& Aadj) {
    if (!on) return;
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i) {
        double s = 1.0;
        for (long e = eoff[i]; e < eoff[i + 1]; ++e) {
          double f, g;
          sp[pair_index(ntype[i], te[e])].eval(r[e], f, g);
          s += f;
        }
        double dot = 0;
        for (int x = 0; x < nlm * C; ++x)
          dot += Aadj[static_cast<size_t>(i) * nlm * C + x] * A[static_cast<size_t>(i) * nlm * C + x];
        for (long e = eoff[i]; e < eoff[i + 1]; ++e) {
          double f, g;
          sp[pair_index(ntype[i], te[e])].eval(r[e], f, g);
          for (int a = 0; a < 3; ++a) node_forces[3 * e + a] += dot / s * g * xyz[3 * e + a] / r[e];
        }
        for (int x = 0; x < nlm * C; ++x) Aadj[static_cast<size_t>(i) * nlm * C + x] /= s;
      }
    });
  }

  // mace.cpp:348-370: per (i, LM, k) polynomial of A0[i, :, k], with gradient
  void stage_M0(int N, const int* ntype) {
    M0.assign(static_cast<size_t>(N) * nLM * C, 0.0);
    M0_grad.assign(static_cast<size_t>(N) * nLM * nlm * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      double x[16], g[16];
      for (int i = i0; i < i1; ++i)
        for (int LM = 0; LM < nLM; ++LM)
          for (int k = 0; k < C; ++k) {
            for (int v = 0; v < nlm; ++v) x[v] = A0[(static_cast<size_t>(i) * nlm + v) * C + k];
            const double* cf = &P0c[((static_cast<size_t>(ntype[i]) * nLM + LM) * C + k) * t_max0];
            M0[(static_cast<size_t>(i) * nLM + LM) * C + k] = poly_eval(P0[LM], cf, x, g, nlm);
            for (int v = 0; v < nlm; ++v)
              M0_grad[((static_cast<size_t>(i) * nLM + LM) * nlm + v) * C + k] = g[v];
          }
    });
  }

  // mace.cpp:372-395
  void reverse_M0(int N) {
    A0_adj.assign(static_cast<size_t>(N) * nlm * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i)
        for (int v = 0; v < nlm; ++v)
          for (int LM = 0; LM < nLM; ++LM)
            for (int k = 0; k < C; ++k)
              A0_adj[(static_cast<size_t>(i) * nlm + v) * C + k] +=
                  M0_grad[((static_cast<size_t>(i) * nLM + LM) * nlm + v) * C + k] *
                  M0_adj[(static_cast<size_t>(i) * nLM + LM) * C + k];
    });
  }

  // rows of block L of X[N][nLM][C] times W_L (C x C), optionally transposed (mace.cpp:397-451)
  void mix(int N, const vecd& X, vecd& Yo, const vecd& W, int Lmax, int nrows, bool trans) {
    Yo.assign(X.size(), 0.0);
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i)
        for (int L = 0; L <= Lmax; ++L) {
          const double* w = &W[static_cast<size_t>(L) * C * C];
          for (int LM = L * L; LM < (L + 1) * (L + 1); ++LM) {
            const double* xr = &X[(static_cast<size_t>(i) * nrows + LM) * C];
            double* yr = &Yo[(static_cast<size_t>(i) * nrows + LM) * C];
            for (int k = 0; k < C; ++k) {
              double s = 0;
              for (int kk = 0; kk < C; ++kk) s += xr[kk] * (trans ? w[k * C + kk] : w[kk * C + k]);
              yr[k] = s;
            }
          }
        }
    });
  }
  void stage_H1(int N) { mix(N, M0, H1, H1w, L_max, nLM, false); }
  void reverse_H1(int N) { mix(N, H1_adj, M0_adj, H1w, L_max, nLM, true); }

  // mace.cpp:453-502
  void stage_Phi1(int N, const int* ntype, const int* nidx, const int* te, const double* r) {
    Phi1r.assign(static_cast<size_t>(N) * n_p * C, 0.0);
    Phi1.assign(static_cast<size_t>(N) * n_lme * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      vecd bR(spl1[0].ns), bRd(spl1[0].ns);
      for (int i = i0; i < i1; ++i) {
        double* out = &Phi1r[static_cast<size_t>(i) * n_p * C];
        for (long e = eoff[i]; e < eoff[i + 1]; ++e) {
          const double* hj = &H1[static_cast<size_t>(nidx[e]) * nLM * C];
          const double *R1e, *R1de;
          radial_row(spl1, R1, R1_deriv, ntype[i], te[e], e, r[e], bR.data(), bRd.data(), R1e, R1de);
          int p = 0;
          for (size_t ins = 0; ins < phi_l.size(); ++ins) {
            const double* R = R1e + ins * C;
            const int l1 = phi_l1[ins], l2 = phi_l2[ins];
            for (int lm1 = l1 * l1; lm1 < (l1 + 1) * (l1 + 1); ++lm1) {
              const double y = Y[e * nlm + lm1];
              for (int lm2 = l2 * l2; lm2 < (l2 + 1) * (l2 + 1); ++lm2, ++p)
                for (int k = 0; k < C; ++k) out[p * C + k] += R[k] * y * hj[lm2 * C + k];
            }
          }
        }
        for (size_t t = 0; t < phi_cg.size(); ++t)
          for (int k = 0; k < C; ++k)
            Phi1[(static_cast<size_t>(i) * n_lme + phi_lme[t]) * C + k] +=
                phi_cg[t] * Phi1r[(static_cast<size_t>(i) * n_p + phi_p[t]) * C + k];
      }
    });
  }

  // mace.cpp:504-605: node_forces of every edge i->j, and H1_adj[j] += R1 Y dPhi1r[i].
  // The H1_adj sums are formed per node j over its incoming edges in ascending edge
  // order, the order a serial pass over the edges adds them in.
  void reverse_Phi1(int N, const int* ntype, const int* nidx, const int* te, const double* xyz, const double* r) {
    const long E = eoff[N];
    dPhi1r.assign(static_cast<size_t>(N) * n_p * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i)
        for (size_t t = 0; t < phi_cg.size(); ++t)
          for (int k = 0; k < C; ++k)
            dPhi1r[(static_cast<size_t>(i) * n_p + phi_p[t]) * C + k] +=
                phi_cg[t] * dPhi1[(static_cast<size_t>(i) * n_lme + phi_lme[t]) * C + k];
    });
    par_nodes(N, [&](int i0, int i1) {
      vecd bR(spl1[0].ns), bRd(spl1[0].ns);
      for (int i = i0; i < i1; ++i) {
        const double* g = &dPhi1r[static_cast<size_t>(i) * n_p * C];
        for (long e = eoff[i]; e < eoff[i + 1]; ++e) {
          const double* hj = &H1[static_cast<size_t>(nidx[e]) * nLM * C];
          const double* u = xyz + 3 * e;
          const double *R1e, *R1de;
          radial_row(spl1, R1, R1_deriv, ntype[i], te[e], e, r[e], bR.data(), bRd.data(), R1e, R1de);
          double f[3] = {0, 0, 0};
          int p = 0;
          for (size_t ins = 0; ins < phi_l.size(); ++ins) {
            const double* R = R1e + ins * C;
            const double* Rd = R1de + ins * C;
            const int l1 = phi_l1[ins], l2 = phi_l2[ins];
            for (int lm1 = l1 * l1; lm1 < (l1 + 1) * (l1 + 1); ++lm1) {
              const double y = Y[e * nlm + lm1];
              const double gy[3] = {Y_grad[(3 * e + 0) * nlm + lm1], Y_grad[(3 * e + 1) * nlm + lm1],
                                    Y_grad[(3 * e + 2) * nlm + lm1]};
              for (int lm2 = l2 * l2; lm2 < (l2 + 1) * (l2 + 1); ++lm2, ++p)
                for (int k = 0; k < C; ++k) {
                  const double gh = g[p * C + k] * hj[lm2 * C + k];
                  for (int a = 0; a < 3; ++a) f[a] -= gh * (u[a] / r[e] * Rd[k] * y + R[k] * gy[a]);
                }
            }
          }
          for (int a = 0; a < 3; ++a) node_forces[3 * e + a] += f[a];
        }
      }
    });
    // incoming edges of every node with an H1 row (the halo's too), ascending, and each
    // edge's source node
    const int NH = static_cast<int>(H1.size() / (static_cast<size_t>(nLM) * C));
    std::vector<long> in_off(NH + 1, 0), in_e(E);
    std::vector<int> src(E);
    for (int i = 0; i < N; ++i)
      for (long e = eoff[i]; e < eoff[i + 1]; ++e) {
        src[e] = i;
        ++in_off[nidx[e] + 1];
      }
    for (int j = 0; j < NH; ++j) in_off[j + 1] += in_off[j];
    {
      std::vector<long> fill(in_off.begin(), in_off.end() - 1);
      for (long e = 0; e < E; ++e) in_e[fill[nidx[e]]++] = e;
    }
    par_nodes(NH, [&](int j0, int j1) {
      vecd bR(spl1[0].ns), bRd(spl1[0].ns);
      for (int j = j0; j < j1; ++j) {
        double* aj = &H1_adj[static_cast<size_t>(j) * nLM * C];
        for (long q = in_off[j]; q < in_off[j + 1]; ++q) {
          const long e = in_e[q];
          const double* g = &dPhi1r[static_cast<size_t>(src[e]) * n_p * C];
          const double *R1e, *R1de;
          radial_row(spl1, R1, R1_deriv, ntype[src[e]], te[e], e, r[e], bR.data(), bRd.data(), R1e, R1de);
          int p = 0;
          for (size_t ins = 0; ins < phi_l.size(); ++ins) {
            const double* R = R1e + ins * C;
            const int l1 = phi_l1[ins], l2 = phi_l2[ins];
            for (int lm1 = l1 * l1; lm1 < (l1 + 1) * (l1 + 1); ++lm1) {
              const double y = Y[e * nlm + lm1];
              for (int lm2 = l2 * l2; lm2 < (l2 + 1) * (l2 + 1); ++lm2, ++p)
                for (int k = 0; k < C; ++k) aj[lm2 * C + k] += R[k] * y * g[p * C + k];
            }
          }
        }
      }
    });
  }

  // mace.cpp:607-679: per l, (2l+1) x (n_e C) times (n_e C) x C
  void stage_A1(int N) {
    A1.assign(static_cast<size_t>(N) * nlm * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i) {
        const double* ph = &Phi1[static_cast<size_t>(i) * n_lme * C];
        double* a = &A1[static_cast<size_t>(i) * nlm * C];
        for (int l = 0; l <= l_max; ++l) {
          const int K = num_e[l] * C;
          for (int m = 0; m < 2 * l + 1; ++m)
            for (int k = 0; k < C; ++k) {
              double s = 0;
              for (int kk = 0; kk < K; ++kk) s += ph[m * K + kk] * A1w[l][static_cast<size_t>(kk) * C + k];
              a[m * C + k] = s;
            }
          ph += (2 * l + 1) * K;
          a += (2 * l + 1) * C;
        }
      }
    });
  }
  void reverse_A1(int N) {
    dPhi1.assign(static_cast<size_t>(N) * n_lme * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i) {
        const double* a = &A1_adj[static_cast<size_t>(i) * nlm * C];
        double* ph = &dPhi1[static_cast<size_t>(i) * n_lme * C];
        for (int l = 0; l <= l_max; ++l) {
          const int K = num_e[l] * C;
          for (int m = 0; m < 2 * l + 1; ++m)
            for (int kk = 0; kk < K; ++kk) {
              double s = 0;
              for (int k = 0; k < C; ++k) s += a[m * C + k] * A1w[l][static_cast<size_t>(kk) * C + k];
              ph[m * K + kk] = s;
            }
          ph += (2 * l + 1) * K;
          a += (2 * l + 1) * C;
        }
      }
    });
  }

  // mace.cpp:759-794
  void stage_M1(int N, const int* ntype) {
    M1.assign(static_cast<size_t>(N) * C, 0.0);
    M1_grad.assign(static_cast<size_t>(N) * nlm * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      double x[16], g[16];
      for (int i = i0; i < i1; ++i)
        for (int k = 0; k < C; ++k) {
          for (int v = 0; v < nlm; ++v) x[v] = A1[(static_cast<size_t>(i) * nlm + v) * C + k];
          const double* cf = &P1c[(static_cast<size_t>(ntype[i]) * C + k) * t_max1];
          M1[static_cast<size_t>(i) * C + k] = poly_eval(P1, cf, x, g, nlm);
          for (int v = 0; v < nlm; ++v) M1_grad[(static_cast<size_t>(i) * nlm + v) * C + k] = g[v];
        }
    });
  }
  void reverse_M1(int N) {
    A1_adj.assign(static_cast<size_t>(N) * nlm * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i)
        for (int v = 0; v < nlm; ++v)
          for (int k = 0; k < C; ++k)
            A1_adj[(static_cast<size_t>(i) * nlm + v) * C + k] =
                M1_grad[(static_cast<size_t>(i) * nlm + v) * C + k] * M1_adj[static_cast<size_t>(i) * C + k];
    });
  }

  // mace.cpp:796-874: H2 = W_H1[type]^T H1[i,0,:] + W_M1^T M1[i]
  void stage_H2(int N, const int* ntype) {
    H2.assign(static_cast<size_t>(N) * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i) {
        const double* W = H2w_H1[ntype[i]].data();
        for (int c = 0; c < C; ++c) {
          double s = 0;
          for (int rr = 0; rr < C; ++rr)
            s += W[rr * C + c] * H1[static_cast<size_t>(i) * nLM * C + rr] +
                 H2w_M1[rr * C + c] * M1[static_cast<size_t>(i) * C + rr];
          H2[static_cast<size_t>(i) * C + c] = s;
        }
      }
    });
  }
  void reverse_H2(int N, const int* ntype) {
    M1_adj.assign(static_cast<size_t>(N) * C, 0.0);
    par_nodes(N, [&](int i0, int i1) {
      for (int i = i0; i < i1; ++i) {
        const double* W = H2w_H1[ntype[i]].data();
        const double* g = &H2_adj[static_cast<size_t>(i) * C];
        for (int rr = 0; rr < C; ++rr) {
          double s1 = 0, s2 = 0;
          for (int c = 0; c < C; ++c) {
            s1 += W[rr * C + c] * g[c];
            s2 += H2w_M1[rr * C + c] * g[c];
          }
          H1_adj[static_cast<size_t>(i) * nLM * C + rr] += s1;
          M1_adj[static_cast<size_t>(i) * C + rr] = s2;
        }
      }
    });
  }

  // mace.cpp:876-903 and multilayer_perceptron.cpp:76-150 (shape {C, 16, 1})
  void stage_readouts(int N, const int* ntype) {
    H1_adj.assign(H1.size(), 0.0);  // every H1 row, a halo's too (mace.cpp:881-885)
    H2_adj.assign(static_cast<size_t>(N) * C, 0.0);
    const int nh = static_cast<int>(ro2_w2.size());
    par_nodes(N, [&](int i0, int i1) {
      vecd act_d(nh);
      for (int i = i0; i < i1; ++i) {
        double E = e0[ntype[i]];
        for (int k = 0; k < C; ++k) {
          E += ro1[k] * H1[static_cast<size_t>(i) * nLM * C + k];
          H1_adj[static_cast<size_t>(i) * nLM * C + k] = ro1[k];
        }
        const double* x = &H2[static_cast<size_t>(i) * C];
        double out = 0;
        for (int u = 0; u < nh; ++u) {
          double s = 0;
          for (int k = 0; k < C; ++k) s += ro2_w1[u * C + k] * x[k];
          const double sg = 1.0 / (1.0 + std::exp(-s));
          out += ro2_w2[u] * ro2_scale * s * sg;
          act_d[u] = ro2_w2[u] * (ro2_scale * sg + ro2_scale * s * sg * (1 - sg));
        }
        for (int k = 0; k < C; ++k) {
          double g = 0;
          for (int u = 0; u < nh; ++u) g += act_d[u] * ro2_w1[u * C + k];
          H2_adj[static_cast<size_t>(i) * C + k] = g;
        }
        node_energies[i] += E + out;
      }
    });
  }

  // mace.cpp:203-271
  void reverse_A0(int N, const int* ntype, const int* te, const double* xyz, const double* r) {
    par_nodes(N, [&](int i0, int i1) {
      vecd phi_adj(nlm * C), bR(spl0[0].ns), bRd(spl0[0].ns);
      for (int i = i0; i < i1; ++i) {
        for (int l = 0; l <= l_max; ++l) {
          const double* W = A0w[ntype[i]][l].data();
          for (int lm = l * l; lm < (l + 1) * (l + 1); ++lm)
            for (int kk = 0; kk < C; ++kk) {
              double s = 0;
              for (int k = 0; k < C; ++k) s += A0_adj[(static_cast<size_t>(i) * nlm + lm) * C + k] * W[kk * C + k];
              phi_adj[lm * C + kk] = s;
            }
        }
        for (long e = eoff[i]; e < eoff[i + 1]; ++e) {
          const double* h0 = &H0w[te[e] * C];
          const double* u = xyz + 3 * e;
          const double *R0e, *R0de;
          radial_row(spl0, R0, R0_deriv, ntype[i], te[e], e, r[e], bR.data(), bRd.data(), R0e, R0de);
          double f[3] = {0, 0, 0};
          for (int l = 0; l <= l_max; ++l) {
            const double* R = R0e + l * C;
            const double* Rd = R0de + l * C;
            for (int lm = l * l; lm < (l + 1) * (l + 1); ++lm) {
              const double y = Y[e * nlm + lm];
              const double gy[3] = {Y_grad[(3 * e + 0) * nlm + lm], Y_grad[(3 * e + 1) * nlm + lm],
                                    Y_grad[(3 * e + 2) * nlm + lm]};
              for (int k = 0; k < C; ++k) {
                const double ph = phi_adj[lm * C + k] * h0[k];
                for (int a = 0; a < 3; ++a) f[a] -= ph * (u[a] / r[e] * Rd[k] * y + R[k] * gy[a]);
              }
            }
          }
          for (int a = 0; a < 3; ++a) node_forces[3 * e + a] += f[a];
        }
      }
    });
  }

  vecd* buffer(const std::string& n) {
    if (n == "node_energies") return &node_energies;
    if (n == "node_forces") return &node_forces;
    if (n == "Y") return &Y;
    if (n == "Y_grad") return &Y_grad;
    if (n == "R0") return &R0;
    if (n == "R0_deriv") return &R0_deriv;
    if (n == "R1") return &R1;
    if (n == "R1_deriv") return &R1_deriv;
    if (n == "A0") return &A0;
    if (n == "A0_adj") return &A0_adj;
    if (n == "M0") return &M0;
    if (n == "M0_adj") return &M0_adj;
    if (n == "H1") return &H1;
    if (n == "H1_adj") return &H1_adj;
    if (n == "Phi1r") return &Phi1r;
    if (n == "Phi1") return &Phi1;
    if (n == "Phi1_adj") return &dPhi1;
    if (n == "A1") return &A1;
    if (n == "A1_adj") return &A1_adj;
    if (n == "M1") return &M1;
    if (n == "M1_adj") return &M1_adj;
    if (n == "H2") return &H2;
    if (n == "H2_adj") return &H2_adj;
    return nullptr;
  }
};

}  // namespace

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

void* orc_load(const char* path) {
  try {
    auto* o = new Oracle();
    o->load(path);
    return o;
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

void orc_free(void* h) { delete static_cast<Oracle*>(h); }

// An independent evaluator sharing nothing with h (copies the loaded model), so
// several threads can evaluate in parallel without re-reading the model file.
void* orc_clone(void* h) { return new Oracle(*static_cast<Oracle*>(h)); }

// Worker threads one evaluation uses (1: serial).
void orc_set_threads(void* h, int n) { static_cast<Oracle*>(h)->nthreads = n < 1 ? 1 : n; }

// 1: evaluate the radials where they are used instead of storing them per edge (large
// boxes; the R0/R1 stage buffers are then empty).  Same results bit for bit.
void orc_set_lean(void* h, int on) { static_cast<Oracle*>(h)->lean = on != 0; }

int orc_info(void* h, int* out) {
  auto* o = static_cast<Oracle*>(h);
  out[0] = o->S;
  out[1] = o->C;
  out[2] = o->l_max;
  out[3] = o->L_max;
  out[4] = o->n_lme;
  out[5] = o->n_p;
  return 0;
}

int orc_compute(void* h, int num_nodes, const int* node_types, const int* num_neigh, const int* neigh_indices,
                const int* neigh_types, long num_edges, const double* xyz, const double* r) {
  try {
    static_cast<Oracle*>(h)->compute(num_nodes, node_types, num_neigh, neigh_indices, neigh_types, num_edges,
                                     xyz, r);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// Layer 0 over num_nodes nodes, layer 1, readouts and ZBL over the first num_local_nodes
// (the pair style's no-MPI-message-passing mode, pair_symmetrix_mace.cpp:672-698).
int orc_compute_halo(void* h, int num_local_nodes, int num_nodes, const int* node_types, const int* num_neigh,
                     const int* neigh_indices, const int* neigh_types, long num_edges, const double* xyz,
                     const double* r) {
  try {
    if (num_local_nodes < 0) throw std::invalid_argument("negative num_local_nodes");
    static_cast<Oracle*>(h)->compute(num_nodes, node_types, num_neigh, neigh_indices, neigh_types, num_edges,
                                     xyz, r, num_local_nodes);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

long orc_get(void* h, const char* name, double* out, long cap) {
  auto* v = static_cast<Oracle*>(h)->buffer(name);
  if (!v) return -1;
  const long n = static_cast<long>(v->size());
  if (out) std::memcpy(out, v->data(), sizeof(double) * (n < cap ? n : cap));
  return n;
}

// ----- model-free primitives (restated), checked against the reference's KATs -----

double orc_zbl_envelope(double r, double r_max, int p) { return Zbl::envelope(r, r_max, p, nullptr); }

double orc_zbl_compute(double a_exp, double a_prefactor, const double* c4, const double* radii, int n_radii,
                       int p, int Zu, int Zv, double r, double* grad) {
  Zbl z;
  z.a_exp = a_exp;
  z.a_pref = a_prefactor;
  z.c.assign(c4, c4 + 4);
  z.radii.assign(radii, radii + n_radii);
  z.p = p;
  double g = 0;
  const double v = z.energy(Zu, Zv, r, &g);
  if (grad) *grad = g;
  return v;
}

int orc_spline_eval(double h, const double* values, const double* derivs, int n, const double* r, int nr,
                    double* f, double* d) {
  try {
    Spline1 s;
    s.build(h, vecd(values, values + n), vecd(derivs, derivs + n));
    for (int i = 0; i < nr; ++i) s.eval(r[i], f[i], d[i]);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

double orc_poly_eval(int num_vars, const double* coeffs, int n_mono, const int* mono_flat, const int* mono_len,
                     const double* x, double* grad) {
  Poly P;
  int off = 0;
  for (int i = 0; i < n_mono; ++i) {
    P.mono.emplace_back(mono_flat + off, mono_flat + off + mono_len[i]);
    off += mono_len[i];
  }
  return poly_eval(P, coeffs, x, grad, num_vars);
}

double orc_mlp_eval(int n_in, int n_hidden, const double* w1, const double* w2, double scale, const double* x,
                    double* grad) {
  double out = 0;
  for (int k = 0; k < n_in; ++k) grad[k] = 0;
  for (int u = 0; u < n_hidden; ++u) {
    double s = 0;
    for (int k = 0; k < n_in; ++k) s += w1[u * n_in + k] * x[k];
    const double sg = 1.0 / (1.0 + std::exp(-s));
    out += w2[u] * scale * s * sg;
    const double d = w2[u] * (scale * sg + scale * s * sg * (1 - sg));
    for (int k = 0; k < n_in; ++k) grad[k] += d * w1[u * n_in + k];
  }
  return out;
}

void orc_sph_harm(const double* xyz, double* Y, double* G) { sph_harm(xyz, Y, G); }

}  // extern "C"
