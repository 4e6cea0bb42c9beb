// C ABI over the reference's own CPU evaluator (libsymmetrix/source/mace.cpp and its
// primitives), compiled unchanged from the reference tree against the stand-in
// headers in oracle/shim.  Test infrastructure only: it pins the oracle's
// restatement (oracle/mace_oracle.cpp) and generates the golden fixtures under
// tests/golden.  The function names and arguments match the oracle's C ABI with
// the prefix ref_ instead of orc_, so tests can drive either one.
#include <algorithm>
#include <cstring>
#include <exception>
#include <span>
#include <string>
#include <vector>

#include "cubic_spline.hpp"
#include "mace.hpp"
#include "multilayer_perceptron.hpp"
#include "multivariate_polynomial.hpp"
#include "zbl.hpp"

namespace {
thread_local std::string g_err;

std::vector<double>* buffer(MACE* m, const std::string& name) {
  if (name == "node_energies") return &m->node_energies;
  if (name == "node_forces") return &m->node_forces;
  if (name == "Y") return &m->Y;
  if (name == "Y_grad") return &m->Y_grad;
  if (name == "R0") return &m->R0;
  if (name == "R0_deriv") return &m->R0_deriv;
  if (name == "R1") return &m->R1;
  if (name == "R1_deriv") return &m->R1_deriv;
  if (name == "A0") return &m->A0;
  if (name == "A0_adj") return &m->A0_adj;
  if (name == "M0") return &m->M0;
  if (name == "M0_adj") return &m->M0_adj;
  if (name == "H1") return &m->H1;
  if (name == "H1_adj") return &m->H1_adj;
  if (name == "Phi1r") return &m->Phi1r;
  if (name == "Phi1") return &m->Phi1;
  if (name == "Phi1_adj") return &m->dPhi1;
  if (name == "A1") return &m->A1;
  if (name == "A1_adj") return &m->A1_adj;
  if (name == "M1") return &m->M1;
  if (name == "M1_adj") return &m->M1_adj;
  if (name == "H2") return &m->H2;
  if (name == "H2_adj") return &m->H2_adj;
  return nullptr;
}
}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

void* ref_load(const char* path) {
  try {
    return new MACE(std::string(path));
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

void ref_free(void* h) { delete static_cast<MACE*>(h); }

int ref_info(void* h, int* out) {
  auto* m = static_cast<MACE*>(h);
  out[0] = m->num_elements;
  out[1] = m->num_channels;
  out[2] = m->l_max;
  out[3] = m->L_max;
  out[4] = m->num_lme;
  out[5] = m->num_lelm1lm2;
  return 0;
}

int ref_compute(void* h, int num_nodes, const int* node_types, const int* num_neigh,
                const int* neigh_indices, const int* neigh_types, long num_edges, const double* xyz,
                const double* r) {
  try {
    auto* m = static_cast<MACE*>(h);
    m->compute_node_energies_forces(
        num_nodes, std::span<const int>(node_types, num_nodes), std::span<const int>(num_neigh, num_nodes),
        std::span<const int>(neigh_indices, num_edges), std::span<const int>(neigh_types, num_edges),
        std::span<const double>(xyz, 3 * num_edges), std::span<const double>(r, num_edges));
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// The reference's stages in the order and with the node counts of the pair style's
// no-MPI-message-passing mode (pair_symmetrix/pair_symmetrix_mace.cpp:657-698): layer 0
// over num_nodes nodes, layer 1, readouts and ZBL over the first num_local_nodes.
int ref_compute_halo(void* h, int num_local_nodes, int num_nodes, const int* node_types, const int* num_neigh,
                     const int* neigh_indices, const int* neigh_types, long num_edges, const double* xyz,
                     const double* r) {
  try {
    auto* m = static_cast<MACE*>(h);
    const int nl = num_local_nodes, na = num_nodes;
    const std::span<const int> nt(node_types, na), nn(num_neigh, na), ni(neigh_indices, num_edges),
        te(neigh_types, num_edges);
    const std::span<const double> x(xyz, 3 * num_edges), rr(r, num_edges);
    m->node_energies.assign(nl, 0.0);
    m->node_forces.assign(3 * num_edges, 0.0);
    if (m->has_zbl)
      m->zbl.compute_ZBL(nl, nt, nn, te, m->atomic_numbers, rr, x, m->node_energies, m->node_forces);
    m->compute_Y(x);
    m->compute_R0(na, nt, nn, te, rr);
    m->compute_A0(na, nt, nn, te);
    m->compute_A0_scaled(na, nt, nn, te, rr);
    m->compute_M0(na, nt);
    m->compute_H1(na);
    m->compute_R1(nl, nt, nn, te, rr);
    m->compute_Phi1(nl, nn, ni);
    m->compute_A1(nl);
    m->compute_A1_scaled(nl, nt, nn, te, rr);
    m->compute_M1(nl, nt);
    m->compute_H2(nl, nt);
    m->compute_readouts(nl, nt);
    m->reverse_H2(nl, nt, false);
    m->reverse_M1(nl, nt);
    m->reverse_A1_scaled(nl, nt, nn, te, x, rr, false);
    m->reverse_A1(nl);
    m->reverse_Phi1(nl, nn, ni, x, rr, false, false);
    m->reverse_H1(na);
    m->reverse_M0(na, nt);
    m->reverse_A0_scaled(na, nt, nn, te, x, rr);
    m->reverse_A0(na, nt, nn, te, x, rr);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// The reference's stages in the order of the pair style's MPI-message-passing mode on one
// rank (pair_symmetrix/pair_symmetrix_mace.cpp:438-497): num_nodes local nodes whose edges
// index atoms (neigh_atoms < num_atoms, local atoms first); H1 rows of the ghost atoms are
// filled from their owners (owner[a], the single-rank forward communication, :462-470) and
// the ghosts' H1_adj rows are added to their owners' (the reverse communication, :487-489).
int ref_compute_message_passing(void* h, int num_nodes, int num_atoms, const int* node_types, const int* num_neigh,
                                const int* neigh_atoms, const int* neigh_types, long num_edges, const double* xyz,
                                const double* r, const int* owner) {
  try {
    auto* m = static_cast<MACE*>(h);
    const int n = num_nodes;
    const std::span<const int> nt(node_types, n), nn(num_neigh, n), nj(neigh_atoms, num_edges),
        te(neigh_types, num_edges);
    const std::span<const double> x(xyz, 3 * num_edges), rr(r, num_edges);
    const long row = static_cast<long>(m->num_LM) * m->num_channels;
    m->node_energies.assign(n, 0.0);
    m->node_forces.assign(3 * num_edges, 0.0);
    if (m->has_zbl)
      m->zbl.compute_ZBL(n, nt, nn, te, m->atomic_numbers, rr, x, m->node_energies, m->node_forces);
    m->compute_Y(x);
    m->compute_R0(n, nt, nn, te, rr);
    m->compute_A0(n, nt, nn, te);
    m->compute_A0_scaled(n, nt, nn, te, rr);
    m->compute_M0(n, nt);
    m->compute_H1(n);
    std::vector<double> H1(static_cast<size_t>(num_atoms) * row, 0.0);
    std::copy(m->H1.begin(), m->H1.begin() + n * row, H1.begin());
    for (int a = n; a < num_atoms; ++a)
      std::copy(H1.begin() + owner[a] * row, H1.begin() + (owner[a] + 1) * row, H1.begin() + a * row);
    m->H1 = H1;
    m->compute_R1(n, nt, nn, te, rr);
    m->compute_Phi1(n, nn, nj);
    m->compute_A1(n);
    m->compute_A1_scaled(n, nt, nn, te, rr);
    m->compute_M1(n, nt);
    m->compute_H2(n, nt);
    m->compute_readouts(n, nt);
    m->reverse_H2(n, nt, false);
    m->reverse_M1(n, nt);
    m->reverse_A1_scaled(n, nt, nn, te, x, rr, false);
    m->reverse_A1(n);
    m->reverse_Phi1(n, nn, nj, x, rr, false, false);
    std::vector<double> H1_adj = m->H1_adj;
    for (int a = n; a < num_atoms; ++a)
      for (long k = 0; k < row; ++k) H1_adj[owner[a] * row + k] += H1_adj[a * row + k];
    m->H1_adj = H1_adj;
    m->reverse_H1(n);
    m->reverse_M0(n, nt);
    m->reverse_A0_scaled(n, nt, nn, te, x, rr);
    m->reverse_A0(n, nt, nn, te, x, rr);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// Copies a stage buffer; returns its length (copies at most cap values).
long ref_get(void* h, const char* name, double* out, long cap) {
  auto* v = buffer(static_cast<MACE*>(h), name);
  if (!v) return -1;
  const long n = static_cast<long>(v->size());
  if (out) std::memcpy(out, v->data(), sizeof(double) * (n < cap ? n : cap));
  return n;
}

// ----- model-free primitives, for the reference's own known-answer tests -----

double ref_zbl_envelope(double r, double r_max, int p) {
  ZBL z(0.3, 0.4543, {0.1818, 0.5099, 0.2802, 0.02817}, {0.2}, 6);
  return z.compute_envelope(r, r_max, p);
}

double ref_zbl_compute(double a_exp, double a_prefactor, const double* c4, const double* radii,
                       int n_radii, int p, int Zu, int Zv, double r, double* grad) {
  ZBL z(a_exp, a_prefactor, std::vector<double>(c4, c4 + 4), std::vector<double>(radii, radii + n_radii), p);
  if (grad) *grad = z.compute_gradient(Zu, Zv, r);
  return z.compute(Zu, Zv, r);
}

int ref_spline_eval(double h, const double* values, const double* derivs, int n, const double* r,
                    int nr, double* f, double* d) {
  try {
    CubicSpline s(h, std::vector<double>(values, values + n), std::vector<double>(derivs, derivs + n));
    for (int i = 0; i < nr; ++i) {
      auto [fv, dv] = s.evaluate_deriv(r[i]);
      f[i] = fv;
      d[i] = dv;
    }
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

double ref_poly_eval(int num_vars, const double* coeffs, int n_mono, const int* mono_flat,
                     const int* mono_len, const double* x, double* grad) {
  std::vector<std::vector<int>> monos;
  int off = 0;
  for (int i = 0; i < n_mono; ++i) {
    monos.emplace_back(mono_flat + off, mono_flat + off + mono_len[i]);
    off += mono_len[i];
  }
  MultivariatePolynomial p(num_vars, std::vector<double>(coeffs, coeffs + n_mono), monos);
  auto [f, g] = p.evaluate_gradient(std::vector<double>(x, x + num_vars));
  for (int i = 0; i < num_vars; ++i) grad[i] = g[i];
  return f;
}

double ref_mlp_eval(int n_in, int n_hidden, const double* w1, const double* w2, double scale,
                    const double* x, double* grad) {
  MultilayerPerceptron m({n_in, n_hidden, 1},
                         {std::vector<double>(w1, w1 + n_in * n_hidden), std::vector<double>(w2, w2 + n_hidden)},
                         scale);
  auto [f, g] = m.evaluate_gradient(std::vector<double>(x, x + n_in));
  for (int i = 0; i < n_in; ++i) grad[i] = g[i];
  return f[0];
}

}  // extern "C"
