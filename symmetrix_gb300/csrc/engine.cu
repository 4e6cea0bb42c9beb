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

#include "engine.hpp"

namespace smx {
thread_local std::string g_last_error;
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
}  // namespace smx

using smx::fail;

namespace {

bool is_finite_d(double v) { return std::isfinite(v); }

}  // namespace

extern "C" {

const char* smx_last_error(void) { return smx::g_last_error.c_str(); }

int smx_save_model_cache(const char* model_path, const char* cache_path) {
  if (!model_path || !cache_path) return fail(SMX_ERR_INVALID, "NULL path");
  try {
    smx::HostModel hm;
    smx::PackedModel pm;
    smx::load_model(model_path, hm, pm);
    smx::save_model_cache(cache_path, hm, pm);
  } catch (const std::exception& e) {
    return fail(SMX_ERR_MODEL, e.what());
  }
  return SMX_OK;
}

smx_engine* smx_create(const char* model_path, int precision, int device) {
  if (!model_path) {
    fail(SMX_ERR_INVALID, "model_path is NULL");
    return nullptr;
  }
  if (precision != SMX_PRECISION_FP32 && precision != SMX_PRECISION_BF16) {
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
    check(cudaHostAlloc(reinterpret_cast<void**>(&eng->status_host), sizeof(unsigned), cudaHostAllocMapped),
          "cudaHostAlloc");
    *eng->status_host = 0;
    check(cudaHostGetDevicePointer(reinterpret_cast<void**>(&eng->status_dev), eng->status_host, 0),
          "cudaHostGetDevicePointer");
    check(cudaHostAlloc(reinterpret_cast<void**>(&eng->check_host), sizeof(unsigned), cudaHostAllocMapped),
          "cudaHostAlloc");
    *eng->check_host = 0;
    check(cudaHostGetDevicePointer(reinterpret_cast<void**>(&eng->check_dev), eng->check_host, 0),
          "cudaHostGetDevicePointer");
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
  for (auto& e : eng->ev)
    if (e) cudaEventDestroy(e);
  if (eng->status_host) cudaFreeHost(eng->status_host);
  if (eng->check_host) cudaFreeHost(eng->check_host);
  delete eng;
}

int smx_num_elements(const smx_engine* eng) { return eng ? eng->hm.S : -1; }
int smx_num_channels(const smx_engine* eng) { return eng ? eng->hm.C : -1; }
double smx_r_cut(const smx_engine* eng) { return eng ? eng->hm.r_cut : -1.0; }
int smx_l_max(const smx_engine* eng) { return eng ? eng->hm.l_max : -1; }
int smx_L_max(const smx_engine* eng) { return eng ? eng->hm.L_max : -1; }
int smx_num_LM(const smx_engine* eng) { return eng ? eng->hm.nLM : -1; }
int smx_has_zbl(const smx_engine* eng) { return eng ? (eng->hm.has_zbl ? 1 : 0) : -1; }
int smx_atomic_numbers(const smx_engine* eng, int* out, int cap) {
  if (!eng) return -1;
  for (int q = 0; out && q < eng->hm.S && q < cap; ++q) out[q] = eng->hm.Z[q];
  return eng->hm.S;
}

void* smx_engine_stream(smx_engine* eng) { return eng ? static_cast<void*>(eng->stream) : nullptr; }

int smx_set_option(smx_engine* eng, const char* key, long value) {
  if (!eng || !key) return fail(SMX_ERR_INVALID, "NULL argument");
  if (std::strcmp(key, "keep_stages") == 0) {
    eng->keep_stages = value != 0;
    return SMX_OK;
  }
  if (std::strcmp(key, "profile") == 0) {
    eng->profile = value != 0;
    return SMX_OK;
  }
  if (std::strcmp(key, "autotune") == 0) {  // (re)tune the GEMM and atom schedules on the next evaluation
    eng->autotune = value != 0;
    for (bool& t : eng->tc_tuned) t = false;
    eng->sched_tuned = false;
    if (!eng->autotune && eng->sched_force < 0) eng->sched_set(0);
    return SMX_OK;
  }
  if (std::strcmp(key, "cg_padded") == 0) {  // 1 (default): padded CG tables; 0: compressed rows
    eng->use_cg_padded(value != 0);
    return SMX_OK;
  }
  if (std::strcmp(key, "species_order") == 0) {  // -1 by table size, 0 input order, 1 species-sorted
    if (value < -1 || value > 1) return fail(SMX_ERR_INVALID, "species_order must be -1, 0 or 1");
    eng->species_order = static_cast<int>(value);
    return SMX_OK;
  }
  if (std::strcmp(key, "persistent") == 0) {  // atom schedule: -1 tuned, 0 one block per atom, 1 persistent
    if (value < -1 || value > 1) return fail(SMX_ERR_INVALID, "persistent must be -1, 0 or 1");
    eng->sched_force = static_cast<int>(value);
    eng->sched_tuned = false;
    eng->sched_set(value == 1 ? 1 : 0);
    return SMX_OK;
  }
  if (std::strcmp(key, "pdl") == 0) {  // programmatic dependent launch of the chained kernels, process-wide
    if (value < 0 || value > 1) return fail(SMX_ERR_INVALID, "pdl must be 0 or 1");
    smx::pdl_enabled() = value != 0;
    return SMX_OK;
  }
  if (std::strcmp(key, "test_gemm_timeout") == 0) {  // test of the error path (see engine.hpp)
    if (value < 0 || value > 16) return fail(SMX_ERR_INVALID, "test_gemm_timeout must be in [0, 16]");
    if (eng->precision != SMX_PRECISION_BF16) return fail(SMX_ERR_INVALID, "test_gemm_timeout applies to the bf16 form");
    eng->test_gemm_timeout = static_cast<int>(value);
    return SMX_OK;
  }
  if (std::strcmp(key, "tc_terms") == 0) {  // precision form: bf16 split terms of the GEMMs
    if (value < 1 || value > 3) return fail(SMX_ERR_INVALID, "tc_terms must be 1, 2 or 3");
    if (eng->precision != SMX_PRECISION_BF16) return fail(SMX_ERR_INVALID, "tc_terms applies to the bf16 form");
    try {
      cudaSetDevice(eng->device);
      cudaStreamSynchronize(eng->stream);
      eng->tc_terms = static_cast<int>(value);
      eng->dm.tc_terms = eng->tc_terms;
      eng->setup_tc_weights();
      eng->free_workspace();  // operand buffers are sized by the term count
    } catch (const std::exception& e) {
      return fail(SMX_ERR_CUDA, e.what());
    }
    return SMX_OK;
  }
  return fail(SMX_ERR_INVALID, std::string("unknown option '") + key + "'");
}

long smx_get_option(const smx_engine* eng, const char* key) {
  if (!eng || !key) return -1;
  const std::string k(key);
  if (k == "keep_stages") return eng->keep_stages;
  if (k == "profile") return eng->profile;
  if (k == "precision") return eng->precision;
  if (k == "tc_terms") return eng->tc_terms;
  if (k == "pdl") return smx::pdl_enabled() ? 1 : 0;
  if (k == "autotune") return eng->autotune;
  if (k == "persistent") return eng->sched_mask();  // bit k: per-atom kernel k runs persistent
  if (k == "species_order") return eng->order_species() ? 1 : 0;  // in effect
  if (k == "poly_canon") return eng->dm.poly_canon;  // 1: generated polynomial kernels
  if (k == "cg_padded") return eng->dm.cg_rev_pad != nullptr || eng->dm.cg_fwd_pad != nullptr;
  if (k == "l2_split") return eng->dm.l2_split;       // channel slices of the L_max = 2 layer-1 kernels
  static const char* groups[4] = {"H1", "A1", "Phi1_adj", "M0_adj"};
  for (int q = 0; q < 4; ++q) {
    if (k == std::string("tc_nt_") + groups[q])
      return eng->tc_cfg[q].NT > 0 ? eng->tc_cfg[q].NT : (eng->tc_cfg[q].NT < 0 ? 0 : eng->dm.C);
    if (k == std::string("tc_stages_") + groups[q]) return eng->tc_cfg[q].stages;
    if (k == std::string("tc_tuned_ns_") + groups[q]) return static_cast<long>(eng->tc_tuned_us[q] * 1000.0f);
  }
  return -1;
}

namespace {

// Copy the host edge list of a call into the engine's workspace (reserved for it) and
// check it on the device; SMX_OK, or the failure recorded by fail().
int upload_edges(smx_engine* eng, int num_nodes, const int* node_types, const int* num_neigh,
                 const int* neigh_indices, const int* neigh_types, long num_edges, const double* xyz,
                 const double* r) {
  if (num_nodes < 0 || num_edges < 0) return fail(SMX_ERR_INVALID, "negative size");
  if (num_nodes > 0 && (!node_types || !num_neigh)) return fail(SMX_ERR_INVALID, "NULL node array");
  if (num_edges > 0 && (!neigh_indices || !neigh_types || !xyz || !r)) return fail(SMX_ERR_INVALID, "NULL edge array");
  const int S = eng->hm.S;
  const double rc = eng->hm.r_cut;
  // The inputs are checked on the device after the copies (the reference trusts its
  // caller here); nothing is evaluated until the check has passed.
  eng->reserve(num_nodes, num_edges);
  cudaStream_t s = eng->stream;
  if (num_nodes > 0) {
    check(cudaMemcpyAsync(eng->ntype, node_types, sizeof(int) * num_nodes, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemcpyAsync(eng->nneigh, num_neigh, sizeof(int) * num_nodes, cudaMemcpyHostToDevice, s), "H2D");
  }
  if (num_edges > 0) {
    check(cudaMemcpyAsync(eng->nidx, neigh_indices, sizeof(int) * num_edges, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemcpyAsync(eng->ntype_e, neigh_types, sizeof(int) * num_edges, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemcpyAsync(eng->xyz, xyz, sizeof(double) * 3 * num_edges, cudaMemcpyHostToDevice, s), "H2D");
    check(cudaMemcpyAsync(eng->r, r, sizeof(double) * num_edges, cudaMemcpyHostToDevice, s), "H2D");
  }
  if (num_nodes > 0)
    smx::launch_scan_first(eng->nneigh, num_nodes, eng->first, s);
  else
    check(cudaMemsetAsync(eng->first, 0, sizeof(int), s), "cudaMemsetAsync");
  *reinterpret_cast<volatile unsigned*>(eng->check_host) = 0;
  smx::launch_validate_inputs(num_nodes, num_edges, S, rc, eng->ntype, eng->nneigh, eng->first, eng->nidx,
                              eng->ntype_e, eng->xyz, eng->r, eng->check_dev, s);
  check(cudaStreamSynchronize(s), "input check");
  const unsigned bad = *reinterpret_cast<volatile unsigned*>(eng->check_host);
  if (bad & smx::kBadNodeType) return fail(SMX_ERR_INVALID, "node_types out of range");
  if (bad & smx::kBadNumNeigh) return fail(SMX_ERR_INVALID, "negative num_neigh");
  if (bad & smx::kBadEdgeCount) return fail(SMX_ERR_INVALID, "sum(num_neigh) != num_edges");
  if (bad & smx::kBadNeighIndex) return fail(SMX_ERR_INVALID, "neigh_indices out of range (must be < num_nodes)");
  if (bad & smx::kBadNeighType) return fail(SMX_ERR_INVALID, "neigh_types out of range");
  if (bad & smx::kBadEdge) return fail(SMX_ERR_INVALID, "edge length outside (0, r_cut) or non-finite edge vector");
  return SMX_OK;
}

}  // namespace

int smx_compute_node_energies_forces(smx_engine* eng, int num_nodes, const int* node_types, const int* num_neigh,
                                     const int* neigh_indices, const int* neigh_types, long num_edges,
                                     const double* xyz, const double* r, double* node_energies,
                                     double* node_forces) {
  if (!eng) return fail(SMX_ERR_INVALID, "engine is NULL");
  if (num_nodes > 0 && !node_energies) return fail(SMX_ERR_INVALID, "NULL node array");
  if (num_edges > 0 && !node_forces) return fail(SMX_ERR_INVALID, "NULL edge array");
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    const int code = upload_edges(eng, num_nodes, node_types, num_neigh, neigh_indices, neigh_types, num_edges, xyz, r);
    if (code != SMX_OK) return code;
    cudaStream_t s = eng->stream;
    eng->lastE = num_edges;
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
  if (eng->take_status() != SMX_OK) return fail(SMX_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
  return SMX_OK;
}

int smx_compute_halo(smx_engine* eng, int num_local_nodes, int num_nodes, const int* node_types,
                     const int* num_neigh, const int* neigh_indices, const int* neigh_types, long num_edges,
                     const double* xyz, const double* r, double* node_energies, double* node_forces) {
  if (!eng) return fail(SMX_ERR_INVALID, "engine is NULL");
  if (num_local_nodes < 0 || num_local_nodes > num_nodes)
    return fail(SMX_ERR_INVALID, "need 0 <= num_local_nodes <= num_nodes");
  if (num_local_nodes > 0 && !node_energies) return fail(SMX_ERR_INVALID, "NULL node array");
  if (num_edges > 0 && !node_forces) return fail(SMX_ERR_INVALID, "NULL edge array");
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    const int code = upload_edges(eng, num_nodes, node_types, num_neigh, neigh_indices, neigh_types, num_edges, xyz, r);
    if (code != SMX_OK) return code;
    if (num_local_nodes == 0) {  // no layer-1 node: no energy, and no force reaches any edge
      if (num_edges > 0) std::memset(node_forces, 0, sizeof(double) * 3 * num_edges);
      return SMX_OK;
    }
    cudaStream_t s = eng->stream;
    eng->lastE = num_edges;
    smx::EdgeIn in{eng->first, eng->ntype, eng->nidx, eng->ntype_e, eng->xyz, eng->r, num_nodes};
    eng->run(in, eng->energies, eng->forces, s, num_local_nodes);
    check(cudaMemcpyAsync(node_energies, eng->energies, sizeof(double) * num_local_nodes, cudaMemcpyDeviceToHost, s),
          "D2H");
    if (num_edges > 0)
      check(cudaMemcpyAsync(node_forces, eng->forces, sizeof(double) * 3 * num_edges, cudaMemcpyDeviceToHost, s), "D2H");
    check(cudaStreamSynchronize(s), "evaluation");
  } catch (const std::exception& e) {
    return fail(SMX_ERR_CUDA, e.what());
  }
  if (eng->take_status() != SMX_OK) return fail(SMX_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
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
    eng->lastE = 0;  // the edge arrays are the caller's: no node_forces stage read
    smx::EdgeIn in{eng->first, node_types, neigh_indices, neigh_types, xyz, r, num_nodes};
    eng->run(in, node_energies, node_forces, s);
  } catch (const std::exception& e) {
    return fail(SMX_ERR_CUDA, e.what());
  }
  return SMX_OK;
}

int smx_sync(smx_engine* eng, void* stream) {
  if (!eng) return fail(SMX_ERR_INVALID, "engine is NULL");
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    check(cudaStreamSynchronize(stream ? static_cast<cudaStream_t>(stream) : eng->stream), "cudaStreamSynchronize");
  } catch (const std::exception& e) {
    return fail(SMX_ERR_CUDA, e.what());
  }
  if (eng->take_status() != SMX_OK) return fail(SMX_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
  return SMX_OK;
}

int smx_stage_times(smx_engine* eng, double* out_ms, int cap) {
  if (!eng) return fail(SMX_ERR_INVALID, "engine is NULL");
  if (!eng->profile || !eng->ev[0]) return 0;
  try {
    check(cudaEventSynchronize(eng->ev[smx_engine::kStages]), "cudaEventSynchronize");
    for (int q = 0; q < smx_engine::kStages && q < cap; ++q) {
      float ms = 0.0f;
      check(cudaEventElapsedTime(&ms, eng->ev[q], eng->ev[q + 1]), "cudaEventElapsedTime");
      out_ms[q] = ms;
    }
  } catch (const std::exception& e) {
    return -fail(SMX_ERR_CUDA, e.what());
  }
  return smx_engine::kStages;
}

long smx_get_stage(smx_engine* eng, const char* name, double* out, long cap) {
  if (!eng || !name) {
    fail(SMX_ERR_INVALID, "NULL argument");
    return -1;
  }
  // layer-0 stages hold a row block per node, layer-1 stages per layer-1 node
  const long N = eng->lastN, N1 = eng->lastN1, C = eng->dm.C;
  const float* src = nullptr;
  bool kept = true;
  long n = 0;
  const std::string s(name);
  if (s == "node_energies" || s == "node_forces") {  // float64 outputs of the last host call or stage call
    if (!eng->evaluated) {
      fail(SMX_ERR_INVALID, "no evaluation has run since the engine's buffers were (re)allocated");
      return -2;
    }
    const double* d = s == "node_energies" ? eng->energies : eng->forces;
    n = s == "node_energies" ? N1 : 3 * eng->lastE;
    if (out && cap > 0 && n > 0) {
      try {
        check(cudaSetDevice(eng->device), "cudaSetDevice");
        check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        check(cudaMemcpy(out, d, sizeof(double) * std::min(n, cap), cudaMemcpyDeviceToHost), "D2H");
      } catch (const std::exception& e) {
        fail(SMX_ERR_CUDA, e.what());
        return -3;
      }
    }
    return n;
  }
  if (s == "A0") { src = eng->A0; n = N * 16 * C; }
  else if (s == "M0") { src = eng->M0; n = N * eng->dm.nLM * C; kept = eng->M0_kept; }
  else if (s == "H1") { src = eng->H1; n = N * eng->dm.nLM * C; }
  else if (s == "Phi1") { src = eng->Phi1; n = N1 * eng->dm.n_lme * C; kept = eng->Phi1_kept; }
  else if (s == "A1") { src = eng->A1; n = N1 * 16 * C; }
  else if (s == "M1") { src = eng->M1; n = N1 * C; }
  else if (s == "H2") { src = eng->H2; n = N1 * C; }
  else if (s == "A0_adj") { src = eng->A0_adj; n = N * 16 * C; }
  else if (s == "M0_adj") { src = eng->M0_adj; n = N * eng->dm.nLM * C; }
  else if (s == "H1_adj") { src = eng->H1_adj; n = N * eng->dm.nLM * C; }
  else if (s == "Phi1_adj") { src = eng->Phi1_adj; n = N1 * eng->dm.n_lme * C; }
  else if (s == "A1_adj") { src = eng->A1_adj; n = N1 * 16 * C; kept = eng->A1adj_kept; }
  else if (s == "M1_adj") { src = eng->M1_adj; n = N1 * C; }
  else if (s == "H2_adj") { src = eng->H2_adj; n = N1 * C; }
  else {
    fail(SMX_ERR_INVALID, std::string("unknown stage '") + name + "'");
    return -1;
  }
  if (!eng->evaluated) {
    fail(SMX_ERR_INVALID, "no evaluation has run since the engine's buffers were (re)allocated");
    return -2;
  }
  if (n == 0) return 0;
  if (!src || !kept) {
    fail(SMX_ERR_INVALID, "stage " + s + " was not written by the last evaluation (set keep_stages)");
    return -2;
  }
  if (out && cap > 0) {
    std::vector<float> tmp(static_cast<size_t>(n));
    try {
      check(cudaSetDevice(eng->device), "cudaSetDevice");
      check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");  // the last call may have run on a caller's stream
      check(cudaMemcpy(tmp.data(), src, sizeof(float) * n, cudaMemcpyDeviceToHost), "D2H");
    } catch (const std::exception& e) {
      fail(SMX_ERR_CUDA, e.what());
      return -3;
    }
    for (long q = 0; q < n && q < cap; ++q) out[q] = tmp[q];
  }
  return n;
}

// Float32 stage buffers are written from float64 values (rounded); node_forces (float64,
// the per-edge forces of the last call's edges) is copied as is.
long smx_set_stage(smx_engine* eng, const char* name, const double* values, long n) {
  if (!eng || !name || (n > 0 && !values)) return -fail(SMX_ERR_INVALID, "NULL argument");
  if (!eng->evaluated) return -fail(SMX_ERR_INVALID, "no evaluation has set up the engine's buffers yet");
  const long N = eng->lastN, N1 = eng->lastN1, C = eng->dm.C;
  const std::string s(name);
  float* dst = nullptr;
  long want = 0;
  if (s == "M0") { dst = eng->M0; want = N * eng->dm.nLM * C; eng->M0_kept = true; }
  else if (s == "H1") { dst = eng->H1; want = N * eng->dm.nLM * C; }
  else if (s == "Phi1") { dst = eng->Phi1; want = N1 * eng->dm.n_lme * C; eng->Phi1_kept = true; }
  else if (s == "A1") { dst = eng->A1; want = N1 * 16 * C; }
  else if (s == "M0_adj") { dst = eng->M0_adj; want = N * eng->dm.nLM * C; }
  else if (s == "H1_adj") { dst = eng->H1_adj; want = N * eng->dm.nLM * C; }
  else if (s == "Phi1_adj") { dst = eng->Phi1_adj; want = N1 * eng->dm.n_lme * C; }
  else if (s == "A1_adj") { dst = eng->A1_adj; want = N1 * 16 * C; eng->A1adj_kept = true; }
  else if (s != "node_forces") return -fail(SMX_ERR_INVALID, std::string("stage '") + name + "' cannot be written");
  if (s == "node_forces") want = 3 * eng->lastE;
  if (n != want)
    return -fail(SMX_ERR_INVALID, "stage " + s + " holds " + std::to_string(want) + " values, got " + std::to_string(n));
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    if (n == 0) return 0;
    if (s == "node_forces") {
      check(cudaMemcpy(eng->forces, values, sizeof(double) * n, cudaMemcpyHostToDevice), "H2D");
    } else {
      std::vector<float> tmp(values, values + n);
      check(cudaMemcpy(dst, tmp.data(), sizeof(float) * n, cudaMemcpyHostToDevice), "H2D");
    }
  } catch (const std::exception& e) {
    return -fail(SMX_ERR_CUDA, e.what());
  }
  return n;
}

int smx_run_stage(smx_engine* eng, const char* stage, int num_nodes, const int* node_types, const int* num_neigh,
                  const int* neigh_indices, const int* neigh_types, long num_edges, const double* xyz,
                  const double* r, int flags) {
  if (!eng || !stage) return fail(SMX_ERR_INVALID, "NULL argument");
  const std::string st(stage);
  const bool edge_stage = st == "compute_Phi1" || st == "reverse_Phi1";
  const bool node_stage = st == "compute_H1" || st == "reverse_H1" || st == "compute_A1" || st == "reverse_A1";
  if (!edge_stage && !node_stage) return fail(SMX_ERR_INVALID, "unknown stage '" + st + "'");
  try {
    check(cudaSetDevice(eng->device), "cudaSetDevice");
    cudaStream_t s = eng->stream;
    if (node_stage) {
      if (!eng->evaluated) return fail(SMX_ERR_INVALID, "no evaluation has set up the engine's buffers yet");
      const bool layer1 = st == "compute_A1" || st == "reverse_A1";
      if (num_nodes != (layer1 ? eng->lastN1 : eng->lastN))
        return fail(SMX_ERR_INVALID, "num_nodes differs from the evaluation that set up the engine's buffers");
      if (st == "reverse_A1" && !eng->A1adj_kept)
        return fail(SMX_ERR_INVALID, "A1_adj was not written by the last evaluation (set it or keep_stages)");
      if (st == "compute_H1" && !eng->M0_kept)
        return fail(SMX_ERR_INVALID, "M0 was not written by the last evaluation (set it or keep_stages)");
      if (st == "compute_A1" && !eng->Phi1_kept)
        return fail(SMX_ERR_INVALID, "Phi1 was not written by the last evaluation (set it or keep_stages)");
      eng->run_node_stage(st, s);
    } else {
      const int code = upload_edges(eng, num_nodes, node_types, num_neigh, neigh_indices, neigh_types, num_edges, xyz, r);
      if (code != SMX_OK) return code;
      // (the upload may have regrown the workspace, which drops its contents)
      if (!eng->evaluated || num_nodes != eng->lastN) {  // buffers for a new node count: nothing to read yet
        const long C = eng->dm.C;
        check(cudaMemsetAsync(eng->H1, 0, sizeof(float) * num_nodes * eng->dm.nLM * C, s), "cudaMemsetAsync");
        check(cudaMemsetAsync(eng->H1_adj, 0, sizeof(float) * num_nodes * eng->dm.nLM * C, s), "cudaMemsetAsync");
        check(cudaMemsetAsync(eng->Phi1_adj, 0, sizeof(float) * num_nodes * eng->dm.n_lme * C, s), "cudaMemsetAsync");
        eng->lastN = eng->lastN1 = num_nodes;
        eng->evaluated = true;
        eng->M0_kept = eng->Phi1_kept = eng->A1adj_kept = false;
      }
      if (num_edges != eng->lastE) check(cudaMemsetAsync(eng->forces, 0, sizeof(double) * 3 * num_edges, s), "memset");
      eng->lastE = num_edges;
      smx::EdgeIn in{eng->first, eng->ntype, eng->nidx, eng->ntype_e, eng->xyz, eng->r, num_nodes};
      eng->run_edge_stage(st == "reverse_Phi1", in, num_edges, (flags & SMX_STAGE_ZERO_DXYZ) != 0,
                          (flags & SMX_STAGE_ZERO_H1_ADJ) != 0, s);
    }
    check(cudaGetLastError(), "kernel launch");
    check(cudaStreamSynchronize(s), "stage");
  } catch (const std::exception& e) {
    return fail(SMX_ERR_CUDA, e.what());
  }
  if (eng->take_status() != SMX_OK) return fail(SMX_ERR_TIMEOUT, "a device-side wait timed out; results are invalid");
  return SMX_OK;
}

}  // extern "C"
