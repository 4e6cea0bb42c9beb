// Node-level kernels: channel-mixing GEMMs, the layer-1 node tail (symmetric
// contraction M1, H2, readouts, energy and the adjoint seeds), and small utilities.
//
// Reference stages restated here (libsymmetrix/source/mace.cpp):
//   k_gemm       : compute_H1 / reverse_H1 (:397-451), compute_A1 / reverse_A1 (:607-679)
//   k_node_tail  : compute_M1 (:759-777), compute_H2 (:796-832), compute_readouts (:876-903)
//                  with MultilayerPerceptron::evaluate_gradient (multilayer_perceptron.cpp:76-150),
//                  reverse_H2 (:834-874), reverse_M1 (:779-794)
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>

#include "device.cuh"
#include "kernels.h"
#include "poly_canon.h"

namespace smx {

// ---------------------------------------------------------------------------
// FP32 SIMT GEMM, 64x64 tile, 16-deep k slices, 256 threads with a 4x4 register
// tile each.  blockIdx.z selects the segment.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gemm(GemmBatch gb) {
  pdl_begin();
  const GemmSeg g = gb.s[blockIdx.z];
  const int row0 = blockIdx.x * 64, col0 = blockIdx.y * 64;
  if (row0 >= g.rows || col0 >= g.ncols) return;
  __shared__ __align__(16) float As[16][64 + 4];
  __shared__ __align__(16) float Bs[16][64];
  const int tid = threadIdx.x;
  const int tr = tid >> 4, tc = tid & 15;
  // A loader: row tid/4, k offset (tid%4)*4
  const int a_row = row0 + (tid >> 2);
  const int a_k = (tid & 3) * 4;
  const float* a_ptr = nullptr;
  if (a_row < g.rows) {
    const int node = a_row / g.rpn, sub = a_row - node * g.rpn;
    a_ptr = g.X + node * g.x_ns + g.x_off + static_cast<long>(sub) * g.x_rs;
  }
  // B loader: k row tid/16, cols (tid%16)*4
  const int b_k = tid >> 4;
  const int b_col = col0 + (tid & 15) * 4;
  float acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0f;
  for (int k0 = 0; k0 < g.K; k0 += 16) {
    float4 av = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a_ptr) av = __ldg(reinterpret_cast<const float4*>(a_ptr + k0 + a_k));
    float4 bv = make_float4(0.f, 0.f, 0.f, 0.f);
    if (b_col < g.ncols) bv = __ldg(reinterpret_cast<const float4*>(g.B + static_cast<long>(k0 + b_k) * g.ncols + b_col));
    __syncthreads();
    As[a_k + 0][tid >> 2] = av.x;
    As[a_k + 1][tid >> 2] = av.y;
    As[a_k + 2][tid >> 2] = av.z;
    As[a_k + 3][tid >> 2] = av.w;
    *reinterpret_cast<float4*>(&Bs[b_k][(tid & 15) * 4]) = bv;
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      const float4 a4 = *reinterpret_cast<const float4*>(&As[kk][tr * 4]);
      const float4 b4 = *reinterpret_cast<const float4*>(&Bs[kk][tc * 4]);
      const float ar[4] = {a4.x, a4.y, a4.z, a4.w};
      const float br[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(ar[a], br[b], acc[a][b]);
    }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int r = row0 + tr * 4 + a;
    if (r >= g.rows) continue;
    const int node = r / g.rpn, sub = r - node * g.rpn;
    float* y = g.Y + node * g.y_ns + g.y_off + static_cast<long>(sub) * g.y_rs + col0 + tc * 4;
    if (col0 + tc * 4 < g.ncols) *reinterpret_cast<float4*>(y) = make_float4(acc[a][0], acc[a][1], acc[a][2], acc[a][3]);
  }
}

void launch_gemm(const GemmBatch& b, cudaStream_t s) {
  int maxr = 0, maxc = 0;
  for (int q = 0; q < b.n; ++q) {
    maxr = b.s[q].rows > maxr ? b.s[q].rows : maxr;
    maxc = b.s[q].ncols > maxc ? b.s[q].ncols : maxc;
  }
  if (maxr == 0 || b.n == 0) return;
  dim3 grid(ceil_div(maxr, 64), ceil_div(maxc, 64), b.n);
  launch_pdl(k_gemm, grid, 256, 0, s, b);
}

// ---------------------------------------------------------------------------
// Layer-1 node tail, one block per node, one thread per channel.
//   M1[k] = P1_{ti,k}(A1[i,:,k]) and its gradient,
//   H2 = W_H1[ti]^T H1[i,0,:] + W_M1^T M1,
//   E_i = e0[ti] + w1 . H1[i,0,:] + w2 . s*silu(W1 H2)           (float64 output),
//   dE/dH2 (MLP gradient), H1_adj[i,0,:] = w1 + W_H1[ti] dE/dH2 (other rows 0; fixed point),
//   M1_adj = W_M1 dE/dH2, A1_adj[i,lm,k] = dM1/dA1[lm] * M1_adj[k].
// ---------------------------------------------------------------------------
__device__ __forceinline__ void node_tail_atom(const DevModel& m, const int* __restrict__ ntype, float* __restrict__ A1,
                                               const float* __restrict__ H1, float* __restrict__ M1o,
                                               float* __restrict__ H2o, float* __restrict__ A1_adj,
                                               fix64* __restrict__ H1_adj, float* __restrict__ M1_adj_o,
                                               float* __restrict__ H2_adj_o, const float* __restrict__ zbl_e,
                                               double* __restrict__ energies, int N, int i) {
  extern __shared__ float dyn[];
  const int C = m.C, k = threadIdx.x;
  const int nwarp = C >> 5, lane = k & 31, warp = k >> 5;
  const int ti = ntype[i];
  const int nh = m.n_hidden;
  float* sX = dyn;              // [17][C]
  float* sG = sX + 17 * C;      // [17][C]
  float* sM1 = sG + 17 * C;     // [C]
  float* sH10 = sM1 + C;        // [C]
  float* sH2 = sH10 + C;        // [C]
  float* sdH2 = sH2 + C;        // [C]
  float* sRed = sdH2 + C;       // [33][8]
  float* sS = sRed + 33 * 8;    // [33]
  float f = 0.0f;
  const float* cf = m.coef1 + static_cast<size_t>(ti) * m.T1 * C + k;
  const bool dens = m.dens_spl[1] != nullptr;
  const float S1 = dens ? m.dens_s[1][i] : 1.0f;
  if (dens) {  // density-normalised A1, kept scaled (compute_A1_scaled, mace.cpp:681-705)
#pragma unroll
    for (int q = 0; q < 16; ++q) A1[(static_cast<size_t>(i) * 16 + q) * C + k] /= S1;
  }
  if (m.poly_canon) {  // generated straight-line M1 polynomial and gradient
    float x[16], g[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      x[q] = A1[(static_cast<size_t>(i) * 16 + q) * C + k];
      g[q] = 0.0f;
    }
    f = poly::value_grad_M1(x, cf, C, g);
#pragma unroll
    for (int q = 0; q < 16; ++q) sG[q * C + k] = g[q];
  } else {
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    sX[q * C + k] = A1[(static_cast<size_t>(i) * 16 + q) * C + k];
    sG[q * C + k] = 0.0f;
  }
  sX[16 * C + k] = 1.0f;
  sG[16 * C + k] = 0.0f;
  for (int t = 0; t < m.T1; ++t) {
    const int pk = __ldg(m.mono1 + t);
    const int a = pk & 255, b = (pk >> 8) & 255, c = pk >> 16;
    const float w = __ldg(cf + static_cast<size_t>(t) * C);
    const float xa = sX[a * C + k], xb = sX[b * C + k], xc = sX[c * C + k];
    f = fmaf(w, xa * xb * xc, f);
    sG[a * C + k] += w * xb * xc;
    sG[b * C + k] += w * xa * xc;
    sG[c * C + k] += w * xa * xb;
  }
  }
  sM1[k] = f;
  const float h10 = H1[static_cast<size_t>(i) * m.nLM * C + k];
  sH10[k] = h10;
  __syncthreads();
  // H2 = W_H1[ti]^T H1[i,0,:] + W_M1^T M1: four partial sums, eight rows' loads in flight
  const float* W = m.H2W_H1 + static_cast<size_t>(ti) * C * C + k;
  const float* WM = m.H2W_M1 + k;
  float hp0 = 0.0f, hp1 = 0.0f, hp2 = 0.0f, hp3 = 0.0f;  // C is a multiple of 32
#pragma unroll 4
  for (int r = 0; r < C; r += 4) {
    const size_t o = static_cast<size_t>(r) * C;
    hp0 = fmaf(sM1[r], __ldg(WM + o), fmaf(sH10[r], __ldg(W + o), hp0));
    hp1 = fmaf(sM1[r + 1], __ldg(WM + o + C), fmaf(sH10[r + 1], __ldg(W + o + C), hp1));
    hp2 = fmaf(sM1[r + 2], __ldg(WM + o + 2 * C), fmaf(sH10[r + 2], __ldg(W + o + 2 * C), hp2));
    hp3 = fmaf(sM1[r + 3], __ldg(WM + o + 3 * C), fmaf(sH10[r + 3], __ldg(W + o + 3 * C), hp3));
  }
  const float h2 = (hp0 + hp1) + (hp2 + hp3);
  sH2[k] = h2;
  // hidden pre-activations s_u = W1[u,:] . H2 and the linear readout w1 . H1[i,0,:] (slot nh)
#pragma unroll 4
  for (int u = 0; u <= nh; ++u) {
    float v = (u < nh) ? __ldg(m.ro2_w1 + static_cast<size_t>(u) * C + k) * h2 : __ldg(m.ro1 + k) * h10;
    v = warp_sum(v);
    if (lane == 0) sRed[u * 8 + warp] = v;
  }
  __syncthreads();
  for (int u = k; u <= nh; u += C) {
    float s = 0.0f;
    for (int w = 0; w < nwarp; ++w) s += sRed[u * 8 + w];
    sS[u] = s;
  }
  __syncthreads();
  float dh2 = 0.0f;
  for (int u = 0; u < nh; ++u) {
    const float s = sS[u];
    const float sg = 1.0f / (1.0f + expf(-s));
    const float dact = m.ro2_scale * sg + m.ro2_scale * s * sg * (1.0f - sg);
    dh2 = fmaf(__ldg(m.ro2_w2 + u) * dact, __ldg(m.ro2_w1 + static_cast<size_t>(u) * C + k), dh2);
  }
  sdH2[k] = dh2;
  if (k == 0) {
    double e = static_cast<double>(__ldg(m.e0 + ti)) + static_cast<double>(sS[nh]);
    for (int u = 0; u < nh; ++u) {
      const float s = sS[u];
      const float sg = 1.0f / (1.0f + expf(-s));
      e += static_cast<double>(__ldg(m.ro2_w2 + u) * (m.ro2_scale * s * sg));
    }
    if (zbl_e) e += static_cast<double>(zbl_e[i]);
    energies[i] = e;
  }
  __syncthreads();
  // H1_adj[i,0,:] = w1 + W_H1[ti] dE/dH2 and M1_adj = W_M1 dE/dH2: as above
  const float* WT = m.H2W_H1_T + static_cast<size_t>(ti) * C * C + k;
  const float* WMT = m.H2W_M1_T + k;
  float ha0 = 0.0f, ha1 = 0.0f, ma0 = 0.0f, ma1 = 0.0f;
#pragma unroll 8
  for (int c = 0; c < C; c += 2) {
    const size_t o = static_cast<size_t>(c) * C;
    const float d0 = sdH2[c], d1 = sdH2[c + 1];
    ha0 = fmaf(__ldg(WT + o), d0, ha0);
    ma0 = fmaf(__ldg(WMT + o), d0, ma0);
    ha1 = fmaf(__ldg(WT + o + C), d1, ha1);
    ma1 = fmaf(__ldg(WMT + o + C), d1, ma1);
  }
  const float ha = __ldg(m.ro1 + k) + (ha0 + ha1);
  const float m1a = ma0 + ma1;
  if (dens) {  // reverse_A1_scaled (mace.cpp:707-757): c_i = dA1 . A1 / s_i, dA1 /= s_i
    float dot = 0.0f;
#pragma unroll
    for (int q = 0; q < 16; ++q) dot = fmaf(sG[q * C + k] * m1a, A1[(static_cast<size_t>(i) * 16 + q) * C + k], dot);
    dot = block_sum(dot);
    if (k == 0) m.dens_c[1][i] = dot / S1;
  }
  // A1_adj = dM1/dA1 * M1_adj (/ S1 when density-normalised; no division sequence otherwise)
  auto a1adj = [&](int q) { return dens ? sG[q * C + k] * m1a / S1 : sG[q * C + k] * m1a; };
  if (A1_adj)  // nullptr: only the split rows below are consumed
#pragma unroll
    for (int q = 0; q < 16; ++q) A1_adj[(static_cast<size_t>(i) * 16 + q) * C + k] = a1adj(q);
  if (m.op_a1adj) {  // BF16 form: the Phi1_adj GEMM's split operand, rows (node, m) per l
    const int T = m.tc_terms;
    const size_t pitch = static_cast<size_t>(split_xterms(T)) * C;
    for (int l = 0; l < 4; ++l) {
      if (m.num_e[l] == 0) continue;
      __nv_bfloat16* row = m.op_a1adj + pitch * (static_cast<size_t>(N) * l * l + static_cast<size_t>(i) * (2 * l + 1));
      for (int mm = 0; mm < 2 * l + 1; ++mm, row += pitch) write_split(row, C, T, k, a1adj(l * l + mm));
    }
  }
  // H1_adj in fixed point: the layer-1 adjoint adds its edge terms to these rows
  H1_adj[static_cast<size_t>(i) * m.nLM * C + k] = to_fixed(ha);
  for (int LM = 1; LM < m.nLM; ++LM) H1_adj[(static_cast<size_t>(i) * m.nLM + LM) * C + k] = 0ull;
  M1o[static_cast<size_t>(i) * C + k] = f;
  H2o[static_cast<size_t>(i) * C + k] = h2;
  M1_adj_o[static_cast<size_t>(i) * C + k] = m1a;
  H2_adj_o[static_cast<size_t>(i) * C + k] = dh2;
}

// at most 64 registers: eight 128-thread blocks per SM instead of six at 80 (0.129 -> 0.124 ms
// on the 4096-atom workload; 12 bytes of spills).  At this cap the register allocation of
// the whole kernel is sensitive to the split-row block: its row pointer is bumped row by
// row (computing each row's address afresh took 16/24 bytes of spills and 0.010 ms).
template <bool P>
__global__ void __launch_bounds__(256, 4) k_node_tail(DevModel m, const int* __restrict__ ntype, float* __restrict__ A1,
                                                   const float* __restrict__ H1, float* __restrict__ M1o,
                                                   float* __restrict__ H2o, float* __restrict__ A1_adj,
                                                   fix64* __restrict__ H1_adj, float* __restrict__ M1_adj_o,
                                                   float* __restrict__ H2_adj_o, const float* __restrict__ zbl_e,
                                                   double* __restrict__ energies, int N) {
  pdl_begin();
  AtomCursor cur{P ? m.sched : nullptr, N, 0};
  for (int i = cur.first(); i < N; i = cur.next())
    node_tail_atom(m, ntype, A1, H1, M1o, H2o, A1_adj, H1_adj, M1_adj_o, H2_adj_o, zbl_e, energies, N, i);
  cur.done();
}

size_t node_tail_smem(const DevModel& m) { return sizeof(float) * (34 * m.C + 4 * m.C + 33 * 8 + 33); }

void launch_node_tail(const DevModel& m, const int* node_type, int N, float* A1, const float* H1, float* M1,
                      float* H2, float* A1_adj, fix64* H1_adj, float* M1_adj, float* H2_adj, const float* zbl_e,
                      double* energies, cudaStream_t s) {
  if (N <= 0) return;
  DevModel mk;
  const int grid = atom_grid(m, kAkNodeTail, N, mk);
  if (mk.sched)
    launch_pdl(k_node_tail<true>, grid, m.C, node_tail_smem(m), s, mk, node_type, A1, H1, M1, H2, A1_adj, H1_adj,
               M1_adj, H2_adj, zbl_e, energies, N);
  else
    launch_pdl(k_node_tail<false>, grid, m.C, node_tail_smem(m), s, mk, node_type, A1, H1, M1, H2, A1_adj, H1_adj,
               M1_adj, H2_adj, zbl_e, energies, N);
}

void node_tail_residency(const DevModel& m, int* per_sm) {
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[kAkNodeTail], k_node_tail<true>, m.C, node_tail_smem(m));
}

// H1_adj from its fixed-point accumulator: float rows for the SIMT GEMM and the stage
// reads, and in the BF16 form the M0_adj GEMM's split operand rows (write_split with
// `terms` products: row pitch split_xterms(terms) * C; rows grouped by L, lgroup_row).
__global__ void k_fixed_rows(const fix64* __restrict__ src, float* __restrict__ dst, __nv_bfloat16* __restrict__ bf,
                             long rows, int C, int terms) {
  pdl_begin();
  const long n = rows * C;
  for (long t = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<long>(gridDim.x) * blockDim.x) {
    const float v = from_fixed(src[t]);
    dst[t] = v;
    if (bf) {  // (L_max 1: nLM = 4)
      const long r = t / C;
      write_split(bf + lgroup_row(rows >> 2, r >> 2, static_cast<int>(r & 3)) * split_xterms(terms) * C, C, terms,
                  static_cast<int>(t - r * C), v);
    }
  }
}

void launch_fixed_rows(const fix64* src, float* dst, __nv_bfloat16* bf, long rows, int C, int terms, int nLM,
                       cudaStream_t s) {
  if (bf && nLM != 4) throw std::invalid_argument("the split H1_adj rows exist for L_max 1 only");
  if (rows <= 0) return;
  const long n = rows * C;
  const int blocks = static_cast<int>(std::min<long>((n + 255) / 256, 152L * 16));
  launch_pdl(k_fixed_rows, blocks, 256, 0, s, src, dst, bf, rows, C, terms);
}

// Single-stage calls (the reference binding's reverse_Phi1): the fixed-point H1_adj
// accumulator from float rows (zero: from nothing), and the per-edge forces of the layer-1
// adjoint, node_forces = (zero ? 0 : node_forces) - sum over channel slices of f1.
__global__ void k_rows_to_fixed(const float* __restrict__ src, fix64* __restrict__ dst, long n, int zero) {
  for (long t = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<long>(gridDim.x) * blockDim.x)
    dst[t] = zero ? 0ull : to_fixed(src[t]);
}

__global__ void k_forces_from_f1(double* __restrict__ forces, const double* __restrict__ f1, long stride, int nslices,
                                 long n, int zero) {
  for (long t = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<long>(gridDim.x) * blockDim.x) {
    double f = f1[t];
    for (int h = 1; h < nslices; ++h) f += f1[h * stride + t];
    forces[t] = (zero ? 0.0 : forces[t]) - f;
  }
}

void launch_rows_to_fixed(const float* src, fix64* dst, long n, bool zero, cudaStream_t s) {
  if (n <= 0) return;
  k_rows_to_fixed<<<static_cast<int>(std::min<long>((n + 255) / 256, 152L * 16)), 256, 0, s>>>(src, dst, n, zero);
}

void launch_forces_from_f1(double* forces, const double* f1, long stride, int nslices, long n, bool zero,
                           cudaStream_t s) {
  if (n <= 0) return;
  k_forces_from_f1<<<static_cast<int>(std::min<long>((n + 255) / 256, 152L * 16)), 256, 0, s>>>(forces, f1, stride,
                                                                                               nslices, n, zero);
}

// Centre atoms sorted by species (a counting sort; the order inside a species is
// arbitrary: every atom's results are computed the same way whichever block takes it).
// One block.
__global__ void __launch_bounds__(1024) k_species_order(const int* __restrict__ ntype, int N, int S,
                                                        int* __restrict__ order) {
  pdl_begin();
  extern __shared__ int cnt[];  // [S]: counts, then scatter cursors
  for (int t = threadIdx.x; t < S; t += blockDim.x) cnt[t] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) atomicAdd(&cnt[ntype[i]], 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    int o = 0;
    for (int t = 0; t < S; ++t) {
      const int c = cnt[t];
      cnt[t] = o;
      o += c;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) order[atomicAdd(&cnt[ntype[i]], 1)] = i;
}

void launch_species_order(const int* node_type, int N, int S, int* order, cudaStream_t s) {
  if (N <= 0) return;
  launch_pdl(k_species_order, 1, 1024, sizeof(int) * S, s, node_type, N, S, order);
}

// The host API's input check, on the device: flags (a mapped host word) receive one bit
// per violated condition (kBad* in kernels.h); first[] must already be the scan of
// num_neigh.  Grid-stride over max(N, E).
__global__ void k_validate_inputs(int N, long E, int S, double r_cut, const int* __restrict__ node_types,
                                  const int* __restrict__ num_neigh, const int* __restrict__ first,
                                  const int* __restrict__ nidx, const int* __restrict__ ntype_e,
                                  const double* __restrict__ xyz, const double* __restrict__ r,
                                  unsigned* __restrict__ flags) {
  unsigned bad = 0;
  const long n = E > N ? E : N;
  for (long t = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<long>(gridDim.x) * blockDim.x) {
    if (t < N) {
      if (node_types[t] < 0 || node_types[t] >= S) bad |= kBadNodeType;
      if (num_neigh[t] < 0) bad |= kBadNumNeigh;
    }
    if (t < E) {
      if (nidx[t] < 0 || nidx[t] >= N) bad |= kBadNeighIndex;
      if (ntype_e[t] < 0 || ntype_e[t] >= S) bad |= kBadNeighType;
      const double re = r[t];
      if (!(re > 0.0 && re < r_cut) || !isfinite(xyz[3 * t]) || !isfinite(xyz[3 * t + 1]) || !isfinite(xyz[3 * t + 2]))
        bad |= kBadEdge;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && static_cast<long>(first[N]) != E) bad |= kBadEdgeCount;
  bad = __reduce_or_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0 && bad) atomicOr(flags, bad);
}

void launch_validate_inputs(int N, long E, int S, double r_cut, const int* node_types, const int* num_neigh,
                            const int* first, const int* nidx, const int* ntype_e, const double* xyz, const double* r,
                            unsigned* flags, cudaStream_t s) {
  const long n = E > N ? E : N;
  const int grid = static_cast<int>(std::min<long>(ceil_div(n > 0 ? n : 1, 256), 152L * 8));
  k_validate_inputs<<<grid, 256, 0, s>>>(N, E, S, r_cut, node_types, num_neigh, first, nidx, ntype_e, xyz, r, flags);
}

// first[0] = 0, first[i+1] = first[i] + num_neigh[i]; one block, sequential tiles.
__global__ void __launch_bounds__(1024) k_scan_first(const int* __restrict__ num_neigh, int N, int* __restrict__ first) {
  __shared__ int sw[32];
  __shared__ int carry;
  if (threadIdx.x == 0) {
    carry = 0;
    first[0] = 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int base = 0; base < N; base += 1024) {
    const int idx = base + threadIdx.x;
    int v = idx < N ? num_neigh[idx] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sw[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = sw[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      sw[lane] = w;
    }
    __syncthreads();
    const int incl = x + (warp > 0 ? sw[warp - 1] : 0) + carry;
    if (idx < N) first[idx + 1] = incl;
    __syncthreads();
    if (threadIdx.x == 1023) carry = incl;
    __syncthreads();
  }
}

void launch_scan_first(const int* num_neigh, int N, int* first, cudaStream_t s) {
  k_scan_first<<<1, 1024, 0, s>>>(num_neigh, N, first);
}

}  // namespace smx
