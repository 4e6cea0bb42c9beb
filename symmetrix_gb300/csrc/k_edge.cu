// Edge kernels: the neighbour sums of both interaction layers and their adjoints.
//
// One thread block per centre node i, one thread per channel k (blockDim = C).
// Edges of node i are staged kernel-wide in chunks of kEdgeChunk: geometry,
// spline interval, Y_lm (and dY/dx in the adjoints) are computed once per edge by
// one thread and shared; every thread then runs the per-channel arithmetic for
// its k with channel-fastest, coalesced loads of spline coefficients (float4:
// one cubic per (spline, channel)) and neighbour features.  Sums over neighbours
// accumulate in registers of the destination node's block, so the forward
// A-basis and Phi1 sums use no atomics.
//
// Reference stages restated here (libsymmetrix/source/mace.cpp):
//   k_layer0_fwd : compute_Y + compute_R0 + compute_A0 (:66-201) + compute_M0 (:348-370)
//   k_layer0_rev : reverse_M0 + reverse_A0 (:372-395, :203-271)
#include <cuda_runtime.h>

#include "device.cuh"
#include "kernels.h"
#include "poly_canon.h"

namespace smx {

namespace {

// Sum a per-thread 3-vector over the block's channels for edge t: float32 warp
// shuffles (float64 arithmetic is slow on this part), then one partial per warp into
// sF, summed across warps in float64 after the chunk.
__device__ __forceinline__ void block_reduce3(float fx, float fy, float fz, float (*sF)[8][3], int t) {
  const float x = warp_sum(fx), y = warp_sum(fy), z = warp_sum(fz);
  if ((threadIdx.x & 31) == 0) {
    const int w = threadIdx.x >> 5;
    sF[t][w][0] = x;
    sF[t][w][1] = y;
    sF[t][w][2] = z;
  }
}

}  // namespace

namespace {

// Edge chunk staged for the layer-0 kernels: Y_lm (and, for the adjoint, dY/dx, dY/dy,
// dY/dz) packed as float4 rows, the ordered-pair spline row of the folded layer-0 table, and the
// compacted list of active edges (r < r_cut).
template <bool GRAD>
struct L0Stage {
  float4 Y[kEdgeChunk][4];
  float4 G[GRAD ? kEdgeChunk : 1][16];  // (dY_lm/dx, dY_lm/dy, dY_lm/dz, 0)
  float4 u[GRAD ? kEdgeChunk : 1];
  float x[kEdgeChunk];
  int row[kEdgeChunk];  // (ti * S + tj) * nint + interval, or -1
  int act[kEdgeChunk];
  int nact;
};

template <bool GRAD>
__device__ __forceinline__ void stage_l0(const DevModel& m, const EdgeIn& in, int ti, int eb, int ne,
                                         L0Stage<GRAD>& st) {
  if (threadIdx.x >= 32) return;
  const int t = threadIdx.x;
  bool active = false;
  if (t < ne) {
    const long e = static_cast<long>(eb) + t;
    const float vx = static_cast<float>(in.xyz[3 * e]);
    const float vy = static_cast<float>(in.xyz[3 * e + 1]);
    const float vz = static_cast<float>(in.xyz[3 * e + 2]);
    const float rr = static_cast<float>(in.r[e]);
    float Y[16], G[GRAD ? 48 : 1];
    sph_harm16<GRAD>(vx, vy, vz, Y, G);
#pragma unroll
    for (int q = 0; q < 4; ++q) st.Y[t][q] = make_float4(Y[4 * q], Y[4 * q + 1], Y[4 * q + 2], Y[4 * q + 3]);
    if constexpr (GRAD) {
#pragma unroll
      for (int c = 0; c < 16; ++c) st.G[t][c] = make_float4(G[c], G[16 + c], G[32 + c], 0.0f);
      const float inv = 1.0f / rr;
      st.u[t] = make_float4(vx * inv, vy * inv, vz * inv, 0.0f);
    }
    int iv = static_cast<int>(rr * m.inv_h);
    iv = iv < 0 ? 0 : (iv >= m.nint ? m.nint - 1 : iv);
    st.x[t] = rr - static_cast<float>(iv) * m.h;
    active = rr < m.r_cut;
    st.row[t] = active ? (ti * m.S + in.ntype_e[e]) * m.nint + iv : -1;
  }
  const unsigned ball = __ballot_sync(0xffffffffu, active);
  if (active) st.act[__popc(ball & ((1u << t) - 1u))] = t;
  if (t == 0) st.nact = __popc(ball);
}

}  // namespace

// ---------------------------------------------------------------------------
// Layer 0 forward: A0[i,lm,k] = sum_j Y_lm(x_ij) R0'_{ti,tj,l}(r_ij)[k] with the
// folded ordered-pair splines, then M0[i,LM,k] = P_{ti,LM,k}(A0[i,:,k]).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_layer0_fwd(DevModel m, EdgeIn in, float* __restrict__ A0,
                                                    float* __restrict__ M0, float* __restrict__ zbl_e) {
  extern __shared__ float dyn[];
  __shared__ L0Stage<false> st;
  const int C = m.C, k = threadIdx.x, i = blockIdx.x;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.first[i + 1];
  float acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = 0.0f;
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_l0<false>(m, in, ti, eb, ne, st);
    __syncthreads();
    // active edges; the next edge's four cubics load while this one accumulates
    const int na = st.nact;
    float4 c[4];
    if (na > 0) {
      const float4* cp = m.spl0 + static_cast<size_t>(st.row[st.act[0]]) * 4 * C + k;
#pragma unroll
      for (int l = 0; l < 4; ++l) c[l] = __ldg(cp + l * C);
    }
    for (int a = 0; a < na; ++a) {
      const int t = st.act[a];
      const float x = st.x[t];
      float R[4];
#pragma unroll
      for (int l = 0; l < 4; ++l) R[l] = spline_val(c[l], x);
      if (a + 1 < na) {
        const float4* cp = m.spl0 + static_cast<size_t>(st.row[st.act[a + 1]]) * 4 * C + k;
#pragma unroll
        for (int l = 0; l < 4; ++l) c[l] = __ldg(cp + l * C);
      }
#pragma unroll
      for (int q4 = 0; q4 < 4; ++q4) {
        const float4 y = st.Y[t][q4];
        const float yy[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int q = 4 * q4 + j;
          const int l = q < 1 ? 0 : (q < 4 ? 1 : (q < 9 ? 2 : 3));
          acc[q] = fmaf(R[l], yy[j], acc[q]);
        }
      }
    }
  }
  if (m.has_zbl) {  // ZBL energy of node i: sum over its directed edges (zbl.cpp:96-125)
    __shared__ float sz[8];
    float z = 0.0f;
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      float V, dV;
      zbl_edge(m, m.zbl_pair[ti * m.S + in.ntype_e[e]], static_cast<float>(in.r[e]), V, dV);
      z += V;
    }
    z = warp_sum(z);
    if ((threadIdx.x & 31) == 0) sz[threadIdx.x >> 5] = z;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.0f;
      for (int w = 0; w < (C >> 5); ++w) t += sz[w];
      zbl_e[i] = t;
    }
  }
  if (m.dens_spl[0]) {  // density-normalised A0: A0 /= 1 + sum_j s(r_ij)  (mace.cpp:273-297)
    const float S = dens_factor(m, 0, in, i, ti);
    if (threadIdx.x == 0) m.dens_s[0][i] = S;
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] /= S;
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) A0[(static_cast<size_t>(i) * 16 + q) * C + k] = acc[q];
  if (m.poly_canon) {  // generated straight-line polynomials, A0 column in registers
    const float* cf = m.coef0 + static_cast<size_t>(ti * m.nLM) * m.T0 * C + k;
    const size_t st = static_cast<size_t>(m.T0) * C;
    float* out = M0 + static_cast<size_t>(i) * m.nLM * C + k;
    const float v[4] = {poly::value_LM0(acc, cf, C), poly::value_LM1(acc, cf + st, C),
                        poly::value_LM2(acc, cf + 2 * st, C), poly::value_LM3(acc, cf + 3 * st, C)};
#pragma unroll
    for (int LM = 0; LM < 4; ++LM) {
      out[LM * C] = v[LM];
      if (m.op_m0)  // BF16 form: the H1 GEMM's split operand
        write_split(m.op_m0 + (static_cast<size_t>(i) * m.nLM + LM) * m.tc_terms * C, C, m.tc_terms, k, v[LM]);
    }
    return;
  }
  float* sA = dyn;  // [17][C]: this thread's A0 column (+ constant one) for the contraction
#pragma unroll
  for (int q = 0; q < 16; ++q) sA[q * C + k] = acc[q];
  sA[16 * C + k] = 1.0f;
  for (int LM = 0; LM < m.nLM; ++LM) {
    const int t0 = m.mono0_off[LM], t1 = m.mono0_off[LM + 1];
    const float* cf = m.coef0 + (static_cast<size_t>(ti * m.nLM + LM) * m.T0) * C + k;
    float f = 0.0f;
    for (int t = t0; t < t1; ++t) {
      const int pk = __ldg(m.mono0 + t);
      const float xa = sA[(pk & 255) * C + k], xb = sA[((pk >> 8) & 255) * C + k], xc = sA[(pk >> 16) * C + k];
      f = fmaf(__ldg(cf + static_cast<size_t>(t - t0) * C), xa * xb * xc, f);
    }
    M0[(static_cast<size_t>(i) * m.nLM + LM) * C + k] = f;
    if (m.op_m0)
      write_split(m.op_m0 + (static_cast<size_t>(i) * m.nLM + LM) * m.tc_terms * C, C, m.tc_terms, k, f);
  }
}

// ---------------------------------------------------------------------------
// Layer-0 contraction adjoint (mace.cpp:372-395):
//   A0_adj[i,:,k] = sum_LM M0_adj[i,LM,k] grad P_{ti,LM,k}(A0[i,:,k]).
// Its own kernel, so its register-heavy generated code does not limit the occupancy
// of the layer-0 edge adjoint.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_contract0_rev(DevModel m, const int* __restrict__ node_type,
                                                       const float* __restrict__ A0, const float* __restrict__ M0_adj,
                                                       float* __restrict__ A0_adj) {
  extern __shared__ float dyn[];
  const int C = m.C, k = threadIdx.x, i = blockIdx.x;
  const int ti = node_type[i];
  float dA[16];
  if (m.poly_canon) {  // dA0 = sum_LM dM0[LM] grad P_LM, generated code, registers only
    float x[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      x[q] = A0[(static_cast<size_t>(i) * 16 + q) * C + k];
      dA[q] = 0.0f;
    }
    const float* cf = m.coef0 + static_cast<size_t>(ti * m.nLM) * m.T0 * C + k;
    const size_t st = static_cast<size_t>(m.T0) * C;
    const float* w = M0_adj + static_cast<size_t>(i) * m.nLM * C + k;
    poly::grad_LM0(x, w[0], cf, C, dA);
    poly::grad_LM1(x, w[C], cf + st, C, dA);
    poly::grad_LM2(x, w[2 * C], cf + 2 * st, C, dA);
    poly::grad_LM3(x, w[3 * C], cf + 3 * st, C, dA);
  } else {  // data-driven monomial lists, this thread's columns in shared memory
    float* sA = dyn;            // [17][C] A0 column
    float* sGd = dyn + 17 * C;  // [17][C] gradient column (row 16 absorbs the constant slot)
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      sA[q * C + k] = A0[(static_cast<size_t>(i) * 16 + q) * C + k];
      sGd[q * C + k] = 0.0f;
    }
    sA[16 * C + k] = 1.0f;
    sGd[16 * C + k] = 0.0f;
    for (int LM = 0; LM < m.nLM; ++LM) {
      const float w = M0_adj[(static_cast<size_t>(i) * m.nLM + LM) * C + k];
      const int t0 = m.mono0_off[LM], t1 = m.mono0_off[LM + 1];
      const float* cf = m.coef0 + (static_cast<size_t>(ti * m.nLM + LM) * m.T0) * C + k;
      for (int t = t0; t < t1; ++t) {
        const int pk = __ldg(m.mono0 + t);
        const int a = pk & 255, b = (pk >> 8) & 255, c = pk >> 16;
        const float cw = __ldg(cf + static_cast<size_t>(t - t0) * C) * w;
        const float xa = sA[a * C + k], xb = sA[b * C + k], xc = sA[c * C + k];
        sGd[a * C + k] += cw * xb * xc;
        sGd[b * C + k] += cw * xa * xc;
        sGd[c * C + k] += cw * xa * xb;
      }
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) dA[q] = sGd[q * C + k];
  }
  if (m.dens_spl[0]) {  // reverse_A0_scaled (mace.cpp:299-346): c_i = dA . A0 / s_i, dA /= s_i
    float dot = 0.0f;
#pragma unroll
    for (int q = 0; q < 16; ++q) dot = fmaf(dA[q], A0[(static_cast<size_t>(i) * 16 + q) * C + k], dot);
    dot = block_sum(dot);
    const float S = m.dens_s[0][i];
    if (threadIdx.x == 0) m.dens_c[0][i] = dot / S;
#pragma unroll
    for (int q = 0; q < 16; ++q) dA[q] /= S;
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) A0_adj[(static_cast<size_t>(i) * 16 + q) * C + k] = dA[q];
}



// ---------------------------------------------------------------------------
// Layer-0 edge adjoint (mace.cpp:203-271): dE/dx_ij from A0_adj through the folded
// radial splines and Y_lm; ZBL and the density factor add their terms; forces =
// -(layer 0 + layer 1).  The next active edge's four spline cubics are loaded while
// this edge computes.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_layer0_rev(DevModel m, EdgeIn in, const float* __restrict__ A0_adj,
                                                    const double* __restrict__ f1, double* __restrict__ forces) {
  __shared__ L0Stage<true> st;
  __shared__ float sF[kEdgeChunk][8][3];
  const int C = m.C, k = threadIdx.x, i = blockIdx.x;
  const int nwarp = C >> 5;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.first[i + 1];
  float dA[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) dA[q] = A0_adj[(static_cast<size_t>(i) * 16 + q) * C + k];
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_l0<true>(m, in, ti, eb, ne, st);
    __syncthreads();
    const int na = st.nact;
    float4 c[4];
    if (na > 0) {
      const float4* cp = m.spl0 + static_cast<size_t>(st.row[st.act[0]]) * 4 * C + k;
#pragma unroll
      for (int l = 0; l < 4; ++l) c[l] = __ldg(cp + l * C);
    }
    for (int a = 0; a < na; ++a) {
      const int t = st.act[a];
      const float x = st.x[t];
      float R[4], Rd[4];
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        R[l] = spline_val(c[l], x);
        Rd[l] = spline_der(c[l], x);
      }
      if (a + 1 < na) {
        const float4* cp = m.spl0 + static_cast<size_t>(st.row[st.act[a + 1]]) * 4 * C + k;
#pragma unroll
        for (int l = 0; l < 4; ++l) c[l] = __ldg(cp + l * C);
      }
      float Y[16];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 v = st.Y[t][q];
        Y[4 * q] = v.x; Y[4 * q + 1] = v.y; Y[4 * q + 2] = v.z; Y[4 * q + 3] = v.w;
      }
      float dr = 0.0f, fx = 0.0f, fy = 0.0f, fz = 0.0f;
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        float dRl = 0.0f;
#pragma unroll
        for (int q = l * l; q < (l + 1) * (l + 1); ++q) {
          dRl = fmaf(dA[q], Y[q], dRl);
          const float w = dA[q] * R[l];
          const float4 g = st.G[t][q];
          fx = fmaf(w, g.x, fx);
          fy = fmaf(w, g.y, fy);
          fz = fmaf(w, g.z, fz);
        }
        dr = fmaf(dRl, Rd[l], dr);
      }
      const float4 u = st.u[t];
      fx = fmaf(dr, u.x, fx);
      fy = fmaf(dr, u.y, fy);
      fz = fmaf(dr, u.z, fz);
      block_reduce3(fx, fy, fz, sF, t);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < ne; t += blockDim.x) {
      const long e = static_cast<long>(eb) + t;
      double s[3] = {0.0, 0.0, 0.0};
      if (st.row[t] >= 0)
        for (int w = 0; w < nwarp; ++w)
          for (int a = 0; a < 3; ++a) s[a] += static_cast<double>(sF[t][w][a]);
      if (m.has_zbl) {  // node_forces -= xyz / r * dV_ZBL/dr (zbl.cpp:118-121)
        float V, dV;
        const double r = in.r[e];
        zbl_edge(m, m.zbl_pair[ti * m.S + in.ntype_e[e]], static_cast<float>(r), V, dV);
        for (int a = 0; a < 3; ++a) s[a] += in.xyz[3 * e + a] / r * static_cast<double>(dV);
      }
      if (m.dens_spl[0]) {  // dE/dx through the layer-0 density factor (mace.cpp:334-339)
        float v, d;
        const double r = in.r[e];
        dens_eval(m, 0, ti, in.ntype_e[e], static_cast<float>(r), v, d);
        const double g = static_cast<double>(m.dens_c[0][i]) * static_cast<double>(d) / r;
        for (int a = 0; a < 3; ++a) s[a] -= g * in.xyz[3 * e + a];
      }
      for (int a = 0; a < 3; ++a) forces[3 * e + a] = -(s[a] + f1[3 * e + a]);
    }
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// Dynamic shared memory above 48 KB must be opted into once per kernel (outside
// any stream capture).
cudaError_t init_edge_kernels(const DevModel& m) { return init_layer1_kernels(m); }

void launch_layer0_fwd(const DevModel& m, const EdgeIn& in, float* A0, float* M0, float* zbl_e, cudaStream_t s) {
  if (in.N <= 0) return;
  const size_t smem = 17 * sizeof(float) * m.C;
  k_layer0_fwd<<<in.N, m.C, smem, s>>>(m, in, A0, M0, zbl_e);
}

void launch_layer0_rev(const DevModel& m, const EdgeIn& in, const float* A0, const float* M0_adj, const double* f1,
                       float* A0_adj, double* forces, cudaStream_t s) {
  if (in.N <= 0) return;
  k_contract0_rev<<<in.N, m.C, m.poly_canon ? 0 : 34 * sizeof(float) * m.C, s>>>(m, in.node_type, A0, M0_adj, A0_adj);
  k_layer0_rev<<<in.N, m.C, 0, s>>>(m, in, A0_adj, f1, forces);
}

}  // namespace smx
