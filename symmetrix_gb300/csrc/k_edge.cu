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
// sF, summed across warps in float64 after the chunk.  The lanes first trade halves of
// the vector (x, y | z, 0) with their xor-1 and xor-2 partners, so each lane then holds
// one component summed over its group of four lanes (lane & 3: 0 x, 1 z, 2 y, 3
// nothing), and three butterfly steps sum the groups: six shuffles where three separate
// warp sums take fifteen (k_layer0_rev 0.313 -> 0.283 ms on the 4096-atom workload).
// The order of the additions is fixed, so results are reproducible.
__device__ __forceinline__ void block_reduce3(float fx, float fy, float fz, float (*sF)[8][3], int t) {
  constexpr unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const bool b0 = lane & 1, b1 = lane & 2;
  float k0 = b0 ? fz : fx, k1 = b0 ? 0.0f : fy;
  const float s0 = b0 ? fx : fz, s1 = b0 ? fy : 0.0f;
  k0 += __shfl_xor_sync(kFull, s0, 1);
  k1 += __shfl_xor_sync(kFull, s1, 1);
  float v = b1 ? k1 : k0;
  v += __shfl_xor_sync(kFull, b1 ? k0 : k1, 2);
  v += __shfl_xor_sync(kFull, v, 4);
  v += __shfl_xor_sync(kFull, v, 8);
  v += __shfl_xor_sync(kFull, v, 16);
  if (lane < 3) sF[t][threadIdx.x >> 5][lane == 1 ? 2 : lane == 2 ? 1 : 0] = v;
}

}  // namespace

namespace {

// Edge chunk staged for the layer-0 kernels: Y_lm (and, for the adjoint, dY/dx, dY/dy,
// dY/dz) packed as float4 rows, the ordered-pair spline row of the folded layer-0 table, and the
// compacted list of active edges (r < r_cut).
template <bool GRAD>
struct L0Stage {
  float2 Y2[kEdgeChunk][16];  // (Y_lm, Y_lm): operand of the packed FMAs
  float4 G[GRAD ? kEdgeChunk : 1][16];  // (dY_lm/dx, dY_lm/dy, dY_lm/dz, Y_lm): one load per lm
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
    for (int q = 0; q < 16; ++q) st.Y2[t][q] = make_float2(Y[q], Y[q]);
    if constexpr (GRAD) {
#pragma unroll
      for (int c = 0; c < 16; ++c) st.G[t][c] = make_float4(G[c], G[16 + c], G[32 + c], Y[c]);
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
template <int NLM>
__device__ __forceinline__ void layer0_fwd_atom(const DevModel& m, const EdgeIn& in, float* __restrict__ A0,
                                                float* __restrict__ M0, float* __restrict__ zbl_e, int i) {
  extern __shared__ float dyn[];  // [17][C]: A0 columns (+ constant one) for the contraction
  __shared__ L0Stage<false> st;
  const int C = m.C, C2 = C >> 1, BW = (C2 + 31) & ~31;
  // two groups of channel-pair threads, each taking every other active edge
  const int half = static_cast<int>(threadIdx.x) >= BW ? 1 : 0;
  const int lt = threadIdx.x - half * BW;
  const bool live = lt < C2;
  const int cp = live ? lt : 0, kc = 2 * cp;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.end(i);
  float2 acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = make_float2(0.0f, 0.0f);
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_l0<false>(m, in, ti, eb, ne, st);
    __syncthreads();
    // this group's active edges; the next one's cubics load while this one accumulates
    const int na = st.nact;
    float4 c[8];
    auto fetch = [&](int a) {
      const float4* p = m.spl0 + static_cast<size_t>(st.row[st.act[a]]) * 4 * C + cp;
#pragma unroll
      for (int q = 0; q < 8; ++q) c[q] = __ldg(p + q * C2);
    };
    if (half < na) fetch(half);
    for (int a = half; a < na; a += 2) {
      const int t = st.act[a];
      const float2 x2 = make_float2(st.x[t], st.x[t]);
      float2 R[4];
#pragma unroll
      for (int l = 0; l < 4; ++l) R[l] = spline2_val(c[2 * l], c[2 * l + 1], x2);
      if (a + 2 < na) fetch(a + 2);
      acc[0] = __fadd2_rn(R[0], acc[0]);  // Y_00 = 1 (sph_harm16)
#pragma unroll
      for (int q = 1; q < 16; ++q) {
        const int l = q < 4 ? 1 : (q < 9 ? 2 : 3);
        acc[q] = fma2(R[l], st.Y2[t][q], acc[q]);
      }
    }
  }
  if (m.has_zbl) {  // ZBL energy of node i: sum over its directed edges (zbl.cpp:96-125)
    float z = 0.0f;
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      float V, dV;
      zbl_edge(m, m.zbl_pair[ti * m.S + in.ntype_e[e]], static_cast<float>(in.r[e]), V, dV);
      z += V;
    }
    z = block_sum(z);
    if (threadIdx.x == 0) zbl_e[i] = z;
  }
  float S = 1.0f;
  if (m.dens_spl[0]) {  // density-normalised A0: A0 /= 1 + sum_j s(r_ij)  (mace.cpp:273-297)
    S = dens_factor(m, 0, in, i, ti);
    if (threadIdx.x == 0) m.dens_s[0][i] = S;
  }
  float* sA = dyn;
  if (half == 1 && live)
#pragma unroll
    for (int q = 0; q < 16; ++q) *reinterpret_cast<float2*>(sA + q * C + kc) = acc[q];
  __syncthreads();
  if (half == 0 && live) {
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const float2 o = *reinterpret_cast<const float2*>(sA + q * C + kc);
      float2 v = make_float2(acc[q].x + o.x, acc[q].y + o.y);
      if (S != 1.0f) v = make_float2(v.x / S, v.y / S);  // (no division sequence without the scaling)
      *reinterpret_cast<float2*>(sA + q * C + kc) = v;
      *reinterpret_cast<float2*>(A0 + (static_cast<size_t>(i) * 16 + q) * C + kc) = v;
    }
  }
  for (int k = threadIdx.x; k < C; k += blockDim.x) sA[16 * C + k] = 1.0f;
  __syncthreads();
  // the symmetric contraction, one thread per channel
  for (int k = threadIdx.x; k < C; k += blockDim.x) {
    if (m.poly_canon) {  // generated straight-line polynomials, A0 column in registers
      float x[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) x[q] = sA[q * C + k];
      const float* cf = m.coef0 + static_cast<size_t>(ti * m.nLM) * m.T0 * C + k;
      const size_t sst = static_cast<size_t>(m.T0) * C;
      float* out = M0 + static_cast<size_t>(i) * m.nLM * C + k;
      float v[9];
      v[0] = poly::value_LM0(x, cf, C);
      v[1] = poly::value_LM1(x, cf + sst, C);
      v[2] = poly::value_LM2(x, cf + 2 * sst, C);
      v[3] = poly::value_LM3(x, cf + 3 * sst, C);
      if constexpr (NLM == 9) {  // L_max = 2: the five l = 2 outputs
        v[4] = poly::value_LM4(x, cf + 4 * sst, C);
        v[5] = poly::value_LM5(x, cf + 5 * sst, C);
        v[6] = poly::value_LM6(x, cf + 6 * sst, C);
        v[7] = poly::value_LM7(x, cf + 7 * sst, C);
        v[8] = poly::value_LM8(x, cf + 8 * sst, C);
      }
#pragma unroll
      for (int LM = 0; LM < NLM; ++LM) {
        if (M0) out[LM * C] = v[LM];  // nullptr: only the split rows are consumed
        if (m.op_m0)  // BF16 form: the H1 GEMM's split operand
          write_split(m.op_m0 + (static_cast<size_t>(i) * m.nLM + LM) * split_xterms(m.tc_terms) * C, C, m.tc_terms,
                      k, v[LM]);
      }
      continue;
    }
    for (int LM = 0; LM < m.nLM; ++LM) {
      const int t0 = m.mono0_off[LM], t1 = m.mono0_off[LM + 1];
      const float* cf = m.coef0 + (static_cast<size_t>(ti * m.nLM + LM) * m.T0) * C + k;
      float f = 0.0f;
      for (int t = t0; t < t1; ++t) {
        const int pk = __ldg(m.mono0 + t);
        const float xa = sA[(pk & 255) * C + k], xb = sA[((pk >> 8) & 255) * C + k], xc = sA[(pk >> 16) * C + k];
        f = fmaf(__ldg(cf + static_cast<size_t>(t - t0) * C), xa * xb * xc, f);
      }
      if (M0) M0[(static_cast<size_t>(i) * m.nLM + LM) * C + k] = f;
      if (m.op_m0)
        write_split(m.op_m0 + (static_cast<size_t>(i) * m.nLM + LM) * split_xterms(m.tc_terms) * C, C, m.tc_terms, k,
                    f);
    }
  }
}

template <bool P, int NLM>
__global__ void __launch_bounds__(256) k_layer0_fwd(DevModel m, EdgeIn in, float* __restrict__ A0,
                                                    float* __restrict__ M0, float* __restrict__ zbl_e) {
  pdl_begin();
  AtomCursor cur{P ? m.sched : nullptr, in.N, 0};
  for (int b = cur.first(); b < in.N; b = cur.next())
    layer0_fwd_atom<NLM>(m, in, A0, M0, zbl_e, in.atom_at(b));
  cur.done();
}

// ---------------------------------------------------------------------------
// Layer-0 contraction adjoint (mace.cpp:372-395):
//   A0_adj[i,:,k] = sum_LM M0_adj[i,LM,k] grad P_{ti,LM,k}(A0[i,:,k]).
// Its own kernel, so its register-heavy generated code does not limit the occupancy
// of the layer-0 edge adjoint.
// ---------------------------------------------------------------------------
template <int NLM>
__device__ __forceinline__ void contract0_rev_atom(const DevModel& m, const int* __restrict__ node_type,
                                                   const float* __restrict__ A0, const float* __restrict__ M0_adj,
                                                   float* __restrict__ A0_adj, int i) {
  extern __shared__ float dyn[];
  const int C = m.C, k = threadIdx.x;
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
    if constexpr (NLM == 9) {  // L_max = 2: the five l = 2 outputs
      poly::grad_LM4(x, w[4 * C], cf + 4 * st, C, dA);
      poly::grad_LM5(x, w[5 * C], cf + 5 * st, C, dA);
      poly::grad_LM6(x, w[6 * C], cf + 6 * st, C, dA);
      poly::grad_LM7(x, w[7 * C], cf + 7 * st, C, dA);
      poly::grad_LM8(x, w[8 * C], cf + 8 * st, C, dA);
    }
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

template <bool P, int NLM>
__global__ void __launch_bounds__(256) k_contract0_rev(DevModel m, const int* __restrict__ node_type,
                                                       const float* __restrict__ A0, const float* __restrict__ M0_adj,
                                                       float* __restrict__ A0_adj, int N) {
  pdl_begin();
  AtomCursor cur{P ? m.sched : nullptr, N, 0};
  for (int i = cur.first(); i < N; i = cur.next()) contract0_rev_atom<NLM>(m, node_type, A0, M0_adj, A0_adj, i);
  cur.done();
}



// ---------------------------------------------------------------------------
// Layer-0 edge adjoint (mace.cpp:203-271): dE/dx_ij from A0_adj through the folded
// radial splines and Y_lm; ZBL and the density factor add their terms; forces =
// -(layer 0 + layer 1).  The next active edge's four spline cubics are loaded while
// this edge computes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void layer0_rev_atom(const DevModel& m, const EdgeIn& in, const float* __restrict__ A0_adj,
                                                const double* __restrict__ f1, double* __restrict__ forces, int i) {
  __shared__ L0Stage<true> st;
  __shared__ float sF[kEdgeChunk][8][3];
  const int C = m.C, C2 = C >> 1;
  const bool live = static_cast<int>(threadIdx.x) < C2;
  const int cp = live ? threadIdx.x : 0, kc = 2 * cp;  // this thread's channel pair
  const int nwarp = blockDim.x >> 5;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.end(i);
  const bool local = i < in.n_local;  // a halo centre: layer 0 only
  float2 dA[16];
#pragma unroll
  for (int q = 0; q < 16; ++q)
    dA[q] = *reinterpret_cast<const float2*>(A0_adj + (static_cast<size_t>(i) * 16 + q) * C + kc);
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_l0<true>(m, in, ti, eb, ne, st);
    __syncthreads();
    const int na = st.nact;
    float4 c[8];
    auto fetch = [&](int a) {
      const float4* p = m.spl0 + static_cast<size_t>(st.row[st.act[a]]) * 4 * C + cp;
#pragma unroll
      for (int q = 0; q < 8; ++q) c[q] = __ldg(p + q * C2);
    };
    if (na > 0) fetch(0);
    for (int a = 0; a < na; ++a) {
      const int t = st.act[a];
      const float2 x2 = make_float2(st.x[t], st.x[t]);
      float2 R[4], Rd[4];
#pragma unroll
      for (int l = 0; l < 4; ++l) spline2(c[2 * l], c[2 * l + 1], x2, R[l], Rd[l]);
      if (a + 1 < na) fetch(a + 1);
      float2 dr = make_float2(0.0f, 0.0f);
      float fx = 0.0f, fy = 0.0f, fz = 0.0f;
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        float2 dRl = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int q = l * l; q < (l + 1) * (l + 1); ++q) {
          if (q == 0) {  // Y_00 = 1 with a zero gradient (sph_harm16): the R_0' term alone
            dRl = dA[0];
            continue;
          }
          const float4 g = st.G[t][q];  // (dY/dx, dY/dy, dY/dz, Y)
          dRl = fma2(dA[q], make_float2(g.w, g.w), dRl);
          const float2 w = mul2(dA[q], R[l]);
          const float s = w.x + w.y;
          fx = fmaf(s, g.x, fx);
          fy = fmaf(s, g.y, fy);
          fz = fmaf(s, g.z, fz);
        }
        dr = fma2(dRl, Rd[l], dr);
      }
      const float d = dr.x + dr.y;
      const float4 u = st.u[t];
      fx = fmaf(d, u.x, fx);
      fy = fmaf(d, u.y, fy);
      fz = fmaf(d, u.z, fz);
      if (!live) fx = fy = fz = 0.0f;
      block_reduce3(fx, fy, fz, sF, t);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < ne; t += blockDim.x) {
      const long e = static_cast<long>(eb) + t;
      double s[3] = {0.0, 0.0, 0.0};
      if (st.row[t] >= 0)
        for (int w = 0; w < nwarp; ++w)
          for (int a = 0; a < 3; ++a) s[a] += static_cast<double>(sF[t][w][a]);
      if (m.has_zbl && local) {  // node_forces -= xyz / r * dV_ZBL/dr (zbl.cpp:118-121)
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
      for (int a = 0; a < 3; ++a) {
        double f = 0.0;
        if (local) {
          f = f1[3 * e + a];
          for (int h = 1; h < m.l2_split; ++h) f += f1[h * m.f1_stride + 3 * e + a];  // channel slices (L_max = 2)
        }
        forces[3 * e + a] = -(s[a] + f);
      }
    }
  }
}

template <bool P>
__global__ void __launch_bounds__(128) k_layer0_rev(DevModel m, EdgeIn in, const float* __restrict__ A0_adj,
                                                    const double* __restrict__ f1, double* __restrict__ forces) {
  pdl_begin();
  AtomCursor cur{P ? m.sched : nullptr, in.N, 0};
  for (int b = cur.first(); b < in.N; b = cur.next())
    layer0_rev_atom(m, in, A0_adj, f1, forces, in.atom_at(b));
  cur.done();
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// Dynamic shared memory above 48 KB must be opted into once per kernel (outside
// any stream capture).
cudaError_t init_edge_kernels(const DevModel& m) { return init_layer1_kernels(m); }

// layer-0 edge kernels: one thread per channel pair, whole warps
int layer0_block(int C) { return ((C >> 1) + 31) & ~31; }

// the canonical polynomial outputs compiled into the layer-0 kernels: 9 (L_max = 2) or 4
// (L_max = 1, and every model on the data-driven polynomial path)
template <typename F>
void dispatch_nlm(const DevModel& m, F&& f) {
  if (m.poly_canon && m.nLM == 9)
    f(std::integral_constant<int, 9>{});
  else
    f(std::integral_constant<int, 4>{});
}

void launch_layer0_fwd(const DevModel& m, const EdgeIn& in, float* A0, float* M0, float* zbl_e, cudaStream_t s) {
  if (in.N <= 0) return;
  const size_t smem = 17 * sizeof(float) * m.C;
  DevModel mk;
  const int grid = atom_grid(m, kAkLayer0Fwd, in.N, mk);
  dispatch_nlm(m, [&](auto nc) {
    constexpr int NLM = decltype(nc)::value;
    if (mk.sched)
      launch_pdl(k_layer0_fwd<true, NLM>, grid, 2 * layer0_block(m.C), smem, s, mk, in, A0, M0, zbl_e);
    else
      launch_pdl(k_layer0_fwd<false, NLM>, grid, 2 * layer0_block(m.C), smem, s, mk, in, A0, M0, zbl_e);
  });
}

void launch_layer0_rev(const DevModel& m, const EdgeIn& in, const float* A0, const float* M0_adj, const double* f1,
                       float* A0_adj, double* forces, cudaStream_t s) {
  if (in.N <= 0) return;
  DevModel mk;
  int grid = atom_grid(m, kAkContract0Rev, in.N, mk);
  const size_t smem = m.poly_canon ? 0 : 34 * sizeof(float) * m.C;
  dispatch_nlm(m, [&](auto nc) {
    constexpr int NLM = decltype(nc)::value;
    if (mk.sched)
      launch_pdl(k_contract0_rev<true, NLM>, grid, m.C, smem, s, mk, in.node_type, A0, M0_adj, A0_adj, in.N);
    else
      launch_pdl(k_contract0_rev<false, NLM>, grid, m.C, smem, s, mk, in.node_type, A0, M0_adj, A0_adj, in.N);
  });
  grid = atom_grid(m, kAkLayer0Rev, in.N, mk);
  if (mk.sched)
    launch_pdl(k_layer0_rev<true>, grid, layer0_block(m.C), 0, s, mk, in, A0_adj, f1, forces);
  else
    launch_pdl(k_layer0_rev<false>, grid, layer0_block(m.C), 0, s, mk, in, A0_adj, f1, forces);
}

// resident blocks per SM of the persistent layer-0 kernels at this model's launch shapes
void layer0_residency(const DevModel& m, int* per_sm) {
  dispatch_nlm(m, [&](auto nc) {
    constexpr int NLM = decltype(nc)::value;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[kAkLayer0Fwd], k_layer0_fwd<true, NLM>,
                                                  2 * layer0_block(m.C), 17 * sizeof(float) * m.C);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[kAkContract0Rev], k_contract0_rev<true, NLM>, m.C,
                                                  m.poly_canon ? 0 : 34 * sizeof(float) * m.C);
  });
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[kAkLayer0Rev], k_layer0_rev<true>, layer0_block(m.C), 0);
}

}  // namespace smx
