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
//   k_layer1_fwd : compute_R1 + compute_Phi1 (:92-116, :453-502)
//   k_layer1_rev : reverse_Phi1 (:504-605)
//   k_layer0_rev : reverse_M0 + reverse_A0 (:372-395, :203-271)
#include <cuda_runtime.h>

#include "device.cuh"
#include "kernels.h"
#include "poly_canon.h"

namespace smx {

namespace {

// Stage the geometry of edges [eb, eb+ne) of centre node i into shared memory.
// base[t] = spline row (pair * nint + interval) * stride, or -1 if r >= r_cut.
template <bool GRAD>
__device__ __forceinline__ void stage_edges(const DevModel& m, const EdgeIn& in, int ti, int eb, int ne,
                                            bool ordered_pair, int stride, float (*sY)[kEdgeChunk],
                                            float (*sG)[kEdgeChunk], float (*su)[kEdgeChunk], float* sx,
                                            int* sbase, int* sj) {
  for (int t = threadIdx.x; t < ne; t += blockDim.x) {
    const long e = static_cast<long>(eb) + t;
    const float vx = static_cast<float>(in.xyz[3 * e]);
    const float vy = static_cast<float>(in.xyz[3 * e + 1]);
    const float vz = static_cast<float>(in.xyz[3 * e + 2]);
    const float rr = static_cast<float>(in.r[e]);
    float Y[16], G[48];
    sph_harm16<GRAD>(vx, vy, vz, Y, G);
#pragma unroll
    for (int q = 0; q < 16; ++q) sY[q][t] = Y[q];
    if constexpr (GRAD) {
#pragma unroll
      for (int q = 0; q < 48; ++q) sG[q][t] = G[q];
      const float inv = 1.0f / rr;
      su[0][t] = vx * inv;
      su[1][t] = vy * inv;
      su[2][t] = vz * inv;
    }
    int iv = static_cast<int>(rr * m.inv_h);
    iv = iv < 0 ? 0 : (iv >= m.nint ? m.nint - 1 : iv);
    sx[t] = rr - static_cast<float>(iv) * m.h;
    const int tj = in.ntype_e[e];
    int pr;
    if (ordered_pair) {
      pr = ti * m.S + tj;
    } else {
      const int a = ti < tj ? ti : tj, b = ti < tj ? tj : ti;
      pr = a * (2 * m.S - a - 1) / 2 + b;
    }
    sbase[t] = (rr < m.r_cut) ? (pr * m.nint + iv) * stride : -1;
    if (sj) sj[t] = in.nidx[e];
  }
}

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

// ---------------------------------------------------------------------------
// Layer 0 forward: A0[i,lm,k] = sum_j Y_lm(x_ij) R0'_{ti,tj,l}(r_ij)[k] with the
// folded ordered-pair splines, then M0[i,LM,k] = P_{ti,LM,k}(A0[i,:,k]).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_layer0_fwd(DevModel m, EdgeIn in, float* __restrict__ A0,
                                                    float* __restrict__ M0, float* __restrict__ zbl_e) {
  extern __shared__ float dyn[];
  __shared__ float sY[16][kEdgeChunk];
  __shared__ float sx[kEdgeChunk];
  __shared__ int sbase[kEdgeChunk];
  const int C = m.C, k = threadIdx.x, i = blockIdx.x;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.first[i + 1];
  float acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = 0.0f;
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_edges<false>(m, in, ti, eb, ne, true, 4, sY, nullptr, nullptr, sx, sbase, nullptr);
    __syncthreads();
    for (int t = 0; t < ne; ++t) {
      const int base = sbase[t];
      if (base < 0) continue;
      const float4* c = m.spl0 + static_cast<size_t>(base) * C + k;
      const float x = sx[t];
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        const float R = spline_val(__ldg(c + l * C), x);
#pragma unroll
        for (int q = l * l; q < (l + 1) * (l + 1); ++q) acc[q] = fmaf(R, sY[q][t], acc[q]);
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
#pragma unroll
  for (int q = 0; q < 16; ++q) A0[(static_cast<size_t>(i) * 16 + q) * C + k] = acc[q];
  if (m.poly_canon) {  // generated straight-line polynomials, A0 column in registers
    const float* cf = m.coef0 + static_cast<size_t>(ti * m.nLM) * m.T0 * C + k;
    const size_t st = static_cast<size_t>(m.T0) * C;
    float* out = M0 + static_cast<size_t>(i) * m.nLM * C + k;
    out[0] = poly::value_LM0(acc, cf, C);
    out[C] = poly::value_LM1(acc, cf + st, C);
    out[2 * C] = poly::value_LM2(acc, cf + 2 * st, C);
    out[3 * C] = poly::value_LM3(acc, cf + 3 * st, C);
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
  }
}

namespace {

// Edge chunk staged for the layer-1 kernels: Y (and, for the adjoint, dY/dx and the
// unit vector) packed as float4 rows, the spline row, and the compacted list of
// active edges (r < r_cut).
template <bool GRAD>
struct EdgeStage {
  float4 Y[kEdgeChunk][4];              // Y_lm, 16 per edge
  float4 G[GRAD ? kEdgeChunk : 1][12];  // dY_lm/dx, dY_lm/dy, dY_lm/dz
  float4 u[GRAD ? kEdgeChunk : 1];      // unit vector (w unused)
  float x[kEdgeChunk];                  // offset inside the spline interval
  int base[kEdgeChunk];                 // spline row * stride, or -1 (r >= r_cut)
  int j[kEdgeChunk];
  int act[kEdgeChunk];                  // compacted list of active edges
  int nact;
};

// Stage edges [eb, eb+ne) (ne <= 32, all handled by warp 0) with the unordered
// species-pair spline rows of layer 1.
template <bool GRAD>
__device__ __forceinline__ void stage_edges_packed(const DevModel& m, const EdgeIn& in, int ti, int eb, int ne,
                                                   int stride, EdgeStage<GRAD>& st) {
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
      for (int q = 0; q < 12; ++q) st.G[t][q] = make_float4(G[4 * q], G[4 * q + 1], G[4 * q + 2], G[4 * q + 3]);
      const float inv = 1.0f / rr;
      st.u[t] = make_float4(vx * inv, vy * inv, vz * inv, 0.0f);
    }
    int iv = static_cast<int>(rr * m.inv_h);
    iv = iv < 0 ? 0 : (iv >= m.nint ? m.nint - 1 : iv);
    st.x[t] = rr - static_cast<float>(iv) * m.h;
    const int tj = in.ntype_e[e];
    const int a = ti < tj ? ti : tj, b = ti < tj ? tj : ti;
    const int pr = a * (2 * m.S - a - 1) / 2 + b;
    active = rr < m.r_cut;
    st.base[t] = active ? (pr * m.nint + iv) * stride : -1;
    st.j[t] = in.nidx[e];
  }
  const unsigned ball = __ballot_sync(0xffffffffu, active);
  if (active) st.act[__popc(ball & ((1u << t) - 1u))] = t;
  if (t == 0) st.nact = __popc(ball);
}

// Gather the spline row (NI float4 cubics) and neighbour features (NL2 floats) of
// active edge a of the staged chunk for channel k.
template <int NI, int NL2, bool GRAD>
__device__ __forceinline__ void fetch_edge(const DevModel& m, const float* __restrict__ H1, const EdgeStage<GRAD>& st,
                                           int a, int C, int k, float4* c, float* h) {
  const int t = st.act[a];
  const float4* cp = m.spl1 + static_cast<size_t>(st.base[t]) * C + k;
#pragma unroll
  for (int q = 0; q < NI; ++q) c[q] = __ldg(cp + q * C);
  const float* hj = H1 + static_cast<size_t>(st.j[t]) * NL2 * C + k;
#pragma unroll
  for (int q = 0; q < NL2; ++q) h[q] = __ldg(hj + q * C);
}

}  // namespace

// ---------------------------------------------------------------------------
// Layer 1 forward: Phi1r[i,p,k] = sum_j R1_q(r_ij)[k] Y_{l1 m1}(x_ij) H1[j, l2 m2, k]
// accumulated in registers (p = (instruction, m1, m2), canonical order), then
// Phi1[i,lme,k] = sum_p CG[lme,p] Phi1r[i,p,k].
// ---------------------------------------------------------------------------
template <int LMAX>
__global__ void __launch_bounds__(256) k_layer1_fwd(DevModel m, EdgeIn in, const float* __restrict__ H1,
                                                    float* __restrict__ Phi1) {
  constexpr int NL2 = (LMAX + 1) * (LMAX + 1);
  constexpr int NI = ins_count(LMAX);
  constexpr int NP = ins_np(LMAX);
  extern __shared__ float dyn[];
  __shared__ EdgeStage<false> st;
  const int C = m.C, k = threadIdx.x, i = blockIdx.x;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.first[i + 1];
  float acc[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) acc[p] = 0.0f;
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_edges_packed<false>(m, in, ti, eb, ne, NI, st);
    __syncthreads();
    // (the accumulators leave no registers for a prefetch of the next edge: residency
    // of four blocks per SM hides the gather latency instead)
    const int na = st.nact;
    for (int a = 0; a < na; ++a) {
      const int t = st.act[a];
      const float x = st.x[t];
      float hv[NL2];
      const float* hj = H1 + static_cast<size_t>(st.j[t]) * NL2 * C + k;
#pragma unroll
      for (int q = 0; q < NL2; ++q) hv[q] = __ldg(hj + q * C);
      const float4* cp = m.spl1 + static_cast<size_t>(st.base[t]) * C + k;
      const float* Y = reinterpret_cast<const float*>(st.Y[t]);
      for_each_ins<LMAX>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        constexpr int l1 = ins_l1(LMAX, q), l2 = ins_l2(LMAX, q), p0 = ins_poff(LMAX, q);
        const float R = spline_val(__ldg(cp + q * C), x);
#pragma unroll
        for (int a1 = 0; a1 < 2 * l1 + 1; ++a1) {
          const float ry = R * Y[l1 * l1 + a1];
#pragma unroll
          for (int b = 0; b < 2 * l2 + 1; ++b)
            acc[p0 + a1 * (2 * l2 + 1) + b] = fmaf(ry, hv[l2 * l2 + b], acc[p0 + a1 * (2 * l2 + 1) + b]);
        }
      });
    }
  }
  float* sP = dyn;  // [NP][C]: this thread's Phi1r column
#pragma unroll
  for (int p = 0; p < NP; ++p) sP[p * C + k] = acc[p];
  for (int lme = 0; lme < m.n_lme; ++lme) {
    float s = 0.0f;
    const int g1 = __ldg(m.cg_fwd_off + lme + 1);
    for (int g = __ldg(m.cg_fwd_off + lme); g < g1; ++g) s = fmaf(__ldg(m.cg_fwd_v + g), sP[__ldg(m.cg_fwd_p + g) * C + k], s);
    Phi1[(static_cast<size_t>(i) * m.n_lme + lme) * C + k] = s;
  }
}

// ---------------------------------------------------------------------------
// Layer 1 adjoint.  g[p] = sum_lme CG[lme,p] dPhi1[i,lme,k]; per edge:
//   dE/dx_ij += sum_k sum_p g_p h_{m2} (R1'_q(r) u Y_{m1} + R1_q(r) dY_{m1}/dx)
//   H1_adj[j, l2 m2, k] += sum_p R1_q(r) Y_{m1} g_p        (atomic scatter)
// f1[e] receives dE/dx_ij from this layer.
//
// Edges of a chunk are compacted to the active ones (r < r_cut) and processed two at
// a time: the two edges' dependent FMA chains interleave, which is what keeps the FMA
// pipe busy at the two resident warps per scheduler the register budget allows.
// ---------------------------------------------------------------------------
namespace {

// One edge of the layer-1 adjoint for this thread's channel.
template <int LMAX>
__device__ __forceinline__ void l1_rev_edge(const float* g, const float* Rv, const float* Rdv, const float4* Yrow,
                                            const float4* Grow, float4 u, const float* hv, float* hadj, float& fx,
                                            float& fy, float& fz) {
  constexpr int NL2 = (LMAX + 1) * (LMAX + 1);
  float Y[16];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float4 v = Yrow[q];
    Y[4 * q] = v.x; Y[4 * q + 1] = v.y; Y[4 * q + 2] = v.z; Y[4 * q + 3] = v.w;
  }
  float dY[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) dY[q] = 0.0f;
  float hA[NL2], hB[NL2];  // two partial sums per H1_adj component (shorter chains)
#pragma unroll
  for (int q = 0; q < NL2; ++q) hA[q] = hB[q] = 0.0f;
  float drA = 0.0f, drB = 0.0f;
  for_each_ins<LMAX>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    constexpr int l1 = ins_l1(LMAX, q), l2 = ins_l2(LMAX, q), p0 = ins_poff(LMAX, q);
    const float R = Rv[q], Rd = Rdv[q];
    float dRq = 0.0f;
#pragma unroll
    for (int a = 0; a < 2 * l1 + 1; ++a) {
      const float y = Y[l1 * l1 + a];
      float gs = 0.0f;
#pragma unroll
      for (int b = 0; b < 2 * l2 + 1; ++b) gs = fmaf(g[p0 + a * (2 * l2 + 1) + b], hv[l2 * l2 + b], gs);
      dRq = fmaf(gs, y, dRq);
      dY[l1 * l1 + a] = fmaf(R, gs, dY[l1 * l1 + a]);
      const float ry = R * y;
#pragma unroll
      for (int b = 0; b < 2 * l2 + 1; ++b) {
        if ((q + a) & 1)
          hB[l2 * l2 + b] = fmaf(ry, g[p0 + a * (2 * l2 + 1) + b], hB[l2 * l2 + b]);
        else
          hA[l2 * l2 + b] = fmaf(ry, g[p0 + a * (2 * l2 + 1) + b], hA[l2 * l2 + b]);
      }
    }
    if (q & 1) drB = fmaf(dRq, Rd, drB);
    else drA = fmaf(dRq, Rd, drA);
  });
#pragma unroll
  for (int q = 0; q < NL2; ++q) hadj[q] = hA[q] + hB[q];
  const float dr = drA + drB;
  float ax = dr * u.x, ay = dr * u.y, az = dr * u.z;
  float bx = 0.0f, by = 0.0f, bz = 0.0f;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float4 gx = Grow[q], gy = Grow[4 + q], gz = Grow[8 + q];
    ax = fmaf(dY[4 * q], gx.x, ax); ay = fmaf(dY[4 * q], gy.x, ay); az = fmaf(dY[4 * q], gz.x, az);
    bx = fmaf(dY[4 * q + 1], gx.y, bx); by = fmaf(dY[4 * q + 1], gy.y, by); bz = fmaf(dY[4 * q + 1], gz.y, bz);
    ax = fmaf(dY[4 * q + 2], gx.z, ax); ay = fmaf(dY[4 * q + 2], gy.z, ay); az = fmaf(dY[4 * q + 2], gz.z, az);
    bx = fmaf(dY[4 * q + 3], gx.w, bx); by = fmaf(dY[4 * q + 3], gy.w, by); bz = fmaf(dY[4 * q + 3], gz.w, bz);
  }
  fx = ax + bx;
  fy = ay + by;
  fz = az + bz;
}

}  // namespace

template <int LMAX>
__global__ void __launch_bounds__(256) k_layer1_rev(DevModel m, EdgeIn in, const float* __restrict__ H1,
                                                    const float* __restrict__ dPhi1, float* __restrict__ H1_adj,
                                                    double* __restrict__ f1) {
  constexpr int NL2 = (LMAX + 1) * (LMAX + 1);
  constexpr int NI = ins_count(LMAX);
  constexpr int NP = ins_np(LMAX);
  extern __shared__ float dyn[];
  __shared__ EdgeStage<true> st;
  __shared__ float sF[kEdgeChunk][8][3];
  const int C = m.C, k = threadIdx.x, i = blockIdx.x;
  const int nwarp = C >> 5;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.first[i + 1];
  // g[p] = sum_lme CG[lme,p] dPhi1[i,lme,k], formed in this thread's shared-memory
  // column (data-driven indices) and then moved to registers with constant indices
  float* sD = dyn;                 // [n_lme][C]
  float* sP = dyn + m.n_lme * C;   // [NP][C]
  for (int lme = 0; lme < m.n_lme; ++lme) sD[lme * C + k] = dPhi1[(static_cast<size_t>(i) * m.n_lme + lme) * C + k];
  for (int p = 0; p < NP; ++p) {
    float s = 0.0f;
    const int q1 = __ldg(m.cg_rev_off + p + 1);
    for (int q = __ldg(m.cg_rev_off + p); q < q1; ++q) s = fmaf(__ldg(m.cg_rev_v + q), sD[__ldg(m.cg_rev_lme + q) * C + k], s);
    sP[p * C + k] = s;
  }
  float g[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) g[p] = sP[p * C + k];
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_edges_packed<true>(m, in, ti, eb, ne, NI, st);
    __syncthreads();
    // Active edges one at a time.  The spline row of an edge is reduced to R and R'
    // first; the gathers of the next edge's spline row and neighbour features are then
    // issued into the freed registers, so their L2 latency overlaps the rest of this
    // edge's arithmetic.
    const int na = st.nact;
    float4 c[NI];
    float h[NL2];
    if (na > 0) fetch_edge<NI, NL2>(m, H1, st, 0, C, k, c, h);
    for (int a = 0; a < na; ++a) {
      const int t = st.act[a];
      const float x = st.x[t];
      float R[NI], Rd[NI], hv[NL2];
#pragma unroll
      for (int q = 0; q < NI; ++q) {
        R[q] = spline_val(c[q], x);
        Rd[q] = spline_der(c[q], x);
      }
#pragma unroll
      for (int q = 0; q < NL2; ++q) hv[q] = h[q];
      const int j = st.j[t];
      if (a + 1 < na) fetch_edge<NI, NL2>(m, H1, st, a + 1, C, k, c, h);
      float hadj[NL2], fx, fy, fz;
      l1_rev_edge<LMAX>(g, R, Rd, st.Y[t], st.G[t], st.u[t], hv, hadj, fx, fy, fz);
      block_reduce3(fx, fy, fz, sF, t);
      float* dst = H1_adj + static_cast<size_t>(j) * NL2 * C + k;
#pragma unroll
      for (int q = 0; q < NL2; ++q) atomicAdd(dst + q * C, hadj[q]);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < ne; t += blockDim.x) {
      double s[3] = {0.0, 0.0, 0.0};
      if (st.base[t] >= 0)
        for (int w = 0; w < nwarp; ++w)
          for (int c = 0; c < 3; ++c) s[c] += static_cast<double>(sF[t][w][c]);
      for (int c = 0; c < 3; ++c) f1[3 * (static_cast<long>(eb) + t) + c] = s[c];
    }
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
#pragma unroll
  for (int q = 0; q < 16; ++q) A0_adj[(static_cast<size_t>(i) * 16 + q) * C + k] = dA[q];
}

// ---------------------------------------------------------------------------
// Layer 0 edge adjoint, from dA0 (k_contract0_rev):
//   dE/dx_ij = sum_k sum_lm dA0[lm] (R0'_l'(r) u Y_lm + R0'_l(r) dY_lm/dx)
// and node_forces[e] = -(layer-0 + layer-1 contributions), in float64.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_layer0_rev(DevModel m, EdgeIn in, const float* __restrict__ A0_adj,
                                                    const double* __restrict__ f1, double* __restrict__ forces) {
  __shared__ float sY[16][kEdgeChunk];
  __shared__ float sG[48][kEdgeChunk];
  __shared__ float su[3][kEdgeChunk];
  __shared__ float sx[kEdgeChunk];
  __shared__ int sbase[kEdgeChunk];
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
    stage_edges<true>(m, in, ti, eb, ne, true, 4, sY, sG, su, sx, sbase, nullptr);
    __syncthreads();
    for (int t = 0; t < ne; ++t) {
      const int base = sbase[t];
      if (base < 0) {
        if ((threadIdx.x & 31) == 0) sF[t][threadIdx.x >> 5][0] = sF[t][threadIdx.x >> 5][1] = sF[t][threadIdx.x >> 5][2] = 0.0f;
        continue;
      }
      const float4* c = m.spl0 + static_cast<size_t>(base) * C + k;
      const float x = sx[t];
      float dr = 0.0f, fx = 0.0f, fy = 0.0f, fz = 0.0f;
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        const float4 cc = __ldg(c + l * C);
        const float R = spline_val(cc, x), Rd = spline_der(cc, x);
        float dRl = 0.0f;
#pragma unroll
        for (int q = l * l; q < (l + 1) * (l + 1); ++q) {
          dRl = fmaf(dA[q], sY[q][t], dRl);
          const float w = dA[q] * R;
          fx = fmaf(w, sG[q][t], fx);
          fy = fmaf(w, sG[16 + q][t], fy);
          fz = fmaf(w, sG[32 + q][t], fz);
        }
        dr = fmaf(dRl, Rd, dr);
      }
      fx = fmaf(dr, su[0][t], fx);
      fy = fmaf(dr, su[1][t], fy);
      fz = fmaf(dr, su[2][t], fz);
      block_reduce3(fx, fy, fz, sF, t);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < ne; t += blockDim.x) {
      const long e = static_cast<long>(eb) + t;
      double s[3] = {0.0, 0.0, 0.0};
      for (int w = 0; w < nwarp; ++w)
        for (int a = 0; a < 3; ++a) s[a] += static_cast<double>(sF[t][w][a]);
      if (m.has_zbl) {  // node_forces -= xyz / r * dV_ZBL/dr (zbl.cpp:118-121)
        float V, dV;
        const double r = in.r[e];
        zbl_edge(m, m.zbl_pair[ti * m.S + in.ntype_e[e]], static_cast<float>(r), V, dV);
        for (int a = 0; a < 3; ++a) s[a] += in.xyz[3 * e + a] / r * static_cast<double>(dV);
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
cudaError_t init_edge_kernels(const DevModel& m) {
  cudaError_t e = cudaFuncSetAttribute(k_layer1_fwd<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sizeof(float) * ins_np(1) * m.C));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_layer1_rev<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(sizeof(float) * (m.n_lme + ins_np(1)) * m.C));
}

void launch_layer0_fwd(const DevModel& m, const EdgeIn& in, float* A0, float* M0, float* zbl_e, cudaStream_t s) {
  if (in.N <= 0) return;
  const size_t smem = 17 * sizeof(float) * m.C;
  k_layer0_fwd<<<in.N, m.C, smem, s>>>(m, in, A0, M0, zbl_e);
}

void launch_layer1_fwd(const DevModel& m, const EdgeIn& in, const float* H1, float* Phi1, cudaStream_t s) {
  if (in.N <= 0) return;
  const size_t smem = sizeof(float) * ins_np(1) * m.C;
  k_layer1_fwd<1><<<in.N, m.C, smem, s>>>(m, in, H1, Phi1);
}

void launch_layer1_rev(const DevModel& m, const EdgeIn& in, const float* H1, const float* dPhi1, float* H1_adj,
                       double* f1, cudaStream_t s) {
  if (in.N <= 0) return;
  const size_t smem = sizeof(float) * (m.n_lme + ins_np(1)) * m.C;
  k_layer1_rev<1><<<in.N, m.C, smem, s>>>(m, in, H1, dPhi1, H1_adj, f1);
}

void launch_layer0_rev(const DevModel& m, const EdgeIn& in, const float* A0, const float* M0_adj, const double* f1,
                       float* A0_adj, double* forces, cudaStream_t s) {
  if (in.N <= 0) return;
  k_contract0_rev<<<in.N, m.C, m.poly_canon ? 0 : 34 * sizeof(float) * m.C, s>>>(m, in.node_type, A0, M0_adj, A0_adj);
  k_layer0_rev<<<in.N, m.C, 0, s>>>(m, in, A0_adj, f1, forces);
}

}  // namespace smx
