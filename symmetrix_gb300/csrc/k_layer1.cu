// Layer-1 edge kernels: the tensor-product neighbour sum and its adjoint.
//
// Reference stages restated here (libsymmetrix/source/mace.cpp):
//   k_layer1_fwd : compute_R1 + compute_Phi1 (:92-116, :453-502)
//   k_layer1_rev : reverse_Phi1 (:504-605)
//
// Every kernel works on one centre node at a time: one block per node, or a persistent
// grid claiming nodes (AtomCursor), in the order EdgeIn::atom_at gives.
//
// The adjoint (the costlier kernel): a thread owns a channel pair (2c, 2c+1) and
// one half of the layer-1 instructions: the block is two groups of HW threads
// (HW = C/2 rounded up to a warp), group 0 runs the instructions of half 0 and
// group 1 those of half 1, so the split is warp-uniform.  All per-channel
// arithmetic is on float2 pairs with the packed FP32 FMA of sm_100 and later
// (__ffma2_rn: two IEEE single-precision FMAs per issued instruction).  These kernels
// are issue-bound, so the packed form halves their instruction stream, and the
// instruction split halves the per-thread footprint of the CG-contracted adjoint g.
//
// Spline rows of layer 1 are packed for channel pairs (model.cpp): for each
// instruction, two planes of C/2 float4: plane 0 = (c0, c0', c1, c1') and plane 1 =
// (c2, c2', c3, c3'), ' marking the odd channel of the pair, so that every cubic
// coefficient pair is one aligned float2 operand.
//
// L_max = 2 (17 instructions, 243 paths): four instruction groups, one channel per
// thread, scalar FMAs; from 64 channels each node's channels are split over two blocks
// (DevModel::l2_split) so that two blocks share an SM.
#include <cuda_runtime.h>

#include <algorithm>

#include "device.cuh"
#include "kernels.h"

namespace smx {

namespace {

// ---------------------------------------------------------------------------
// Instruction halves for L_max = 1 (canonical instruction order, see ins_l1/ins_l2):
// {1, 6, 7, 8} and {0, 2, 3, 4, 5, 9}.  Chosen by exhaustive search over the 2^10
// splits for equal packed-FMA work per edge (spline + per-row terms: 212 vs 210) and
// near-equal CG path counts (46 vs 42 register pairs).
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int half_count(int H) { return H == 0 ? 4 : 6; }
__host__ __device__ constexpr int half_ins(int H, int i) {
  constexpr int h0[4] = {1, 6, 7, 8};
  constexpr int h1[6] = {0, 2, 3, 4, 5, 9};
  return H == 0 ? h0[i] : h1[i];
}
// number of CG paths (l1 m1, l2 m2) of instruction q
__host__ __device__ constexpr int ins_paths(int LMAX, int q) {
  return (2 * ins_l1(LMAX, q) + 1) * (2 * ins_l2(LMAX, q) + 1);
}
// offset of the i-th instruction of half H inside the half's path list
template <int LMAX, int H>
__host__ __device__ constexpr int half_goff(int i) {
  int s = 0;
  for (int w = 0; w < i; ++w) s += ins_paths(LMAX, half_ins(H, w));
  return s;
}
template <int LMAX, int H>
__host__ __device__ constexpr int half_np() {
  return half_goff<LMAX, H>(half_count(H));
}
// does half H use Y component c (lm index)?
template <int LMAX, int H>
__host__ __device__ constexpr bool half_uses_y(int c) {
  for (int w = 0; w < half_count(H); ++w) {
    const int l1 = ins_l1(LMAX, half_ins(H, w));
    if (c >= l1 * l1 && c < (l1 + 1) * (l1 + 1)) return true;
  }
  return false;
}

// Sum a per-thread 3-vector over the block for edge t (float32 shuffles; one
// partial per warp into sF, summed across warps in float64 after the chunk).  The
// six-shuffle exchange form of k_edge.cu measured slower here (0.692 -> 0.709 ms on the
// 4096-atom workload): three plain butterflies.
__device__ __forceinline__ void block_reduce3(float fx, float fy, float fz, float (*sF)[8][3], int t) {
  const float x = warp_sum(fx), y = warp_sum(fy), z = warp_sum(fz);
  if ((threadIdx.x & 31) == 0) {
    const int w = threadIdx.x >> 5;
    sF[t][w][0] = x;
    sF[t][w][1] = y;
    sF[t][w][2] = z;
  }
}

// sum_p CG[lme,p] sP[p][k] over row lme of the padded forward table, KF terms, all loads
// independent
template <int KF>
__device__ __forceinline__ float cg_row(const int2* __restrict__ row, const float* sP, int stride, int k) {
  int2 t[KF];
#pragma unroll
  for (int u = 0; u < KF; ++u) t[u] = __ldg(row + u);
  float s = 0.0f;
#pragma unroll
  for (int u = 0; u < KF; ++u) s = fmaf(__int_as_float(t[u].y), sP[t[u].x * stride + k], s);
  return s;
}

// f(std::integral_constant<int, KF>) for the padded forward table's row length, KF = 0
// for the compressed-row walk (no padded table)
template <typename F>
__device__ __forceinline__ void dispatch_kf(int kp, F&& f) {
  switch (kp) {
    case 1: f(std::integral_constant<int, 1>{}); break;
    case 2: f(std::integral_constant<int, 2>{}); break;
    case 3: f(std::integral_constant<int, 3>{}); break;
    case 4: f(std::integral_constant<int, 4>{}); break;
    case 5: f(std::integral_constant<int, 5>{}); break;
    case 6: f(std::integral_constant<int, 6>{}); break;
    case 7: f(std::integral_constant<int, 7>{}); break;
    case 8: f(std::integral_constant<int, 8>{}); break;
    default: f(std::integral_constant<int, 0>{}); break;
  }
}

// Phi1[i,lme,k] = sum_p CG[lme,p] sP[p][k] for the rows lme with (lme mod nrow_groups) ==
// row_group (the BF16 form also writes them as the A1 GEMM's split operand, regrouped per
// l); sP holds this block's channels with row stride `stride`, k is the global channel
template <int KF>
__device__ __forceinline__ void l1_fwd_epilogue(const DevModel& m, int N, int i, const float* sP, int stride, int kk,
                                                int k, int row_group, int nrow_groups, float* __restrict__ Phi1) {
  const int C = m.C, T = m.tc_terms, XT = split_xterms(T);
  for (int l = 0; l < 4; ++l) {
    const int ne = m.num_e[l], Kl = ne * C;
    for (int mm = 0; mm < 2 * l + 1; ++mm)
      for (int e = 0; e < ne; ++e) {
        const int lme = m.lme_off[l] + mm * ne + e;
        if (lme % nrow_groups != row_group) continue;
        float s = 0.0f;
        if constexpr (KF > 0) {
          s = cg_row<KF>(m.cg_fwd_pad + static_cast<size_t>(lme) * KF, sP, stride, kk);
        } else {
          const int p1 = __ldg(m.cg_fwd_off + lme + 1);
          for (int p = __ldg(m.cg_fwd_off + lme); p < p1; ++p)
            s = fmaf(__ldg(m.cg_fwd_v + p), sP[__ldg(m.cg_fwd_p + p) * stride + kk], s);
        }
        if (Phi1) Phi1[(static_cast<size_t>(i) * m.n_lme + lme) * C + k] = s;  // nullptr: split rows only
        if (m.op_phi1) {
          __nv_bfloat16* row = m.op_phi1 + static_cast<size_t>(XT) * N * m.lme_off[l] * C +
                               (static_cast<size_t>(i) * (2 * l + 1) + mm) * XT * Kl;
          write_split(row, Kl, T, e * C + k, s);
        }
      }
  }
}

// Edge chunk staged for the layer-1 kernels.
template <bool GRAD>
struct L1Stage {
  float2 Y2[kEdgeChunk][16];            // (Y_lm, Y_lm): operand of the packed FMAs
  float4 G[GRAD ? kEdgeChunk : 1][16];  // (dY_lm/dx, dY_lm/dy, dY_lm/dz, 0)
  float4 u[GRAD ? kEdgeChunk : 1];      // unit vector (w unused)
  float x[kEdgeChunk];                  // offset inside the spline interval
  int row[kEdgeChunk];                  // spline row (pair * nint + interval), or -1
  int j[kEdgeChunk];
  int act[kEdgeChunk];                  // compacted list of active edges (r < r_cut)
  int nact;
};

// Stage edges [eb, eb+ne) (ne <= 32; warp 0) with the unordered species-pair rows.
template <bool GRAD>
__device__ __forceinline__ void stage_l1(const DevModel& m, const EdgeIn& in, int ti, int eb, int ne,
                                         L1Stage<GRAD>& st) {
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
    for (int c = 0; c < 16; ++c) st.Y2[t][c] = make_float2(Y[c], Y[c]);
    if constexpr (GRAD) {
#pragma unroll
      for (int c = 0; c < 16; ++c) st.G[t][c] = make_float4(G[c], G[16 + c], G[32 + c], 0.0f);
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
    st.row[t] = active ? pr * m.nint + iv : -1;
    st.j[t] = in.nidx[e];
  }
  const unsigned ball = __ballot_sync(0xffffffffu, active);
  if (active) st.act[__popc(ball & ((1u << t) - 1u))] = t;
  if (t == 0) st.nact = __popc(ball);
}

// Per-thread view of the block layout.
struct Lane2 {
  int C, C2;   // channels, channel pairs
  int cp;      // this thread's channel pair (clamped to a valid one on idle lanes)
  int kc;      // first channel of the pair
  bool live;   // owns a real channel pair
};

// Gather the spline coefficients of half H's instructions for spline row `row` and
// the neighbour features H1[j] of this channel pair.
template <int LMAX, int H, int NL2>
__device__ __forceinline__ void fetch_l1(const DevModel& m, const float* __restrict__ H1, int row, int j,
                                         const Lane2& L, float4* c, float2* h) {
  const float4* rp = m.spl1 + static_cast<size_t>(row) * ins_count(LMAX) * L.C + L.cp;
  static_for<half_count(H)>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    constexpr int q = half_ins(H, i);
    c[2 * i] = __ldg(rp + (2 * q) * L.C2);
    c[2 * i + 1] = __ldg(rp + (2 * q + 1) * L.C2);
  });
  const float2* hp = reinterpret_cast<const float2*>(H1 + static_cast<size_t>(j) * NL2 * L.C + L.kc);
#pragma unroll
  for (int b = 0; b < NL2; ++b) h[b] = __ldg(hp + b * L.C2);
}

// Read half H's CG-contracted adjoint pairs from the block's [NP][C] column array.
template <int LMAX, int H>
__device__ __forceinline__ void l1_load_g(const float* sP, const Lane2& L, float2* g) {
  static_for<half_count(H)>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    constexpr int q = half_ins(H, i);
    constexpr int np = ins_paths(LMAX, q), p0 = ins_poff(LMAX, q), g0 = half_goff<LMAX, H>(i);
#pragma unroll
    for (int p = 0; p < np; ++p) g[g0 + p] = *reinterpret_cast<const float2*>(sP + (p0 + p) * L.C + L.kc);
  });
}

// g_p for this thread's channel pair straight from the node's staged dPhi1 rows (sD,
// [n_lme][C]) through the two-term padded CG table
template <int LMAX, int H>
__device__ __forceinline__ void l1_load_g_sd(const DevModel& m, const float* sD, const Lane2& L, float2* g) {
  static_for<half_count(H)>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    constexpr int q = half_ins(H, i);
    constexpr int np = ins_paths(LMAX, q), p0 = ins_poff(LMAX, q), g0 = half_goff<LMAX, H>(i);
#pragma unroll
    for (int p = 0; p < np; ++p) {
      const int2 t0 = __ldg(m.cg_rev_pad + 2 * (p0 + p)), t1 = __ldg(m.cg_rev_pad + 2 * (p0 + p) + 1);
      const float2 d0 = *reinterpret_cast<const float2*>(sD + t0.x * L.C + L.kc);
      const float2 d1 = *reinterpret_cast<const float2*>(sD + t1.x * L.C + L.kc);
      const float v0 = __int_as_float(t0.y), v1 = __int_as_float(t1.y);
      g[g0 + p] = make_float2(fmaf(v1, d1.x, v0 * d0.x), fmaf(v1, d1.y, v0 * d0.y));
    }
  });
}

// ---------------------------------------------------------------------------
// Adjoint, one edge, half H.  With g_p = sum_lme CG[lme,p] dPhi1[i,lme,k]:
//   dE/dx_ij += sum_k sum_p g_p h_{m2} (R1'_q u Y_{m1} + R1_q dY_{m1}/dx)
//   H1_adj[j, l2 m2, k] += sum_p R1_q Y_{m1} g_p
// ---------------------------------------------------------------------------
template <int LMAX, int H>
__device__ __forceinline__ void l1_rev_edge(const float2* g, const float2* R, const float2* Rd, const float2* Y2,
                                            const float4* G, float4 u, const float2* hv, float2* hadj, float& fx,
                                            float& fy, float& fz) {
  constexpr int NL2 = (LMAX + 1) * (LMAX + 1);
  float2 dY[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) dY[c] = make_float2(0.0f, 0.0f);
  // two partial sums per H1_adj component (even / odd rows) halve the dependent chains
  float2 hA[NL2], hB[NL2];
#pragma unroll
  for (int b = 0; b < NL2; ++b) hA[b] = hB[b] = make_float2(0.0f, 0.0f);
  float2 dr = make_float2(0.0f, 0.0f);
  static_for<half_count(H)>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    constexpr int q = half_ins(H, i);
    constexpr int l1 = ins_l1(LMAX, q), l2 = ins_l2(LMAX, q), g0 = half_goff<LMAX, H>(i);
    constexpr int nb = 2 * l2 + 1;
    float2 dRq = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int a = 0; a < 2 * l1 + 1; ++a) {
      const float2 y = Y2[l1 * l1 + a];
      float2 gs = mul2(g[g0 + a * nb], hv[l2 * l2]);
#pragma unroll
      for (int b = 1; b < nb; ++b) gs = fma2(g[g0 + a * nb + b], hv[l2 * l2 + b], gs);
      dRq = fma2(gs, y, dRq);
      dY[l1 * l1 + a] = fma2(R[i], gs, dY[l1 * l1 + a]);
      const float2 ry = mul2(R[i], y);
      float2* hs = ((i + a) & 1) ? hB : hA;
#pragma unroll
      for (int b = 0; b < nb; ++b) hs[l2 * l2 + b] = fma2(ry, g[g0 + a * nb + b], hs[l2 * l2 + b]);
    }
    dr = fma2(dRq, Rd[i], dr);
  });
#pragma unroll
  for (int b = 0; b < NL2; ++b) hadj[b] = __fadd2_rn(hA[b], hB[b]);
  const float d = dr.x + dr.y;
  float ax = d * u.x, ay = d * u.y, az = d * u.z;
  static_for<16>([&](auto cc) {
    constexpr int c = decltype(cc)::value;
    if constexpr (half_uses_y<LMAX, H>(c)) {
      const float s = dY[c].x + dY[c].y;
      const float4 gc = G[c];
      ax = fmaf(s, gc.x, ax);
      ay = fmaf(s, gc.y, ay);
      az = fmaf(s, gc.z, az);
    }
  });
  fx = ax;
  fy = ay;
  fz = az;
}

// Barrier of the two warps (one per half) that own the same channel pairs: id 1 + p for
// pair p, 64 threads; the block's barrier 0 is __syncthreads.
__device__ __forceinline__ void pair_barrier(int pair) {
  asm volatile("bar.sync %0, 64;" ::"r"(1 + pair) : "memory");
}

// Adjoint, one staged chunk, half H.  The spline row of an edge is reduced to R and
// R' first; the gathers of the next edge are then issued into the freed registers so
// that their L2 latency overlaps this edge's arithmetic.
//
// Both halves produce terms for all NL2 H1_adj rows of the same channel pair.  Half H
// adds rows [H NL2/2, (H + 1) NL2/2) of both halves to the fixed-point accumulator and
// hands the other rows to its partner warp through xchg ([2][NL2][C/2] float2,
// double-buffered by edge parity, so one pair barrier per edge suffices): half the
// atomics of each half adding every row.
template <int LMAX, int H>
__device__ __forceinline__ void l1_rev_chunk(const DevModel& m, const float* __restrict__ H1,
                                             fix64* __restrict__ H1_adj, const L1Stage<true>& st, const Lane2& L,
                                             const float2* g, float* sFT, float2* xchg, int pair) {
  constexpr int NL2 = (LMAX + 1) * (LMAX + 1);
  constexpr int NQ = half_count(H);
  const int na = st.nact;
  float4 c[2 * NQ];
  float2 h[NL2];
  if (na > 0) fetch_l1<LMAX, H, NL2>(m, H1, st.row[st.act[0]], st.j[st.act[0]], L, c, h);
  for (int a = 0; a < na; ++a) {
    const int t = st.act[a];
    const float2 x2 = make_float2(st.x[t], st.x[t]);
    float2 R[NQ], Rd[NQ], hv[NL2];
#pragma unroll
    for (int i = 0; i < NQ; ++i) spline2(c[2 * i], c[2 * i + 1], x2, R[i], Rd[i]);
#pragma unroll
    for (int b = 0; b < NL2; ++b) hv[b] = h[b];
    const int j = st.j[t];
    if (a + 1 < na) {
      const int tn = st.act[a + 1];
      fetch_l1<LMAX, H, NL2>(m, H1, st.row[tn], st.j[tn], L, c, h);
    }
    float2 hadj[NL2];
    float fx, fy, fz;
    l1_rev_edge<LMAX, H>(g, R, Rd, st.Y2[t], st.G[t], st.u[t], hv, hadj, fx, fy, fz);
    if (!L.live) fx = fy = fz = 0.0f;
    // this thread's share of the edge force, summed over the block after the chunk
    sFT[(3 * t) * blockDim.x + threadIdx.x] = fx;
    sFT[(3 * t + 1) * blockDim.x + threadIdx.x] = fy;
    sFT[(3 * t + 2) * blockDim.x + threadIdx.x] = fz;
    constexpr int NR = NL2 / 2;
    float2* xb = xchg + (a & 1) * NL2 * L.C2;
    if (L.live) {
#pragma unroll
      for (int b = 0; b < NL2; ++b)
        if (b / NR != H) xb[b * L.C2 + L.cp] = hadj[b];
    }
    pair_barrier(pair);
    if (L.live) {
      fix64* dst = H1_adj + static_cast<size_t>(j) * NL2 * L.C + L.kc;
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        const int b = H * NR + q;
        const float2 o = xb[b * L.C2 + L.cp];
        add_fixed(dst + b * L.C, hadj[b].x + o.x);
        add_fixed(dst + b * L.C + 1, hadj[b].y + o.y);
      }
    }
  }
}

__device__ __forceinline__ Lane2 lane2(const int C, int& half) {
  Lane2 L;
  L.C = C;
  L.C2 = C >> 1;
  const int HW = (L.C2 + 31) & ~31;
  half = threadIdx.x >= HW ? 1 : 0;
  const int cp = threadIdx.x - half * HW;
  L.live = cp < L.C2;
  L.cp = L.live ? cp : 0;
  L.kc = 2 * L.cp;
  return L;
}

}  // namespace

// ---------------------------------------------------------------------------
// Layer 1 forward: Phi1r[i,p,k] = sum_j R1_q(r_ij)[k] Y_{l1 m1}(x_ij) H1[j, l2 m2, k]
// accumulated in registers, then Phi1[i,lme,k] = sum_p CG[lme,p] Phi1r[i,p,k].
//
// One thread per channel with scalar FMAs over all instructions, on the per-channel
// spline table spl1_fwd ([npairs][nint][n_instr][C] float4).  The forward pass moves
// the same 20 KB spline row per edge as the adjoint but does a third of its
// arithmetic, so it is bound by the L2 gathers: it is laid out for residency (128
// registers, four blocks of 128 threads per SM) rather than for the packed FMAs.
// ---------------------------------------------------------------------------
template <int LMAX, int CT>
__device__ __forceinline__ void layer1_fwd_atom(const DevModel& m, const EdgeIn& in, const float* __restrict__ H1,
                                                float* __restrict__ Phi1, int i) {
  constexpr int NL2 = (LMAX + 1) * (LMAX + 1);
  constexpr int NI = ins_count(LMAX);
  constexpr int NP = ins_np(LMAX);
  extern __shared__ float dyn[];
  __shared__ L1Stage<false> st;
  const int C = CT > 0 ? CT : m.C;
  const int k = threadIdx.x;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.end(i);
  float acc[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) acc[p] = 0.0f;
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_l1<false>(m, in, ti, eb, ne, st);
    __syncthreads();
    const int na = st.nact;
    for (int a = 0; a < na; ++a) {
      const int t = st.act[a];
      const float x = st.x[t];
      float hv[NL2];
      const float* hj = H1 + static_cast<size_t>(st.j[t]) * NL2 * C + k;
#pragma unroll
      for (int b = 0; b < NL2; ++b) hv[b] = __ldg(hj + b * C);
      const float4* cp = m.spl1_fwd + static_cast<size_t>(st.row[t]) * NI * C + k;
      const float2* Y2 = st.Y2[t];
      for_each_ins<LMAX>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        constexpr int l1 = ins_l1(LMAX, q), l2 = ins_l2(LMAX, q), p0 = ins_poff(LMAX, q);
        const float R = spline_val(__ldg(cp + q * C), x);
#pragma unroll
        for (int a1 = 0; a1 < 2 * l1 + 1; ++a1) {
          const float ry = R * Y2[l1 * l1 + a1].x;
#pragma unroll
          for (int b = 0; b < 2 * l2 + 1; ++b)
            acc[p0 + a1 * (2 * l2 + 1) + b] = fmaf(ry, hv[l2 * l2 + b], acc[p0 + a1 * (2 * l2 + 1) + b]);
        }
      });
    }
  }
  if (m.dens_spl[1]) {  // layer-1 density factor for node_tail (mace.cpp:681-705)
    const float S = dens_factor(m, 1, in, i, ti);
    if (threadIdx.x == 0) m.dens_s[1][i] = S;
  }
  float* sP = dyn;  // [NP][C]: this thread's Phi1r column
#pragma unroll
  for (int p = 0; p < NP; ++p) sP[p * C + k] = acc[p];
  // Phi1 rows are [l][m][e] (lme = lme_off[l] + m n_e + e); each thread reads back only its
  // own column of sP
  dispatch_kf(m.cg_fwd_kp, [&](auto kc) {
    l1_fwd_epilogue<decltype(kc)::value>(m, in.N, i, sP, C, k, k, 0, 1, Phi1);
  });
}

template <int LMAX, int CT, bool P>
__global__ void __launch_bounds__(256) k_layer1_fwd(DevModel m, EdgeIn in, const float* __restrict__ H1,
                                                    float* __restrict__ Phi1) {
  pdl_begin();
  AtomCursor cur{P ? m.sched : nullptr, in.N, 0};
  for (int b = cur.first(); b < in.N; b = cur.next())
    layer1_fwd_atom<LMAX, CT>(m, in, H1, Phi1, in.atom_at(b));
  cur.done();
}

// ---------------------------------------------------------------------------
// Layer 1 adjoint.  g (this thread's half of the CG-contracted dPhi1 paths, channel
// pair) stays in registers across the node's edges; f1[e] receives dE/dx_ij.
// ---------------------------------------------------------------------------
template <int LMAX, int CT>
__device__ __forceinline__ void layer1_rev_atom(const DevModel& m, const EdgeIn& in, const float* __restrict__ H1,
                                                const float* __restrict__ dPhi1, fix64* __restrict__ H1_adj,
                                                double* __restrict__ f1, int i) {
  static_assert(LMAX == 1, "instruction halves are tabulated for L_max = 1");
  constexpr int NP = ins_np(LMAX);
  constexpr int NL2 = (LMAX + 1) * (LMAX + 1);
  constexpr int NG = half_np<LMAX, 0>() > half_np<LMAX, 1>() ? half_np<LMAX, 0>() : half_np<LMAX, 1>();
  extern __shared__ float dyn[];
  __shared__ L1Stage<true> st;
  __shared__ float sF[kEdgeChunk][8][3];
  __shared__ float2 xchg[2 * NL2 * 128];  // the halves' H1_adj hand-over, up to 256 channels
  const int C = CT > 0 ? CT : m.C;
  int half;
  const Lane2 L = lane2(C, half);
  const int pair = (threadIdx.x >> 5) % (blockDim.x >> 6);  // warp w of half 0 with warp w of half 1
  const int nwarp = blockDim.x >> 5;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.end(i);
  // g_p = sum_lme CG[lme,p] dPhi1[i,lme,k]: the node's dPhi1 rows staged in shared
  // memory, then (padded table) each thread gathers its channel pair's g from them, or
  // (compressed rows) sP[p][k] is formed first, one channel per thread
  float* sD = dyn;                // [n_lme][C]
  float* sP = dyn + m.n_lme * C;  // [NP][C]
  for (int k = threadIdx.x; k < C; k += blockDim.x) {
    for (int lme = 0; lme < m.n_lme; ++lme) sD[lme * C + k] = dPhi1[(static_cast<size_t>(i) * m.n_lme + lme) * C + k];
    if (!m.cg_rev_pad) {  // any number of terms: sP through a chain of dependent loads per path
      for (int p = 0; p < NP; ++p) {
        float s = 0.0f;
        const int q1 = __ldg(m.cg_rev_off + p + 1);
        for (int q = __ldg(m.cg_rev_off + p); q < q1; ++q)
          s = fmaf(__ldg(m.cg_rev_v + q), sD[__ldg(m.cg_rev_lme + q) * C + k], s);
        sP[p * C + k] = s;
      }
    }
  }
  __syncthreads();
  float2 g[NG];
  // during the edge loop the staged dPhi1 rows (and sP) are dead: the dynamic shared memory
  // holds every thread's share of the chunk's edge forces, [kEdgeChunk][3][blockDim] floats
  // (the chunk loop's first barrier follows every read of sD and sP)
  float* sFT = dyn;
  if (m.cg_rev_pad) {
    if (half == 0)
      l1_load_g_sd<LMAX, 0>(m, sD, L, g);
    else
      l1_load_g_sd<LMAX, 1>(m, sD, L, g);
  } else if (half == 0) {
    l1_load_g<LMAX, 0>(sP, L, g);
  } else {
    l1_load_g<LMAX, 1>(sP, L, g);
  }
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_l1<true>(m, in, ti, eb, ne, st);
    __syncthreads();
    if (half == 0)
      l1_rev_chunk<LMAX, 0>(m, H1, H1_adj, st, L, g, sFT, xchg, pair);
    else
      l1_rev_chunk<LMAX, 1>(m, H1, H1_adj, st, L, g, sFT, xchg, pair);
    __syncthreads();
    {  // each warp sums its 32 lanes' shares of every (edge, component): four partial sums of
       // eight in a fixed order, the reads rotated by lane so the warp hits 32 banks
      const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      for (int q = lane; q < 3 * ne; q += 32) {
        const float* row = sFT + q * blockDim.x + w * 32;
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
#pragma unroll
        for (int i = 0; i < 32; i += 4) {
          a0 += row[(i + lane) & 31];
          a1 += row[(i + 1 + lane) & 31];
          a2 += row[(i + 2 + lane) & 31];
          a3 += row[(i + 3 + lane) & 31];
        }
        sF[q / 3][w][q % 3] = (a0 + a1) + (a2 + a3);
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < ne; t += blockDim.x) {
      double s[3] = {0.0, 0.0, 0.0};
      const long e = static_cast<long>(eb) + t;
      if (st.row[t] >= 0)
        for (int w = 0; w < nwarp; ++w)
          for (int c = 0; c < 3; ++c) s[c] += static_cast<double>(sF[t][w][c]);
      if (m.dens_spl[1]) {  // dE/dx through the layer-1 density factor (mace.cpp:744-749)
        float v, d;
        const double r = in.r[e];
        dens_eval(m, 1, ti, in.ntype_e[e], static_cast<float>(r), v, d);
        const double g = static_cast<double>(m.dens_c[1][i]) * static_cast<double>(d) / r;
        for (int c = 0; c < 3; ++c) s[c] -= g * in.xyz[3 * e + c];
      }
      for (int c = 0; c < 3; ++c) f1[3 * e + c] = s[c];
    }
  }
}

template <int LMAX, int CT, bool P>
__global__ void __launch_bounds__(256) k_layer1_rev(DevModel m, EdgeIn in, const float* __restrict__ H1,
                                                    const float* __restrict__ dPhi1, fix64* __restrict__ H1_adj,
                                                    double* __restrict__ f1) {
  pdl_begin();
  AtomCursor cur{P ? m.sched : nullptr, in.N, 0};
  for (int b = cur.first(); b < in.N; b = cur.next())
    layer1_rev_atom<LMAX, CT>(m, in, H1, dPhi1, H1_adj, f1, in.atom_at(b));
  cur.done();
}

// ===========================================================================
// L_max = 2 (hidden irreps up to 2e: 17 instructions, 243 CG paths).  The paths do not
// fit one thread's registers, so the instructions are split over four thread groups
// per channel ({11,13,15,16}, {1,4,5,8,12}, {0,2,6,10}, {3,7,9,14}: exhaustive local
// search for equal scalar work, 202/201/196/202 FMAs per edge, and 62/57/62/62 paths);
// one channel per thread, scalar FMAs.  Block = 4 groups x C threads.
// ===========================================================================
namespace {

constexpr int kL2Groups = 4;
// channels per block of the L_max = 2 layer-1 kernels (a warp multiple)
__host__ __device__ inline int l2_slice_width(const DevModel& m) {
  return ((m.C + m.l2_split - 1) / m.l2_split + 31) & ~31;
}
__host__ __device__ constexpr int l2_count(int g) { return g == 1 ? 5 : 4; }
__host__ __device__ constexpr int l2_ins(int g, int i) {
  constexpr int t0[4] = {11, 13, 15, 16}, t1[5] = {1, 4, 5, 8, 12}, t2[4] = {0, 2, 6, 10}, t3[4] = {3, 7, 9, 14};
  return g == 0 ? t0[i] : (g == 1 ? t1[i] : (g == 2 ? t2[i] : t3[i]));
}
template <int G>
__host__ __device__ constexpr int l2_goff(int i) {
  int s = 0;
  for (int w = 0; w < i; ++w) s += ins_paths(2, l2_ins(G, w));
  return s;
}
template <int G>
__host__ __device__ constexpr int l2_np() {
  return l2_goff<G>(l2_count(G));
}
template <int G>
__host__ __device__ constexpr bool l2_uses_y(int c) {
  for (int w = 0; w < l2_count(G); ++w) {
    const int l1 = ins_l1(2, l2_ins(G, w));
    if (c >= l1 * l1 && c < (l1 + 1) * (l1 + 1)) return true;
  }
  return false;
}
constexpr int kL2MaxNp = 62;

// block-wide sum of a 3-vector per edge for up to 16 warps
__device__ __forceinline__ void block_reduce3_w16(float fx, float fy, float fz, float (*sF)[16][3], int t) {
  const float x = warp_sum(fx), y = warp_sum(fy), z = warp_sum(fz);
  if ((threadIdx.x & 31) == 0) {
    const int w = threadIdx.x >> 5;
    sF[t][w][0] = x;
    sF[t][w][1] = y;
    sF[t][w][2] = z;
  }
}

// Forward, group G, one staged chunk: acc[local path] += R_q Y_{l1 m1} H1[j, l2 m2, k].
template <int G>
__device__ __forceinline__ void l2_fwd_chunk(const DevModel& m, const float* __restrict__ H1,
                                             const L1Stage<false>& st, int C, int k, float* acc) {
  constexpr int NL2 = 9, NI = 17;
  const int na = st.nact;
  for (int a = 0; a < na; ++a) {
    const int t = st.act[a];
    const float x = st.x[t];
    float hv[NL2];
    const float* hj = H1 + static_cast<size_t>(st.j[t]) * NL2 * C + k;
#pragma unroll
    for (int b = 0; b < NL2; ++b) hv[b] = __ldg(hj + b * C);
    const float4* cp = m.spl1_fwd + static_cast<size_t>(st.row[t]) * NI * C + k;
    static_for<l2_count(G)>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
      constexpr int q = l2_ins(G, i);
      constexpr int l1 = ins_l1(2, q), l2 = ins_l2(2, q), g0 = l2_goff<G>(i);
      const float R = spline_val(__ldg(cp + q * C), x);
#pragma unroll
      for (int a1 = 0; a1 < 2 * l1 + 1; ++a1) {
        const float ry = R * st.Y2[t][l1 * l1 + a1].x;
#pragma unroll
        for (int b = 0; b < 2 * l2 + 1; ++b)
          acc[g0 + a1 * (2 * l2 + 1) + b] = fmaf(ry, hv[l2 * l2 + b], acc[g0 + a1 * (2 * l2 + 1) + b]);
      }
    });
  }
}

template <int G>
__device__ __forceinline__ void l2_store(float* sP, int C, int k, const float* acc) {
  static_for<l2_count(G)>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    constexpr int q = l2_ins(G, i);
    constexpr int np = ins_paths(2, q), p0 = ins_poff(2, q), g0 = l2_goff<G>(i);
#pragma unroll
    for (int p = 0; p < np; ++p) sP[(p0 + p) * C + k] = acc[g0 + p];
  });
}

template <int G>
__device__ __forceinline__ void l2_load_g(const float* sP, int C, int k, float* g) {
  static_for<l2_count(G)>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    constexpr int q = l2_ins(G, i);
    constexpr int np = ins_paths(2, q), p0 = ins_poff(2, q), g0 = l2_goff<G>(i);
#pragma unroll
    for (int p = 0; p < np; ++p) g[g0 + p] = sP[(p0 + p) * C + k];
  });
}

// g of group G for channel kk straight from the staged dPhi1 rows sD ([n_lme][stride])
// through the two-term padded CG table
template <int G>
__device__ __forceinline__ void l2_load_g_sd(const DevModel& m, const float* sD, int stride, int kk, float* g) {
  static_for<l2_count(G)>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    constexpr int q = l2_ins(G, i);
    constexpr int np = ins_paths(2, q), p0 = ins_poff(2, q), g0 = l2_goff<G>(i);
#pragma unroll
    for (int p = 0; p < np; ++p) {
      const int2 t0 = __ldg(m.cg_rev_pad + 2 * (p0 + p)), t1 = __ldg(m.cg_rev_pad + 2 * (p0 + p) + 1);
      g[g0 + p] = fmaf(__int_as_float(t1.y), sD[t1.x * stride + kk], __int_as_float(t0.y) * sD[t0.x * stride + kk]);
    }
  });
}

}  // namespace

// Layer-1 forward, L_max = 2: slice h of the channels of node i (channels h*CH ..
// h*CH + CH - 1, CH = l2_slice_width(m)); four groups of CH threads, group G running the
// instructions of group G.
__device__ __forceinline__ void layer1_fwd_l2_atom(const DevModel& m, const EdgeIn& in, const float* __restrict__ H1,
                                                   float* __restrict__ Phi1, int i, int h) {
  extern __shared__ float dyn[];
  __shared__ L1Stage<false> st;
  const int C = m.C, CH = l2_slice_width(m);
  const int grp = threadIdx.x / CH, kk = threadIdx.x - grp * CH;
  const bool live = kk < CH && h * CH + kk < C;
  const int k = live ? h * CH + kk : 0;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.end(i);
  float acc[kL2MaxNp];
#pragma unroll
  for (int p = 0; p < kL2MaxNp; ++p) acc[p] = 0.0f;
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_l1<false>(m, in, ti, eb, ne, st);
    __syncthreads();
    switch (grp) {
      case 0: l2_fwd_chunk<0>(m, H1, st, C, k, acc); break;
      case 1: l2_fwd_chunk<1>(m, H1, st, C, k, acc); break;
      case 2: l2_fwd_chunk<2>(m, H1, st, C, k, acc); break;
      default: l2_fwd_chunk<3>(m, H1, st, C, k, acc); break;
    }
  }
  if (m.dens_spl[1]) {
    const float S = dens_factor(m, 1, in, i, ti);
    if (threadIdx.x == 0 && h == 0) m.dens_s[1][i] = S;
  }
  float* sP = dyn;  // [NP][CH]: Phi1r of the slice
  if (live) {
    switch (grp) {
      case 0: l2_store<0>(sP, CH, kk, acc); break;
      case 1: l2_store<1>(sP, CH, kk, acc); break;
      case 2: l2_store<2>(sP, CH, kk, acc); break;
      default: l2_store<3>(sP, CH, kk, acc); break;
    }
  }
  __syncthreads();
  // Phi1 rows of the slice, group G taking the rows lme = G (mod 4)
  if (!live) return;
  dispatch_kf(m.cg_fwd_kp, [&](auto kc) {
    l1_fwd_epilogue<decltype(kc)::value>(m, in.N, i, sP, CH, kk, k, grp, kL2Groups, Phi1);
  });
}

// work item b = (atom, channel slice); the return in the atom body above happens after
// its last barrier
template <bool P>
__global__ void __launch_bounds__(512, 1) k_layer1_fwd_l2(DevModel m, EdgeIn in, const float* __restrict__ H1,
                                                          float* __restrict__ Phi1) {
  pdl_begin();
  const int ns = m.l2_split, n = in.N * ns;
  AtomCursor cur{P ? m.sched : nullptr, n, 0};
  for (int b = cur.first(); b < n; b = cur.next()) layer1_fwd_l2_atom(m, in, H1, Phi1, in.atom_at(b / ns), b % ns);
  cur.done();
}

namespace {

template <int G>
__host__ __device__ constexpr bool l2_uses_l2(int l2) {
  for (int w = 0; w < l2_count(G); ++w)
    if (ins_l2(2, l2_ins(G, w)) == l2) return true;
  return false;
}

// Adjoint, group G, edges [a0, a1) of a staged chunk (as l1_rev_edge, scalar, this
// group's paths).  The H1_adj terms of the four groups meet in hold ([kSub2][4 groups]
// [NL2][CH] floats, zero for the rows a group does not touch), and after a block barrier
// l2_rev_flush adds each row once per channel (as in the L_max = 1 adjoint); each thread's
// share of the edge force goes to the [kSub2][3][blockDim] floats after hold, summed by
// l2_rev_flush too.
constexpr int kSub2 = 7;
template <int G>
__device__ __forceinline__ void l2_rev_chunk(const DevModel& m, const float* __restrict__ H1, const L1Stage<true>& st,
                                             int C, int k, bool live, const float* g, float* hold, int CH, int kk,
                                             int a0, int a1) {
  constexpr int NL2 = 9, NI = 17;
  for (int a = a0; a < a1; ++a) {
    const int t = st.act[a];
    const float x = st.x[t];
    const int j = st.j[t];
    float hv[NL2];
    const float* hj = H1 + static_cast<size_t>(j) * NL2 * C + k;
#pragma unroll
    for (int b = 0; b < NL2; ++b) hv[b] = __ldg(hj + b * C);
    const float4* cp = m.spl1_fwd + static_cast<size_t>(st.row[t]) * NI * C + k;
    float dY[16], hadj[NL2], dr = 0.0f;
#pragma unroll
    for (int c = 0; c < 16; ++c) dY[c] = 0.0f;
#pragma unroll
    for (int b = 0; b < NL2; ++b) hadj[b] = 0.0f;
    static_for<l2_count(G)>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
      constexpr int q = l2_ins(G, i);
      constexpr int l1 = ins_l1(2, q), l2 = ins_l2(2, q), g0 = l2_goff<G>(i), nb = 2 * l2 + 1;
      const float4 cc = __ldg(cp + q * C);
      const float R = spline_val(cc, x), Rd = spline_der(cc, x);
      float dRq = 0.0f;
#pragma unroll
      for (int a1 = 0; a1 < 2 * l1 + 1; ++a1) {
        const float y = st.Y2[t][l1 * l1 + a1].x;
        float gs = 0.0f;
#pragma unroll
        for (int b = 0; b < nb; ++b) gs = fmaf(g[g0 + a1 * nb + b], hv[l2 * l2 + b], gs);
        dRq = fmaf(gs, y, dRq);
        dY[l1 * l1 + a1] = fmaf(R, gs, dY[l1 * l1 + a1]);
        const float ry = R * y;
#pragma unroll
        for (int b = 0; b < nb; ++b) hadj[l2 * l2 + b] = fmaf(ry, g[g0 + a1 * nb + b], hadj[l2 * l2 + b]);
      }
      dr = fmaf(dRq, Rd, dr);
    });
    const float4 u = st.u[t];
    float fx = dr * u.x, fy = dr * u.y, fz = dr * u.z;
    static_for<16>([&](auto cc) {
      constexpr int c = decltype(cc)::value;
      if constexpr (l2_uses_y<G>(c)) {
        const float4 gc = st.G[t][c];
        fx = fmaf(dY[c], gc.x, fx);
        fy = fmaf(dY[c], gc.y, fy);
        fz = fmaf(dY[c], gc.z, fz);
      }
    });
    if (!live) fx = fy = fz = 0.0f;
    float* fs = hold + kSub2 * kL2Groups * NL2 * CH + (3 * (a - a0)) * blockDim.x + threadIdx.x;
    fs[0] = fx;
    fs[blockDim.x] = fy;
    fs[2 * blockDim.x] = fz;
    if (live) {
      float* hb = hold + ((a - a0) * kL2Groups + G) * NL2 * CH + kk;
#pragma unroll
      for (int b = 0; b < NL2; ++b) hb[b * CH] = hadj[b];
    }
  }
}

// After the barrier that follows l2_rev_chunk: the rows b = grp (mod 4) of edges [a0, a1),
// the four groups' terms summed in group order, to the fixed-point accumulator.
__device__ __forceinline__ void l2_rev_flush(fix64* __restrict__ H1_adj, const L1Stage<true>& st, int C, int k,
                                             bool live, const float* hold, int CH, int kk, int grp, int a0, int a1) {
  constexpr int NL2 = 9;
  if (!live) return;
  for (int a = a0; a < a1; ++a) {
    const float* hb = hold + (a - a0) * kL2Groups * NL2 * CH + kk;
    fix64* dst = H1_adj + static_cast<size_t>(st.j[st.act[a]]) * NL2 * C + k;
    for (int b = grp; b < NL2; b += kL2Groups) {
      float v = hb[b * CH];
#pragma unroll
      for (int q = 1; q < kL2Groups; ++q) v += hb[(q * NL2 + b) * CH];
      add_fixed(dst + b * C, v);
    }
  }
}

// After the same barrier: each warp sums its 32 lanes' shares of the force of edges
// [a0, a1) (fs: [kSub2][3][blockDim] floats; four partial sums in a fixed order, the reads
// rotated by lane so that the warp hits 32 banks) into sF[staged slot][warp].
__device__ __forceinline__ void l2_rev_force_sums(const L1Stage<true>& st, const float* fs, float (*sF)[16][3], int a0,
                                                  int a1) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int q = lane; q < 3 * (a1 - a0); q += 32) {
    const float* row = fs + q * blockDim.x + w * 32;
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
#pragma unroll
    for (int i = 0; i < 32; i += 4) {
      s0 += row[(i + lane) & 31];
      s1 += row[(i + 1 + lane) & 31];
      s2 += row[(i + 2 + lane) & 31];
      s3 += row[(i + 3 + lane) & 31];
    }
    sF[st.act[a0 + q / 3]][w][q % 3] = (s0 + s1) + (s2 + s3);
  }
}

}  // namespace

// Layer-1 adjoint, L_max = 2, channel slice h of node i (as the forward).  Each slice
// writes its partial per-edge forces to its own f1 slice (f1 + h * f1_stride); the
// layer-0 adjoint adds the slices.
__device__ __forceinline__ void layer1_rev_l2_atom(const DevModel& m, const EdgeIn& in, const float* __restrict__ H1,
                                                   const float* __restrict__ dPhi1, fix64* __restrict__ H1_adj,
                                                   double* __restrict__ f1, int i, int h) {
  constexpr int NP = 243;
  extern __shared__ float dyn[];
  __shared__ L1Stage<true> st;
  __shared__ float sF[kEdgeChunk][16][3];  // up to 16 warps (512 threads)
  const int C = m.C, CH = l2_slice_width(m);
  const int grp = threadIdx.x / CH, kk = threadIdx.x - grp * CH;
  const bool live = kk < CH && h * CH + kk < C;
  const int k = live ? h * CH + kk : 0;
  const int nwarp = blockDim.x >> 5;
  const int ti = in.node_type[i];
  const int e0 = in.first[i], e1 = in.end(i);
  float* sD = dyn;                  // [n_lme][CH]
  float* sP = dyn + m.n_lme * CH;   // [NP][CH]
  // g_p = sum_lme CG[lme,p] dPhi1[i,lme,k] from the node's staged dPhi1 rows (staging
  // split over the four groups)
  if (live)
    for (int lme = grp; lme < m.n_lme; lme += kL2Groups)
      sD[lme * CH + kk] = dPhi1[(static_cast<size_t>(i) * m.n_lme + lme) * C + k];
  __syncthreads();
  float g[kL2MaxNp];
  if (m.cg_rev_pad) {  // each thread gathers its group's g from the staged rows
    switch (grp) {
      case 0: l2_load_g_sd<0>(m, sD, CH, kk, g); break;
      case 1: l2_load_g_sd<1>(m, sD, CH, kk, g); break;
      case 2: l2_load_g_sd<2>(m, sD, CH, kk, g); break;
      default: l2_load_g_sd<3>(m, sD, CH, kk, g); break;
    }
  } else {  // sP first, rows split over the four groups, through the compressed rows
    if (live)
      for (int p = grp; p < NP; p += kL2Groups) {
        float sum = 0.0f;
        const int q1 = __ldg(m.cg_rev_off + p + 1);
        for (int q = __ldg(m.cg_rev_off + p); q < q1; ++q)
          sum = fmaf(__ldg(m.cg_rev_v + q), sD[__ldg(m.cg_rev_lme + q) * CH + kk], sum);
        sP[p * CH + kk] = sum;
      }
    __syncthreads();
    switch (grp) {
      case 0: l2_load_g<0>(sP, CH, kk, g); break;
      case 1: l2_load_g<1>(sP, CH, kk, g); break;
      case 2: l2_load_g<2>(sP, CH, kk, g); break;
      default: l2_load_g<3>(sP, CH, kk, g); break;
    }
  }
  double* f1h = f1 + h * m.f1_stride;
  for (int eb = e0; eb < e1; eb += kEdgeChunk) {
    const int ne = min(kEdgeChunk, e1 - eb);
    __syncthreads();
    stage_l1<true>(m, in, ti, eb, ne, st);
    __syncthreads();
    // the staged dPhi1 rows and sP are dead now: the H1_adj terms and the force shares of
    // kSub2 edges at a time
    float* hold = dyn;
    for (int a0 = 0; a0 < st.nact; a0 += kSub2) {
      const int a1 = min(st.nact, a0 + kSub2);
      switch (grp) {
        case 0: l2_rev_chunk<0>(m, H1, st, C, k, live, g, hold, CH, kk, a0, a1); break;
        case 1: l2_rev_chunk<1>(m, H1, st, C, k, live, g, hold, CH, kk, a0, a1); break;
        case 2: l2_rev_chunk<2>(m, H1, st, C, k, live, g, hold, CH, kk, a0, a1); break;
        default: l2_rev_chunk<3>(m, H1, st, C, k, live, g, hold, CH, kk, a0, a1); break;
      }
      __syncthreads();
      l2_rev_flush(H1_adj, st, C, k, live, hold, CH, kk, grp, a0, a1);
      l2_rev_force_sums(st, hold + kSub2 * kL2Groups * 9 * CH, sF, a0, a1);
      __syncthreads();
    }
    for (int t = threadIdx.x; t < ne; t += blockDim.x) {
      double sum[3] = {0.0, 0.0, 0.0};
      const long e = static_cast<long>(eb) + t;
      if (st.row[t] >= 0)
        for (int w = 0; w < nwarp; ++w)
          for (int c = 0; c < 3; ++c) sum[c] += static_cast<double>(sF[t][w][c]);
      if (m.dens_spl[1] && h == 0) {
        float v, d;
        const double r = in.r[e];
        dens_eval(m, 1, ti, in.ntype_e[e], static_cast<float>(r), v, d);
        const double gg = static_cast<double>(m.dens_c[1][i]) * static_cast<double>(d) / r;
        for (int c = 0; c < 3; ++c) sum[c] -= gg * in.xyz[3 * e + c];
      }
      for (int c = 0; c < 3; ++c) f1h[3 * e + c] = sum[c];
    }
  }
}

template <bool P>
__global__ void __launch_bounds__(512, 1) k_layer1_rev_l2(DevModel m, EdgeIn in, const float* __restrict__ H1,
                                                          const float* __restrict__ dPhi1,
                                                          fix64* __restrict__ H1_adj, double* __restrict__ f1) {
  pdl_begin();
  const int ns = m.l2_split, n = in.N * ns;
  AtomCursor cur{P ? m.sched : nullptr, n, 0};
  for (int b = cur.first(); b < n; b = cur.next())
    layer1_rev_l2_atom(m, in, H1, dPhi1, H1_adj, f1, in.atom_at(b / ns), b % ns);
  cur.done();
}

// threads per block of the layer-1 kernels: two warp-aligned groups of C/2
int layer1_block(int C) { return 2 * (((C >> 1) + 31) & ~31); }

namespace {

// dynamic shared memory of the L_max = 2 adjoint: the staged dPhi1 rows and the g table,
// and later the H1_adj terms of kSub2 edges (see l2_rev_chunk)
size_t rev_l2_smem(const DevModel& m) {  // (the block is kL2Groups * CH threads)
  return sizeof(float) * std::max<size_t>(m.n_lme + ins_np(2), kSub2 * kL2Groups * (9 + 3)) * l2_slice_width(m);
}

// dynamic shared memory of the L_max = 1 adjoint: the staged dPhi1 rows and the g table
size_t rev_l1_smem(const DevModel& m) {
  return sizeof(float) * std::max<size_t>((m.n_lme + ins_np(1)) * m.C, kEdgeChunk * 3 * layer1_block(m.C));
}

template <int CT, bool P>
cudaError_t set_smem(const DevModel& m) {
  cudaError_t e = cudaFuncSetAttribute(k_layer1_fwd<1, CT, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sizeof(float) * ins_np(1) * m.C));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_layer1_rev<1, CT, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(rev_l1_smem(m)));
}

template <bool P>
cudaError_t set_smem_l2(const DevModel& m) {
  cudaError_t e = cudaFuncSetAttribute(k_layer1_fwd_l2<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(sizeof(float) * ins_np(2) * m.C));
  if (e != cudaSuccess) return e;
  // (sized for one slice of all C channels: the largest rev_l2_smem of any slice count)
  return cudaFuncSetAttribute(k_layer1_rev_l2<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(sizeof(float) * std::max(m.n_lme + ins_np(2), kSub2 * kL2Groups * (9 + 3)) *
                                               m.C));
}

// Channel counts with a compile-time specialisation (addresses fold to immediates).
template <typename F>
void dispatch_c(int C, F&& f) {
  switch (C) {
    case 32: f(std::integral_constant<int, 32>{}); break;
    case 64: f(std::integral_constant<int, 64>{}); break;
    case 128: f(std::integral_constant<int, 128>{}); break;
    case 256: f(std::integral_constant<int, 256>{}); break;
    default: f(std::integral_constant<int, 0>{}); break;
  }
}

// the one-block-per-atom (false) or persistent (true) instantiation
template <typename F>
void dispatch_p(bool persistent, F&& f) {
  if (persistent)
    f(std::true_type{});
  else
    f(std::false_type{});
}

}  // namespace

cudaError_t init_layer1_kernels(const DevModel& m) {
  cudaError_t e = cudaSuccess;
  for (bool p : {false, true}) {
    if (m.L_max == 2)
      dispatch_p(p, [&](auto pc) { e = set_smem_l2<decltype(pc)::value>(m); });
    else
      dispatch_c(m.C, [&](auto ct) {
        dispatch_p(p, [&](auto pc) { e = set_smem<decltype(ct)::value, decltype(pc)::value>(m); });
      });
    if (e != cudaSuccess) return e;
  }
  return e;
}

void launch_layer1_fwd(const DevModel& m, const EdgeIn& in, const float* H1, float* Phi1, cudaStream_t s) {
  if (in.N <= 0) return;
  DevModel mk;
  const int grid = atom_grid(m, kAkLayer1Fwd, m.L_max == 2 ? in.N * m.l2_split : in.N, mk);
  dispatch_p(mk.sched != nullptr, [&](auto pc) {
    constexpr bool P = decltype(pc)::value;
    if (m.L_max == 2) {
      launch_pdl(k_layer1_fwd_l2<P>, grid, kL2Groups * l2_slice_width(m),
                 sizeof(float) * ins_np(2) * l2_slice_width(m), s, mk, in, H1, Phi1);
      return;
    }
    const size_t smem = sizeof(float) * ins_np(1) * m.C;
    dispatch_c(m.C, [&](auto ct) {
      launch_pdl(k_layer1_fwd<1, decltype(ct)::value, P>, grid, m.C, smem, s, mk, in, H1, Phi1);
    });
  });
}

void launch_layer1_rev(const DevModel& m, const EdgeIn& in, const float* H1, const float* dPhi1, fix64* H1_adj,
                       double* f1, cudaStream_t s) {
  if (in.N <= 0) return;
  DevModel mk;
  const int grid = atom_grid(m, kAkLayer1Rev, m.L_max == 2 ? in.N * m.l2_split : in.N, mk);
  dispatch_p(mk.sched != nullptr, [&](auto pc) {
    constexpr bool P = decltype(pc)::value;
    if (m.L_max == 2) {
      launch_pdl(k_layer1_rev_l2<P>, grid, kL2Groups * l2_slice_width(m), rev_l2_smem(m), s, mk, in, H1, dPhi1,
                 H1_adj, f1);
      return;
    }
    const size_t smem = rev_l1_smem(m);
    dispatch_c(m.C, [&](auto ct) {
      launch_pdl(k_layer1_rev<1, decltype(ct)::value, P>, grid, layer1_block(m.C), smem, s, mk, in, H1, dPhi1, H1_adj,
                 f1);
    });
  });
}

// resident blocks per SM of the persistent layer-1 kernels at this model's launch shapes
void layer1_residency(const DevModel& m, int* per_sm) {
  int f = 0, r = 0;
  if (m.L_max == 2) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, k_layer1_fwd_l2<true>, kL2Groups * l2_slice_width(m),
                                                  sizeof(float) * ins_np(2) * l2_slice_width(m));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_layer1_rev_l2<true>, kL2Groups * l2_slice_width(m),
                                                  rev_l2_smem(m));
  } else {
    dispatch_c(m.C, [&](auto ct) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, k_layer1_fwd<1, decltype(ct)::value, true>, m.C,
                                                    sizeof(float) * ins_np(1) * m.C);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_layer1_rev<1, decltype(ct)::value, true>,
                                                    layer1_block(m.C), rev_l1_smem(m));
    });
  }
  per_sm[kAkLayer1Fwd] = f;
  per_sm[kAkLayer1Rev] = r;
}

}  // namespace smx
