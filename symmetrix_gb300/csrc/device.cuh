// Device-side model view and helpers shared by the GB300 kernels.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <type_traits>
#include <utility>

namespace smx {

constexpr int kEdgeChunk = 32;  // edges staged in shared memory per block iteration

// Device view of a packed model (see model.hpp for layouts).  Passed by value.
struct DevModel {
  int S, C, L_max, nLM, n_lme, n_instr, n_p, nint, T0, T1, n_hidden;
  int poly_canon;  // coefficients in canonical order: use the generated polynomials
  float h, inv_h, r_cut, ro2_scale;
  const float4* spl0;  // [S*S][nint][4][2][C/2]: channel-pair planes
  const float4* spl1;      // [npairs][nint][n_instr][2][C/2]: channel-pair planes (adjoint)
  const float4* spl1_fwd;  // [npairs][nint][n_instr][C]: per-channel cubics (forward)
  const int* mono0;
  int mono0_off[10];
  const float* coef0;  // [S][nLM][T0][C]
  const int* mono1;
  const float* coef1;  // [S][T1][C]
  const float* H1W;
  const float* H1W_T;
  const int* cg_fwd_off;
  const int* cg_fwd_p;
  const float* cg_fwd_v;
  // the same table padded to cg_fwd_kp terms per output row (<= 8), (p, float bits of the
  // value), zero terms as (0, 0); nullptr (kp 0) when some row has more terms
  const int2* cg_fwd_pad;
  int cg_fwd_kp;
  const int* cg_rev_off;
  const int* cg_rev_lme;
  const float* cg_rev_v;
  // the same table padded to two terms per path, (lme, float bits of the value), zero
  // terms as (0, 0); nullptr when some path has more terms
  const int2* cg_rev_pad;
  int lme_off[4], num_e[4];
  const float* A1W[4];
  const float* A1W_T[4];
  const float* H2W_H1;
  const float* H2W_H1_T;
  const float* H2W_M1;
  const float* H2W_M1_T;
  const float* ro1;
  const float* ro2_w1;
  const float* ro2_w2;
  const float* e0;
  // ZBL pair repulsion (optional)
  int has_zbl, zbl_p;
  float zbl_c[4];
  const float4* zbl_pair;  // [S*S]: (1/a, 0.5*14.3996*Zu*Zv, r_max, 0)
  // density-normalised blocks: layer 0 / 1 spline tables [npairs][nint][4] (or nullptr)
  const float4* dens_spl[2];
  int dens_nint[2];
  float dens_h[2], dens_inv_h[2];
  // and their per-node workspace (set by the engine with its buffers): the factor
  // s_i = 1 + sum_j s(r_ij) and c_i = (dE/dA_scaled . A_scaled) / s_i
  float* dens_s[2];
  float* dens_c[2];
  // BF16 form: the producers also write the tensor-core GEMM X operands as
  // XT = split_xterms(tc_terms) bf16 split terms per row (see write_split); nullptr in
  // the FP32 form.  Offsets and pitches below are in units of T = XT.
  //   op_m0    [N*nLM][T*C]                rows (node, LM)              (H1 GEMM)
  //   op_phi1  per l: [N(2l+1)][T*n_e*C]   at T*N*lme_off[l]*C          (A1 GEMM)
  //   op_a1adj per l: [N(2l+1)][T*C]       at T*N*l*l*C                 (Phi1_adj GEMM)
  __nv_bfloat16* op_m0;
  __nv_bfloat16* op_phi1;
  __nv_bfloat16* op_a1adj;
  int tc_terms;
  // Centre-atom schedule of the per-atom kernels (AtomCursor): pgrid[k] > 0 runs kernel k
  // as a persistent grid of that many blocks claiming atoms from the counter pair
  // sched[0..1]; 0 launches one block per atom.  pgrid is read on the host only.
  int* sched;
  int pgrid[8];
  // L_max = 2 layer-1 kernels: channel slices per node (one block each) and the offset
  // between the per-slice partial edge forces in f1 (0: one slice)
  int l2_split;
  long f1_stride;
  // the engine's status word (mapped host memory): a bounded wait that gave up sets bit 0
  unsigned* status;
};

// Per-atom kernels, indices into DevModel::pgrid.
enum AtomKernel { kAkLayer0Fwd = 0, kAkContract0Rev, kAkLayer0Rev, kAkLayer1Fwd, kAkLayer1Rev, kAkNodeTail,
                  kAkCount };

// The centre atoms a block of a per-atom kernel works on.  Without a counter (one block
// per atom) the block takes atom blockIdx.x.  With one (a persistent grid sized to the
// resident blocks) blocks claim atoms in order from sched[0]; thread 0 claims the next
// atom while the block works on the current one, so the atomic's latency is hidden.  The
// last block to finish resets the counters for the next launch on the stream, which
// keeps the launch self-contained (graph replays need no memset).
struct AtomCursor {
  int* sched;
  int n;
  int ahead;  // thread 0: the atom claimed for after the current one
  __device__ __forceinline__ int first() {
    if (!sched) return blockIdx.x;
    __shared__ int slot;
    if (threadIdx.x == 0) {
      slot = atomicAdd(sched, 1);
      ahead = atomicAdd(sched, 1);
    }
    __syncthreads();
    return slot;
  }
  // call from uniform control flow after the block is done with the current atom
  __device__ __forceinline__ int next() {
    if (!sched) return n;
    __shared__ int slot;
    __syncthreads();  // every thread has finished the current atom (and read slot)
    if (threadIdx.x == 0) {
      slot = ahead;
      ahead = ahead < n ? atomicAdd(sched, 1) : ahead;
    }
    __syncthreads();
    return slot;
  }
  __device__ __forceinline__ void done() const {
    if (!sched || threadIdx.x != 0) return;
    __threadfence();
    if (atomicAdd(sched + 1, 1) == static_cast<int>(gridDim.x) - 1) {
      sched[0] = 0;
      sched[1] = 0;
    }
  }
};

// H1_adj accumulation in 64-bit fixed point.  The layer-1 adjoint scatters every edge's
// R1 Y g term into H1_adj of the neighbour node; float atomics would make the sum depend
// on the order in which blocks arrive.  Integer addition is associative, so each term is
// rounded once to a multiple of 2^-34 and added as a two's-complement int64: the sum is
// the same bit pattern on every run, and converted to float once at the end.  Range:
// |H1_adj| < 2^29 (5.4e8, far above any model's dE/dH1: O(1)); resolution 2^-34
// (5.8e-11, far below the float32 rounding of a term).
using fix64 = unsigned long long;
// round(v 2^34) as an int64, round-to-nearest-even, for |v| < 2^29, in three exact FP32
// steps and no conversion instruction (whose issue cost is several times these): v is
// split as a 2^10 + b 2^-12 + c 2^-34 with a, b, c integers of at most 22 bits, each
// found by adding 1.5 2^23 (whose ulp is 1) to the scaled remainder and reading the
// integer from the low mantissa bits.  Each remainder is exact (v minus its rounding to
// a multiple of a power of two at or above its ulp), and a 2^44 + b 2^22 is an even
// integer, so a 2^44 + b 2^22 + c is the rounding of v 2^34 itself.
__device__ __forceinline__ fix64 to_fixed(float v) {
  constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
  const float ta = fmaf(v, 1.0f / 1024.0f, kMagic);
  const float va = fmaf(-(ta - kMagic), 1024.0f, v);  // v - a 2^10
  const float tb = fmaf(va, 4096.0f, kMagic);
  const float vb = fmaf(-(tb - kMagic), 1.0f / 4096.0f, va);  // va - b 2^-12
  const float tc = fmaf(vb, 17179869184.0f, kMagic);
  const int a = __float_as_int(ta) - 0x4B400000, b = __float_as_int(tb) - 0x4B400000,
            c = __float_as_int(tc) - 0x4B400000;
  // a 2^44 + b 2^22 + c
  return (static_cast<fix64>(static_cast<long long>(a)) << 44) + (static_cast<fix64>(static_cast<long long>(b)) << 22) +
         static_cast<fix64>(static_cast<long long>(c));
}
__device__ __forceinline__ void add_fixed(fix64* dst, float v) { atomicAdd(dst, to_fixed(v)); }
// q 2^-34 as a float without float64 arithmetic (whose conversions run on this part's
// slow float64 pipe): q = a 2^44 + b 2^22 + c with a signed, b and c in [0, 2^22), all
// exact as floats; t = a 2^10 + b 2^-12 is exact when |q 2^-34| < 2^10 (then |a 2^22 + b|
// < 2^22 + 1), so the last fmaf rounds once: the float nearest q 2^-34, as the float64
// route gives; above 2^10, within one ulp of it.
__device__ __forceinline__ float from_fixed(fix64 q) {
  const long long s = static_cast<long long>(q);
  const float a = static_cast<float>(static_cast<int>(s >> 44));
  const float b = static_cast<float>(static_cast<int>((s >> 22) & 0x3FFFFF));
  const float c = static_cast<float>(static_cast<int>(s & 0x3FFFFF));
  const float t = fmaf(a, 1024.0f, b * (1.0f / 4096.0f));
  return fmaf(c, 1.0f / 17179869184.0f, t);
}

// Programmatic dependent launch.  The chained kernels of an evaluation and of an MD step
// are launched with the programmatic-serialization attribute (launch_pdl); each starts
// with pdl_begin, whose griddepcontrol.wait holds its blocks until the previous grid has
// completed and its writes are visible (a no-op after a normal launch), and reads or
// writes nothing before it.  No kernel signals griddepcontrol.launch_dependents early, so
// a dependent grid is launched as its predecessor's blocks exit: on the 4096-atom MD step
// this saves ~4 us (1.911 -> 1.907 ms), while a signal at every block's start, which
// lets the next grid's blocks sit waiting on the SMs through the last wave, cost 0.03 ms.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
// process-wide switch (option "pdl"); off: plain launches
inline bool& pdl_enabled() {
  static bool on = true;
  return on;
}
// launch errors surface through cudaGetLastError, as for <<<...>>>
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  (void)cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// Row of node i's component LM in the L-grouped split operand of the M0_adj GEMM (L_max
// 1): the N rows of L = 0, then the 3N rows of L = 1, so that each L block is one
// contiguous GEMM segment with its own weights.  (The H1 GEMM keeps rows (node, LM) and
// computes both L blocks for every row, keeping the rows of its block: written this way
// by the layer-0 forward, its rows made that kernel 0.006 ms slower than the 0.002 ms the
// GEMM gained.)
__host__ __device__ __forceinline__ long lgroup_row(long N, long i, int LM) { return LM == 0 ? i : N + 3 * i + LM - 1; }

// Host side: the kernel's model copy and grid for n atoms under the current schedule.
inline int atom_grid(const DevModel& m, int k, int n, DevModel& mk) {
  mk = m;
  if (m.sched && m.pgrid[k] > 0) return m.pgrid[k] < n ? m.pgrid[k] : n;
  mk.sched = nullptr;
  return n;
}

// The split-term products of a tensor-core GEMM with T terms: x_hi W_hi (T = 1),
// + x_hi W_lo (T = 2), + x_lo W_hi (T = 3), hi = bf16(v), lo = bf16(v - hi).  An X
// operand row stores split_xterms(T) blocks of width K, (hi) or (hi | lo); a B operand
// row stores (W_hi) for T = 1, else (W_hi | W_lo); the GEMM reads each block once per
// k-block and issues the T products from shared memory.
__host__ __device__ __forceinline__ int split_xterms(int T) { return T == 3 ? 2 : 1; }
__host__ __device__ __forceinline__ int split_wterms(int T) { return T == 1 ? 1 : 2; }
// element `col` of an X operand row of width K (row pitch split_xterms(T) * K)
__device__ __forceinline__ void write_split(__nv_bfloat16* row, int K, int T, int col, float v) {
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  row[col] = hi;
  if (T == 3) row[K + col] = __float2bfloat16_rn(v - __bfloat162float(hi));
}

// ZBL energy of one directed edge and its r-derivative, as zbl.cpp:22-94
// (energy 0.5 * v(r) * envelope(r); each pair appears as two directed edges).
__device__ __forceinline__ void zbl_edge(const DevModel& m, float4 pq, float r, float& V, float& dV) {
  V = 0.0f;
  dV = 0.0f;
  const float rmax = pq.z;
  if (!(r < rmax)) return;
  const float ce[4] = {-3.2f, -0.9423f, -0.4028f, -0.2016f};
  float phi = 0.0f, dphi = 0.0f;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float e = m.zbl_c[q] * expf(ce[q] * r * pq.x);
    phi += e;
    dphi += ce[q] * pq.x * e;
  }
  const float v = pq.y * 2.0f * phi / r;                      // 14.3996 Zu Zv phi / r
  const float dv = pq.y * 2.0f * (r * dphi - phi) / (r * r);
  const float t = r / rmax;
  const int p = m.zbl_p;
  float tp1 = 1.0f;  // t^(p-1)
  for (int q = 0; q < p - 1; ++q) tp1 *= t;
  const float tp = tp1 * t, tp2 = tp * t, tp3 = tp2 * t;
  const float fp = static_cast<float>(p);
  const float env = 1.0f - (fp + 1.0f) * (fp + 2.0f) * 0.5f * tp + fp * (fp + 2.0f) * tp2 -
                    fp * (fp + 1.0f) * 0.5f * tp3;
  const float denv = (-(fp + 1.0f) * (fp + 2.0f) * 0.5f * fp * tp1 + fp * (fp + 2.0f) * (fp + 1.0f) * tp -
                      fp * (fp + 1.0f) * 0.5f * (fp + 2.0f) * tp2) / rmax;
  V = 0.5f * v * env;
  dV = 0.5f * (v * denv + dv * env);
}

// Edge list in the evaluator's layout (libsymmetrix/source/mace.hpp:29-35): CSR by
// centre node, xyz = x_j - x_i, r = |xyz|.  Edges with r >= r_cut are skipped
// (they contribute nothing), which lets an MD driver keep a skin list.
struct EdgeIn {
  const int* first;      // [N+1]
  const int* node_type;  // [N]
  const int* nidx;       // [E]
  const int* ntype_e;    // [E]
  const double* xyz;     // [E][3]
  const double* r;       // [E]
  int N;
  // Processing order of the centre atoms (block b works on atom order[b]); nullptr: the
  // identity.  A species-sorted order keeps the spline rows the blocks in flight gather
  // (the pairs of one centre species) inside L2 when the whole table is larger.
  const int* order = nullptr;
  // End of each centre atom's edges (nullptr: first[i + 1]): a list whose segments are
  // only partly filled, e.g. the in-cut-off edges packed at the front of a skin list's.
  const int* last = nullptr;
  // Centres i >= n_local are a halo evaluated by layer 0 only (the pair style's
  // no-MPI-message-passing form): their edges carry neither ZBL nor layer-1 forces.
  int n_local = 0x7fffffff;
  __device__ __forceinline__ int atom_at(int b) const { return order ? order[b] : b; }
  __device__ __forceinline__ int end(int i) const { return last ? last[i] : first[i + 1]; }
};

// Canonical layer-1 tensor-product instructions (l1 from Y_lm, l2 from H1),
// ordered by output l; the loader reorders model data to this order.
__host__ __device__ constexpr int ins_count(int LMAX) { return LMAX == 1 ? 10 : 17; }
__host__ __device__ constexpr int ins_l1(int LMAX, int q) {
  constexpr int a1[10] = {0, 1, 1, 0, 2, 2, 1, 3, 3, 2};
  constexpr int a2[17] = {0, 1, 2, 1, 0, 2, 1, 3, 2, 1, 3, 0, 2, 3, 2, 1, 3};
  return LMAX == 1 ? a1[q] : a2[q];
}
__host__ __device__ constexpr int ins_l2(int LMAX, int q) {
  constexpr int b1[10] = {0, 1, 0, 1, 1, 0, 1, 1, 0, 1};
  constexpr int b2[17] = {0, 1, 2, 0, 1, 1, 2, 2, 0, 1, 1, 2, 2, 0, 1, 2, 2};
  return LMAX == 1 ? b1[q] : b2[q];
}
// offset of instruction q's (m1, m2) block in the Phi1r row p = (q, m1, m2)
__host__ __device__ constexpr int ins_poff(int LMAX, int q) {
  int p = 0;
  for (int w = 0; w < q; ++w) p += (2 * ins_l1(LMAX, w) + 1) * (2 * ins_l2(LMAX, w) + 1);
  return p;
}
__host__ __device__ constexpr int ins_np(int LMAX) { return ins_poff(LMAX, ins_count(LMAX)); }

// Calls f(std::integral_constant<int, q>) for every instruction q, so that the
// loop body sees l1, l2 and the Phi1r offset as compile-time constants.
template <typename F, int... Q>
__device__ __forceinline__ void for_each_ins_impl(F&& f, std::integer_sequence<int, Q...>) {
  (f(std::integral_constant<int, Q>{}), ...);
}
template <int LMAX, typename F>
__device__ __forceinline__ void for_each_ins(F&& f) {
  for_each_ins_impl(f, std::make_integer_sequence<int, ins_count(LMAX)>{});
}

__device__ __forceinline__ float spline_val(const float4 c, float x) {
  return fmaf(x, fmaf(x, fmaf(x, c.w, c.z), c.y), c.x);
}
__device__ __forceinline__ float spline_der(const float4 c, float x) {
  return fmaf(x, fmaf(3.0f * x, c.w, 2.0f * c.z), c.y);
}

// Real spherical harmonics l <= 3 of the edge vector v in the evaluator's
// convention: shuffle (x,y,z) -> (z,x,y), orthonormal real Y_lm without the
// Condon-Shortley phase, times 2 sqrt(pi) (libsymmetrix/source/mace.cpp:118-148).
// Each Y_lm = s P_lm(u) with P_lm homogeneous of degree l and u the unit vector;
// the gradient with respect to v is s (grad P_lm(u) - l P_lm(u) u) / |v|.
template <bool GRAD>
__device__ __forceinline__ void sph_harm16(float vx, float vy, float vz, float* Y, float* G /*[3][16]*/) {
  const float r2 = vx * vx + vy * vy + vz * vz;
  const float inv_r = rsqrtf(r2);
  const float X = vz * inv_r, Yv = vx * inv_r, Z = vy * inv_r;  // shuffled unit vector
  // 2 sqrt(pi) times the orthonormal normalisation constants
  const float s0 = 1.0f;
  const float s1 = 1.7320508075688772f;                      // sqrt(3)
  const float s2a = 3.872983346207417f;                      // sqrt(15)
  const float s2b = 1.118033988749895f;                      // sqrt(5)/2
  const float s2c = 1.9364916731037085f;                     // sqrt(15)/2
  const float s3a = 2.091650066335189f;                      // sqrt(35/8)
  const float s3b = 10.246950765959598f;                     // sqrt(105)
  const float s3c = 1.620185174601965f;                      // sqrt(21/8)
  const float s3d = 1.3228756555322954f;                     // sqrt(7)/2
  const float s3e = 5.123475382979799f;                      // sqrt(105)/2
  const float XX = X * X, YY = Yv * Yv, ZZ = Z * Z;
  Y[0] = s0;
  Y[1] = s1 * Yv;
  Y[2] = s1 * Z;
  Y[3] = s1 * X;
  Y[4] = s2a * X * Yv;
  Y[5] = s2a * Yv * Z;
  Y[6] = s2b * (2.0f * ZZ - XX - YY);
  Y[7] = s2a * X * Z;
  Y[8] = s2c * (XX - YY);
  Y[9] = s3a * Yv * (3.0f * XX - YY);
  Y[10] = s3b * X * Yv * Z;
  Y[11] = s3c * Yv * (4.0f * ZZ - XX - YY);
  Y[12] = s3d * Z * (2.0f * ZZ - 3.0f * XX - 3.0f * YY);
  Y[13] = s3c * X * (4.0f * ZZ - XX - YY);
  Y[14] = s3e * Z * (XX - YY);
  Y[15] = s3a * X * (XX - 3.0f * YY);
  if constexpr (GRAD) {
    // dP/d(X, Y, Z) in shuffled axes
    float D[3][16];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int q = 0; q < 16; ++q) D[a][q] = 0.0f;
    D[1][1] = s1;
    D[2][2] = s1;
    D[0][3] = s1;
    D[0][4] = s2a * Yv; D[1][4] = s2a * X;
    D[1][5] = s2a * Z;  D[2][5] = s2a * Yv;
    D[0][6] = -2.0f * s2b * X; D[1][6] = -2.0f * s2b * Yv; D[2][6] = 4.0f * s2b * Z;
    D[0][7] = s2a * Z; D[2][7] = s2a * X;
    D[0][8] = 2.0f * s2c * X; D[1][8] = -2.0f * s2c * Yv;
    D[0][9] = 6.0f * s3a * X * Yv; D[1][9] = 3.0f * s3a * (XX - YY);
    D[0][10] = s3b * Yv * Z; D[1][10] = s3b * X * Z; D[2][10] = s3b * X * Yv;
    D[0][11] = -2.0f * s3c * X * Yv; D[1][11] = s3c * (4.0f * ZZ - XX - 3.0f * YY); D[2][11] = 8.0f * s3c * Yv * Z;
    D[0][12] = -6.0f * s3d * X * Z; D[1][12] = -6.0f * s3d * Yv * Z; D[2][12] = s3d * (6.0f * ZZ - 3.0f * XX - 3.0f * YY);
    D[0][13] = s3c * (4.0f * ZZ - 3.0f * XX - YY); D[1][13] = -2.0f * s3c * X * Yv; D[2][13] = 8.0f * s3c * X * Z;
    D[0][14] = 2.0f * s3e * X * Z; D[1][14] = -2.0f * s3e * Yv * Z; D[2][14] = s3e * (XX - YY);
    D[0][15] = 3.0f * s3a * (XX - YY); D[1][15] = -6.0f * s3a * X * Yv;
    const float u[3] = {X, Yv, Z};
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const float l = q == 0 ? 0.0f : (q < 4 ? 1.0f : (q < 9 ? 2.0f : 3.0f));
      const float lp = l * Y[q];
      const float gX = (D[0][q] - lp * u[0]) * inv_r;
      const float gY = (D[1][q] - lp * u[1]) * inv_r;
      const float gZ = (D[2][q] - lp * u[2]) * inv_r;
      // back to (x, y, z): d/dx = d/dY', d/dy = d/dZ', d/dz = d/dX'
      G[0 * 16 + q] = gY;
      G[1 * 16 + q] = gZ;
      G[2 * 16 + q] = gX;
    }
  }
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

inline int ceil_div(long a, long b) { return static_cast<int>((a + b - 1) / b); }

// ---- channel-pair helpers: packed FP32 (sm_100 and later: two FMAs per instruction) ----
template <typename F, int... I>
__device__ __forceinline__ void static_for_impl(F&& f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
// f(std::integral_constant<int, i>) for i in [0, N)
template <int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }

// Cubic of a channel pair at offset x2 = (x, x) inside its interval, value only.
__device__ __forceinline__ float2 spline2_val(float4 lo, float4 hi, float2 x2) {
  const float2 c0 = make_float2(lo.x, lo.y), c1 = make_float2(lo.z, lo.w);
  const float2 c2 = make_float2(hi.x, hi.y), c3 = make_float2(hi.z, hi.w);
  return fma2(fma2(fma2(c3, x2, c2), x2, c1), x2, c0);
}
// Value and derivative by the two-row Horner scheme (5 packed FMAs).
__device__ __forceinline__ void spline2(float4 lo, float4 hi, float2 x2, float2& R, float2& Rd) {
  const float2 c0 = make_float2(lo.x, lo.y), c1 = make_float2(lo.z, lo.w);
  const float2 c2 = make_float2(hi.x, hi.y), c3 = make_float2(hi.z, hi.w);
  float2 p = fma2(c3, x2, c2);
  float2 d = fma2(c3, x2, p);
  p = fma2(p, x2, c1);
  d = fma2(d, x2, p);
  R = fma2(p, x2, c0);
  Rd = d;
}


// Density-normalisation spline of `layer` for the unordered pair (ti, tj) at r: value
// and r-derivative (CubicSpline::evaluate_deriv, libsymmetrix/source/cubic_spline.cpp:29-41).
__device__ __forceinline__ void dens_eval(const DevModel& m, int layer, int ti, int tj, float r, float& v,
                                          float& d) {
  const int a = ti < tj ? ti : tj, b = ti < tj ? tj : ti;
  const int pr = a * (2 * m.S - a - 1) / 2 + b;
  int iv = static_cast<int>(r * m.dens_inv_h[layer]);
  iv = iv < 0 ? 0 : (iv >= m.dens_nint[layer] ? m.dens_nint[layer] - 1 : iv);
  const float x = r - static_cast<float>(iv) * m.dens_h[layer];
  const float4 c = __ldg(m.dens_spl[layer] + static_cast<size_t>(pr) * m.dens_nint[layer] + iv);
  v = spline_val(c, x);
  d = spline_der(c, x);
}

// Sum of v over the block (blockDim a multiple of 32, at most 1024 threads); every
// thread gets the total.  Contains __syncthreads: call from uniform control flow.
__device__ __forceinline__ float block_sum(float v) {
  __shared__ float red[33];
  v = warp_sum(v);
  const int nw = blockDim.x >> 5;
  __syncthreads();  // red may still be read by a previous call
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < nw; ++w) t += red[w];
    red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// s_i = 1 + sum over the node's edges of the density spline (compute_A0_scaled /
// compute_A1_scaled, libsymmetrix/source/mace.cpp:273-297, :681-705).
__device__ __forceinline__ float dens_factor(const DevModel& m, int layer, const EdgeIn& in, int i, int ti) {
  float z = 0.0f;
  for (int e = in.first[i] + threadIdx.x; e < in.end(i); e += blockDim.x) {
    float v, d;
    dens_eval(m, layer, ti, in.ntype_e[e], static_cast<float>(in.r[e]), v, d);
    z += v;
  }
  return 1.0f + block_sum(z);
}

}  // namespace smx
