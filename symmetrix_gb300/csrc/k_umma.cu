// Channel-mixing GEMMs on the tcgen05 tensor cores (the BF16 precision form).
//
//   Y[rows, N] = X[rows, K] . B[N, K]^T     X, B bf16 (K contiguous), Y f32
//
// One CTA per 128-row x NT-column tile.  Thread 0 streams 64-wide k-blocks of the X
// tile and the B tile with TMA (128-byte swizzled boxes) through a ring of up to four
// shared-memory stages (full/empty mbarriers); a stage holds the k-block of every stored
// split term (X: hi, lo; B: W_hi, W_lo).  Thread 32 issues, per 16-wide step of the
// k-block, one tcgen05.mma (M=128, N=NT, K=16) per split product (x_hi W_hi, x_hi W_lo,
// x_lo W_hi) into an f32 accumulator in tensor memory, so each term is loaded once and
// used by every product that needs it, and releases each stage with tcgen05.commit;
// after the last commit the four warps read their 32 accumulator lanes back with
// tcgen05.ld and store them through an affine row map straight into the engine's
// feature layouts.
//
// These GEMMs restate compute_H1, compute_A1, reverse_A1 and reverse_H1
// (libsymmetrix/source/mace.cpp:397-451, :607-679) with bf16 operands and f32
// accumulation.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>

#include "kernels.h"
#include "sm100.cuh"

namespace smx {

namespace {

constexpr int kBoxK = 64;      // bf16 elements per TMA box row (128 B: one swizzle atom row)
constexpr int kTileM = 128;

__device__ __forceinline__ void record_timeout(unsigned* status) {
  if (status) atomicOr(status, 1u);
}

constexpr int kStages = 4;     // maximum shared-memory ring depth (k-blocks in flight)

// Up to four independent GEMMs in one launch (blockIdx.z selects the segment; the
// blocks beyond a segment's tile counts return at once).  blockIdx.x runs over the
// segment's tiles N-tile fastest, so the CTAs that read the same 128-row X tile run
// back to back and all but the first find it in L2.
struct UmmaSegDev {
  CUtensorMap ta, tb;
  UmmaOut o;
  int K, NT, tiles_m, tiles_n, stages, terms;
};
struct UmmaGroupDev {
  UmmaSegDev s[4];
  // test of the error path: the producer issues no load and the MMA thread waits
  // wait_ns for one, so its bounded wait runs out with nothing in flight
  int skip_loads;
  uint64_t wait_ns;
};

__global__ void __launch_bounds__(128, 1) k_umma_gemm(const __grid_constant__ UmmaGroupDev grp, unsigned* status) {
  pdl_begin();
  const UmmaSegDev& seg = grp.s[blockIdx.z];
  const int tile_n = static_cast<int>(blockIdx.x % static_cast<unsigned>(seg.tiles_n));
  const int tile_m = static_cast<int>(blockIdx.x / static_cast<unsigned>(seg.tiles_n));
  if (tile_m >= seg.tiles_m) return;
  const CUtensorMap& ta = seg.ta;
  const CUtensorMap& tb = seg.tb;
  const UmmaOut& o = seg.o;
  const int K = seg.K, NT = seg.NT, terms = seg.terms;
  const int XT = split_xterms(terms), WT = split_wterms(terms);
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kStages], empty[kStages], bar_mma;  // kStages >= seg.stages
  __shared__ uint32_t tmem_base;
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int KB = K / kBoxK;
  const int S = KB < seg.stages ? KB : seg.stages;
  const uint32_t a_bytes = kTileM * kBoxK * 2, b_bytes = static_cast<uint32_t>(NT) * kBoxK * 2;
  // stage = the XT X boxes, then the WT B boxes (all 1024-B multiples)
  const uint32_t stage_bytes = XT * a_bytes + WT * b_bytes;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = tile_m * kTileM, n0 = tile_n * NT;
  const uint32_t ncols = NT <= 32 ? 32u : (NT <= 64 ? 64u : (NT <= 128 ? 128u : 256u));

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      sm100::mbar_init(&full[s], 1);
      sm100::mbar_init(&empty[s], 1);
    }
    sm100::mbar_init(&bar_mma, 1);
    sm100::fence_mbar_init();
  }
  if (warp == 0) {
    sm100::tmem_alloc(&tmem_base, ncols);
    sm100::tmem_relinquish();
  }
  sm100::tc_fence_before();
  __syncthreads();
  sm100::tc_fence_after();
  const uint32_t tmem = tmem_base;

  // producer: k-block kb goes to stage kb % S once the MMAs of k-block kb - S released it
  int loads = 0;
  bool prod_ok = true;
  if (threadIdx.x == 0 && !grp.skip_loads) {
    for (int kb = 0; kb < KB; ++kb) {
      const int s = kb % S;
      if (kb >= S && !sm100::mbar_wait(&empty[s], ((kb / S) - 1) & 1)) {
        prod_ok = false;
        break;
      }
      uint8_t* st = smem + static_cast<size_t>(s) * stage_bytes;
      sm100::mbar_arrive_expect_tx(&full[s], stage_bytes);
      for (int t = 0; t < XT; ++t) sm100::tma_load_2d(st + t * a_bytes, &ta, t * K + kb * kBoxK, m0, &full[s]);
      for (int u = 0; u < WT; ++u)
        sm100::tma_load_2d(st + XT * a_bytes + u * b_bytes, &tb, u * K + kb * kBoxK, n0, &full[s]);
      ++loads;
    }
  }
  // MMA issuer
  bool issued = false, mma_ok = true;
  if (threadIdx.x == 32) {
    const uint32_t idesc = sm100::idesc_bf16_f32(kTileM, NT);
    for (int kb = 0; kb < KB; ++kb) {
      const int s = kb % S;
      if (!sm100::mbar_wait(&full[s], (kb / S) & 1, grp.wait_ns)) {
        mma_ok = false;
        break;
      }
      sm100::tc_fence_after();
      const uint32_t x0 = sm100::smem_u32(smem + static_cast<size_t>(s) * stage_bytes), w0 = x0 + XT * a_bytes;
#pragma unroll
      for (int k = 0; k < kBoxK / 16; ++k) {  // 16 elements (32 B) per MMA inside the 128-B swizzled row
        // x_hi W_hi, then x_hi W_lo (terms >= 2), then x_lo W_hi (terms 3)
        sm100::umma_bf16(tmem, sm100::sdesc_sw128(x0 + k * 32), sm100::sdesc_sw128(w0 + k * 32), idesc,
                         (kb | k) != 0 ? 1u : 0u);
        if (terms >= 2)
          sm100::umma_bf16(tmem, sm100::sdesc_sw128(x0 + k * 32), sm100::sdesc_sw128(w0 + b_bytes + k * 32), idesc,
                           1u);
        if (terms == 3)
          sm100::umma_bf16(tmem, sm100::sdesc_sw128(x0 + a_bytes + k * 32), sm100::sdesc_sw128(w0 + k * 32), idesc,
                           1u);
      }
      sm100::umma_commit(&empty[s]);
      issued = true;
    }
    // bar_mma: every MMA issued above has completed (also on the error path)
    if (issued) sm100::umma_commit(&bar_mma);
  }
  const int ok = __syncthreads_and((prod_ok && mma_ok) ? 1 : 0);
  const int any_mma = __syncthreads_or(issued ? 1 : 0);
  bool done = false;
  if (any_mma) done = sm100::mbar_wait(&bar_mma, 0);
  const int all_done = __syncthreads_and((done && ok) ? 1 : 0);
  sm100::tc_fence_after();
  if (all_done) {
    const int r = m0 + warp * 32 + lane;
    const bool row_ok = r < o.rows;
    long base = 0;
    bool write = row_ok;
    if (row_ok) {
      base = static_cast<long>(r / o.rpn) * o.y_ns + o.y_off + static_cast<long>(r % o.rpn) * o.y_rs +
             (o.select ? 0 : n0);
      if (o.select) write = ((r % o.rpn) == 0) == (tile_n == 0);
    }
    // Each 32-column chunk goes through a 4 KB staging tile per warp (the ring's shared
    // memory is free once every MMA has completed): a lane holds one row after tcgen05.ld,
    // while a coalesced store wants eight lanes on 128 contiguous bytes of one row.  The
    // float4 groups of row t sit at slot q ^ (t & 7), so both the row-wise writes and the
    // transposed reads hit all 32 banks.
    float* stg = reinterpret_cast<float*>(smem) + warp * 32 * 32;
    const int sub = lane >> 3, c4 = lane & 7;
    for (int c0 = 0; c0 < NT; c0 += 32) {
      float v[32];
      sm100::tmem_ld32(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0), v);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        reinterpret_cast<float4*>(stg + lane * 32)[q ^ (lane & 7)] =
            make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      __syncwarp();
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int t = 4 * j + sub;  // the warp's row this lane stores now
        const long b = __shfl_sync(0xffffffffu, base, t);
        const int w = __shfl_sync(0xffffffffu, write ? 1 : 0, t);
        const float4 val = reinterpret_cast<const float4*>(stg + t * 32)[c4 ^ (t & 7)];
        if (w) reinterpret_cast<float4*>(o.Y + b + c0)[c4] = val;
      }
      __syncwarp();  // the next chunk overwrites the staging tile
    }
  } else if (threadIdx.x == 0) {
    record_timeout(status);
    // no TMA copy may still be landing in shared memory when the CTA exits: wait for
    // the last load issued into each stage
    for (int kb = loads - S > 0 ? loads - S : 0; kb < loads; ++kb) sm100::mbar_wait(&full[kb % S], (kb / S) & 1);
  }
  sm100::tc_fence_before();
  __syncthreads();
  if (warp == 0) sm100::tmem_dealloc(tmem, ncols);
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encoder() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  if (!fn) throw std::runtime_error("cuTensorMapEncodeTiled is not available from the driver");
  return fn;
}

// 2-D bf16 tensor map over a row-major [rows][K] matrix, box = 64 x box_rows, 128-B swizzle.
CUtensorMap make_map(const void* base, long rows, int K, int box_rows) {
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0) throw std::invalid_argument("tensor map base not 16-byte aligned");
  if (K % kBoxK != 0) throw std::invalid_argument("GEMM K must be a multiple of 64");
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  const cuuint64_t dims[2] = {static_cast<cuuint64_t>(K), static_cast<cuuint64_t>(rows)};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(K) * 2};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(kBoxK), static_cast<cuuint32_t>(box_rows)};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box,
                               estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (" + std::to_string(r) + ")");
  return m;
}

}  // namespace

size_t umma_smem_bytes(int K, int NT, int stages, int terms) {
  stages = std::min(K / kBoxK, std::min(stages, kStages));
  return static_cast<size_t>(stages) * (split_xterms(terms) * kTileM + split_wterms(terms) * NT) * kBoxK * 2 + 1024;
}

// dynamic shared memory available next to the kernel's few static words
constexpr size_t kMaxDynSmem = 226 * 1024;

// (the launch lowers a schedule's ring depth until its stages fit)
bool umma_supported(int K, int NT, int terms) {
  return K % kBoxK == 0 && K > 0 && NT % 32 == 0 && NT >= 32 && NT <= 256 && terms >= 1 && terms <= 3 &&
         umma_smem_bytes(K, NT, 1, terms) <= kMaxDynSmem;
}

cudaError_t init_umma_kernels() {
  return cudaFuncSetAttribute(k_umma_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              static_cast<int>(kMaxDynSmem));
}

void launch_umma_gemms(const UmmaGemm* g, int n, unsigned* status, cudaStream_t s, bool test_timeout) {
  if (n < 1 || n > 4) throw std::invalid_argument("1 to 4 tensor-core GEMMs per launch");
  UmmaGroupDev grp;
  std::memset(&grp, 0, sizeof(grp));
  grp.skip_loads = test_timeout ? 1 : 0;
  grp.wait_ns = test_timeout ? 2000000ull : sm100::kWaitLimitNs;  // 2 ms when testing
  long gx = 0;
  size_t smem = 0;
  int used = 0;
  for (int q = 0; q < n; ++q) {
    const UmmaGemm& a = g[q];
    if (!umma_supported(a.K, a.NT, a.terms) || a.nb_rows % a.NT != 0)
      throw std::invalid_argument("unsupported tensor-core GEMM shape");
    if (a.rows <= 0) continue;
    UmmaSegDev& d = grp.s[used++];
    d.ta = make_map(a.X, a.rows, split_xterms(a.terms) * a.K, kTileM);
    d.tb = make_map(a.B, a.nb_rows, split_wterms(a.terms) * a.K, a.NT);
    d.o = a.o;
    d.K = a.K;
    d.NT = a.NT;
    d.terms = a.terms;
    d.tiles_m = static_cast<int>((a.rows + kTileM - 1) / kTileM);
    d.tiles_n = a.nb_rows / a.NT;
    d.stages = a.stages >= 1 && a.stages <= kStages ? a.stages : kStages;
    while (d.stages > 1 && umma_smem_bytes(a.K, a.NT, d.stages, a.terms) > kMaxDynSmem) --d.stages;
    gx = std::max(gx, static_cast<long>(d.tiles_m) * d.tiles_n);
    smem = std::max(smem, umma_smem_bytes(a.K, a.NT, d.stages, a.terms));
  }
  if (used == 0) return;
  if (gx > 0x7fffffffL) throw std::invalid_argument("tensor-core GEMM too large for one launch");
  launch_pdl(k_umma_gemm, dim3(static_cast<unsigned>(gx), 1, used), 128, smem, s, grp, status);
}

}  // namespace smx
