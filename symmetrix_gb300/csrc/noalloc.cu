// Allocation-free energy and virial reduction on device arrays.
//
// Some callers cannot call cudaMalloc at the point where they need this sum: a
// LAMMPS-Kokkos pair style, for example, works on device views that Kokkos owns and
// reduces energy and virial inside its compute() (pair_symmetrix_mace_kokkos.cpp
// does these reductions on device), and code running under another framework's
// memory pool or a fixed memory budget must not grow the device heap behind its back.
// This entry point therefore allocates nothing: the caller passes the inputs and the
// output, and the only scratch (one float64 partial sum per 4096-element chunk) lives
// in the file-scope device array below, which every GPU that loads the library keeps
// (1.25 MiB) until the process exits.
//
// The other reductions of this engine (smx_compute_atoms, smx_md_state) keep their
// partial sums in cudaMalloc'd workspaces; this one is separate code and changes none
// of them.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/smx_gb300.h"
#include "compsum.h"

namespace smx {
int fail(int code, const std::string& msg);
}

namespace {

constexpr int kChunk = 4096;          // nodes and edges summed by one block into one partial
constexpr int kMaxPartials = 16384;   // => at most 16384 * 4096 = 67,108,864 nodes, and as many edges
constexpr int kMaxDevices = 128;

// 10 float64 per partial: energy, then the 9 virial components.  Every slot the final
// pass reads is written by the first pass of the same call, so nothing here has to
// start at zero; the array simply keeps the last call's values.
static __device__ __align__(256) double g_partials[kMaxPartials * 10];

std::mutex g_mu;
double* g_partials_addr[kMaxDevices] = {};  // device address of g_partials, per device

// Device address of g_partials on the current device.  Resolved once per device, on
// that device's first call (which should therefore happen before any stream capture).
// The address belongs to the device's primary context: after cudaDeviceReset (or
// anything else that destroys and recreates that context) it is stale, and a caller
// that resets a device must not call this entry point on it again in the same process.
cudaError_t scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_partials_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_partials);
    if (e != cudaSuccess) return e;
    g_partials_addr[dev] = static_cast<double*>(p);
  }
  *out = g_partials_addr[dev];
  return cudaSuccess;
}

// Block b sums nodes and edges [b*kChunk, (b+1)*kChunk) in a fixed order, so the
// result does not depend on the GPU or on timing.
__global__ void __launch_bounds__(256) k_partials_noalloc(int N, long E, const double* __restrict__ energies,
                                                          const double* __restrict__ xyz,
                                                          const double* __restrict__ f,
                                                          double* __restrict__ partial) {
  __shared__ double sh[10][256];
  smx::CompSum acc[10];
  const long b0 = static_cast<long>(blockIdx.x) * kChunk;
  for (long e = b0 + threadIdx.x; e < b0 + kChunk && e < E; e += blockDim.x)
    for (int a = 0; a < 3; ++a)
      // __dmul_rn: the product is rounded on its own (no fused multiply-add with the
      // compensated sum's addition), so add() sees exactly the value it compensates for
      for (int c = 0; c < 3; ++c) acc[1 + 3 * a + c].add(__dmul_rn(xyz[3 * e + a], f[3 * e + c]));
  for (long i = b0 + threadIdx.x; i < b0 + kChunk && i < N; i += blockDim.x) acc[0].add(energies[i]);
  for (int q = 0; q < 10; ++q) sh[q][threadIdx.x] = acc[q].value();
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 10; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 10) partial[static_cast<long>(blockIdx.x) * 10 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_final_noalloc(int nb, const double* __restrict__ partial, double* __restrict__ out) {
  if (threadIdx.x < 10) {
    smx::CompSum s;
    for (int b = 0; b < nb; ++b) s.add(partial[static_cast<long>(b) * 10 + threadIdx.x]);
    out[threadIdx.x] = s.value();
  }
}

}  // namespace

extern "C" int smx_energy_virial_device_noalloc(int num_nodes, long num_edges, const double* node_energies,
                                                const double* xyz, const double* node_forces, double* out,
                                                void* stream) {
  if (num_nodes < 0 || num_edges < 0) return smx::fail(SMX_ERR_INVALID, "negative size");
  const long chunks = std::max<long>(std::max<long>((num_nodes + kChunk - 1) / kChunk,
                                                    (num_edges + kChunk - 1) / kChunk), 1);
  if (chunks > kMaxPartials)
    return smx::fail(SMX_ERR_CAPACITY,
                     "smx_energy_virial_device_noalloc: at most " + std::to_string(long(kMaxPartials) * kChunk) +
                         " nodes and at most " + std::to_string(long(kMaxPartials) * kChunk) +
                         " edges (fixed device scratch of " + std::to_string(kMaxPartials) +
                         " partial sums); got " + std::to_string(num_nodes) + " nodes, " +
                         std::to_string(num_edges) + " edges");
  if (!out || (num_nodes > 0 && !node_energies) || (num_edges > 0 && (!xyz || !node_forces)))
    return smx::fail(SMX_ERR_INVALID, "NULL device array");
  double* partial = nullptr;
  cudaError_t e = scratch_address(&partial);
  if (e != cudaSuccess) return smx::fail(SMX_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_partials_noalloc<<<static_cast<int>(chunks), 256, 0, s>>>(num_nodes, num_edges, node_energies, xyz, node_forces,
                                                                 partial);
  k_final_noalloc<<<1, 32, 0, s>>>(static_cast<int>(chunks), partial, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return smx::fail(SMX_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return SMX_OK;
}
