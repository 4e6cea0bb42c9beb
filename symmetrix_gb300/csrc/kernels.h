// Kernel launchers of the GB300 MACE engine (host-callable).
#pragma once

#include <cuda_runtime.h>

#include "device.cuh"

namespace smx {

// k_edge.cu
void launch_layer0_fwd(const DevModel& m, const EdgeIn& in, float* A0, float* M0, cudaStream_t s);
void launch_layer1_fwd(const DevModel& m, const EdgeIn& in, const float* H1, float* Phi1, cudaStream_t s);
void launch_layer1_rev(const DevModel& m, const EdgeIn& in, const float* H1, const float* dPhi1, float* H1_adj,
                       float* f1, cudaStream_t s);
void launch_layer0_rev(const DevModel& m, const EdgeIn& in, const float* A0, const float* M0_adj, const float* f1,
                       float* A0_adj, double* forces, cudaStream_t s);

// k_node.cu
// One segment of a row-gathered GEMM  Y[rows, ncols] = X[rows, K] @ B[K, ncols].
// Row r of a segment lives at  X + (r / rpn) * x_ns + x_off + (r % rpn) * x_rs
// (all in floats), which addresses one l-block of the [node][component][channel]
// feature layouts directly; likewise for Y.
struct GemmSeg {
  const float* X;
  float* Y;
  const float* B;
  int rows, K, ncols, rpn;
  long x_ns;
  int x_off, x_rs;
  long y_ns;
  int y_off, y_rs;
};
struct GemmBatch {
  GemmSeg s[4];
  int n;
};
void launch_gemm(const GemmBatch& b, cudaStream_t s);

void launch_node_tail(const DevModel& m, const int* node_type, int N, const float* A1, const float* H1, float* M1,
                      float* H2, float* A1_adj, float* H1_adj, float* M1_adj, float* H2_adj, double* energies,
                      cudaStream_t s);
void launch_scan_first(const int* num_neigh, int N, int* first, cudaStream_t s);

}  // namespace smx
