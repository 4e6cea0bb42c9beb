// Kernel launchers of the GB300 MACE engine (host-callable).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "device.cuh"

namespace smx {

// k_edge.cu
cudaError_t init_edge_kernels(const DevModel& m);
// resident blocks per SM of each per-atom kernel (indexed by AtomKernel) at the launch
// shapes of this model: the persistent grid is this times the SM count
void layer0_residency(const DevModel& m, int* per_sm);
void layer1_residency(const DevModel& m, int* per_sm);
void node_tail_residency(const DevModel& m, int* per_sm);
void launch_layer0_fwd(const DevModel& m, const EdgeIn& in, float* A0, float* M0, float* zbl_e, cudaStream_t s);
void launch_layer0_rev(const DevModel& m, const EdgeIn& in, const float* A0, const float* M0_adj, const double* f1,
                       float* A0_adj, double* forces, cudaStream_t s);

// k_layer1.cu
cudaError_t init_layer1_kernels(const DevModel& m);
int layer1_block(int C);
void launch_layer1_fwd(const DevModel& m, const EdgeIn& in, const float* H1, float* Phi1, cudaStream_t s);
// H1_adj: fixed-point accumulator (see to_fixed), seeded by launch_node_tail
void launch_layer1_rev(const DevModel& m, const EdgeIn& in, const float* H1, const float* dPhi1, fix64* H1_adj,
                       double* f1, cudaStream_t s);

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

void launch_node_tail(const DevModel& m, const int* node_type, int N, float* A1, const float* H1, float* M1,
                      float* H2, float* A1_adj, fix64* H1_adj, float* M1_adj, float* H2_adj, const float* zbl_e,
                      double* energies, cudaStream_t s);
// dst[rows][C] = the fixed-point rows src ([N][nLM][C]) as float; bf (optional, L_max 1):
// their bf16 split terms for a GEMM with `terms` products (write_split), row pitch
// split_xterms(terms) * C, rows grouped by L (lgroup_row)
void launch_fixed_rows(const fix64* src, float* dst, __nv_bfloat16* bf, long rows, int C, int terms, int nLM,
                       cudaStream_t s);
// single-stage calls: dst = fixed-point copy of src (zero: dst = 0); forces = (zero ? 0 :
// forces) - the sum of the nslices f1 slices (stride apart), n = 3 * edges
void launch_rows_to_fixed(const float* src, fix64* dst, long n, bool zero, cudaStream_t s);
void launch_forces_from_f1(double* forces, const double* f1, long stride, int nslices, long n, bool zero,
                           cudaStream_t s);
void launch_scan_first(const int* num_neigh, int N, int* first, cudaStream_t s);
// input check of the host API (bits of the flags word)
constexpr unsigned kBadNodeType = 1, kBadNumNeigh = 2, kBadEdgeCount = 4, kBadNeighIndex = 8, kBadNeighType = 16,
                   kBadEdge = 32;
void launch_validate_inputs(int N, long E, int S, double r_cut, const int* node_types, const int* num_neigh,
                            const int* first, const int* nidx, const int* ntype_e, const double* xyz, const double* r,
                            unsigned* flags, cudaStream_t s);
// order[N]: the atoms sorted by species (node_type in [0, S))
void launch_species_order(const int* node_type, int N, int S, int* order, cudaStream_t s);

// k_umma.cu: Y = X . B^T on the tcgen05 tensor cores (bf16 operands, f32 accumulation).
// Row r of the GEMM, column c of N-tile y lands at
//   Y + (r / rpn) * y_ns + y_off + (r % rpn) * y_rs + (select ? 0 : y * NT) + c;
// with select, N-tile y is written only for rows with (r % rpn == 0) == (y == 0) (the
// L = 0 and L = 1 weight blocks of the H1 and M0_adj GEMMs, computed as two N-tiles).
struct UmmaOut {
  float* Y;
  long rows;
  int rpn;
  long y_ns;
  int y_off, y_rs;
  int select;
};
cudaError_t init_umma_kernels();
size_t umma_smem_bytes(int K, int NT, int stages, int terms);
bool umma_supported(int K, int NT, int terms);
// One GEMM, Y = sum of the `terms` split products (write_split): X [rows][XT * K] bf16
// (XT = split_xterms(terms) blocks of K), B [nb_rows][WT * K] bf16 (WT = split_wterms(terms);
// N-tiles of NT rows), output map o.
struct UmmaGemm {
  const __nv_bfloat16* X;
  long rows;
  int K;
  const __nv_bfloat16* B;
  int nb_rows, NT;
  UmmaOut o;
  int stages = 4;  // shared-memory ring depth, 1..4
  int terms = 1;   // split products: 1, 2 or 3
};
// 1 to 4 GEMMs in one launch.
// test_timeout: a test of the error path (no TMA load is issued and the MMA thread's
// wait gives up after 2 ms: the launch records a timeout in *status and writes nothing)
void launch_umma_gemms(const UmmaGemm* g, int n, unsigned* status, cudaStream_t s, bool test_timeout = false);

// k_md.cu
void launch_wrap(int N, double3 box, int3 periodic, double* pos, cudaStream_t s);
void launch_cell_list(const double* pos, int N, double3 box, int3 nc, int* cell, int* cell_count, int* cell_start,
                      int* cell_fill, int* cell_tmp, int* cell_atoms, cudaStream_t s);
// slot k of the MD atom arrays takes atom perm[k]: gathered into tmp_d [pos 3N | vel 3N |
// F 3N | inv_m N] and tmp_i [species N | orig N]
void launch_permute_atoms(int N, const int* perm, const double* pos, const double* vel, const double* F,
                          const double* inv_m, const int* species, const int* orig, double* tmp_d, int* tmp_i,
                          cudaStream_t s);
// the two passes of the neighbour build (count, then fill); the count pass writes pos, the
// float32 copy of pos_d that both search
void launch_neigh_pass(bool fill, bool brute, const double* pos_d, float4* pos, const int* species, int N,
                       double3 box_d, int3 nc, int3 periodic, int3 nimg, double rl, const int* cell,
                       const int* cell_start, const int* cell_atoms, const int* seg_of, const int* seg_first,
                       int* num_neigh, const int* first, int* nidx, int* ntype_e, int* edge_i, char4* shift, long cap,
                       cudaStream_t s, int* cellseg = nullptr);
// rev[e] from the cell-list fill pass's per-atom segments (cellseg [N][28]: where each of
// the 27 neighbour cells' hits start in an atom's list, then its end)
void launch_reverse_edges_cells(long cap, int N, const int* first, const int* nidx, const int* edge_i,
                                const char4* shift, const int* cell, int3 nc, const int* cellseg, int* rev,
                                cudaStream_t s);
void launch_reverse_edges(long cap, int N, const int* first, const int* nidx, const int* edge_i, const char4* shift,
                          int* rev, cudaStream_t s);
void launch_edge_geometry(long cap, int N, const int* first, const double* pos, double3 box, const int* nidx,
                          const int* edge_i, const char4* shift, double* xyz, double* r, cudaStream_t s);
// the in-cut-off edges of a skin list packed per centre atom, with the maps both ways
// (see k_md.cu)
void launch_edge_geometry_packed(int N, const int* first, const double* pos, double3 box, const int* nidx,
                                 const int* ntype_e, const char4* shift, double r_cut, int* pinv, int* last, int* emap,
                                 int* nidx_p, int* ntype_p, double* xyz_p, double* r_p, cudaStream_t s);
// atomic forces from the packed edges' forces; dt > 0: also the second velocity-Verlet half
void launch_atom_forces_packed(int N, const int* first, const int* last, const int* emap, const int* rev,
                               const int* pinv, const double* f_p, double* F, double dt, const double* inv_m, double* v,
                               cudaStream_t s);
void launch_scatter_packed_forces(int N, const int* first, const int* last, const int* emap, const double* f_p,
                                  double* f_skin, cudaStream_t s);
void launch_atom_forces(int N, const int* first, const int* rev, const double* f, double* F, cudaStream_t s);
void launch_reduce(int N, const int* first, const double* energies, const double* xyz, const double* f,
                   double* partial, int nblocks, double* out, cudaStream_t s);
void launch_vv_first(int N, double dt, const double* F, const double* inv_m, double* v, double* x, cudaStream_t s);
void launch_vv_second(int N, double dt, const double* F, const double* inv_m, double* v, cudaStream_t s);

}  // namespace smx
