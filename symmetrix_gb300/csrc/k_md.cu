// Neighbour lists, per-step edge geometry, atomic forces / virial and velocity
// Verlet for the MD driver and the atom-level API.
//
// The reference delegates neighbour lists to its callers: the LAMMPS pair style
// filters LAMMPS's full list to r < r_cut (pair_symmetrix_mace.cpp:242-315) and
// the ASE calculator calls neighbor_list('ijdD') (symmetrix_calc.py:77).  Here a
// cell list builds the same full, directed, CSR-ordered list on the GPU with a
// skin, deterministically: atoms are binned, each cell's atom list is sorted by
// index, and every centre scans its 27 neighbour cells in a fixed order.
// Atomic forces and the virial follow pair_symmetrix_mace.cpp:324-368
// (F_j += f_e, F_i -= f_e; W = sum_e xyz_e (x) f_e), reduced without atomics via
// the reverse-edge map, in float64.
#include <cuda_runtime.h>

#include <algorithm>

#include "compsum.h"
#include "device.cuh"
#include "kernels.h"

namespace smx {

// ---- cell list ----
__global__ void k_cell_assign(const double* __restrict__ pos, int N, double3 box, int3 nc, int* __restrict__ cell,
                              int* __restrict__ cell_count) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  double p[3] = {pos[3 * a], pos[3 * a + 1], pos[3 * a + 2]};
  const double L[3] = {box.x, box.y, box.z};
  const int n[3] = {nc.x, nc.y, nc.z};
  int c[3];
  for (int d = 0; d < 3; ++d) {
    double f = p[d] / L[d];
    f -= floor(f);
    int q = static_cast<int>(f * n[d]);
    c[d] = q < 0 ? 0 : (q >= n[d] ? n[d] - 1 : q);
  }
  const int id = (c[0] * n[1] + c[1]) * n[2] + c[2];
  cell[a] = id;
  atomicAdd(cell_count + id, 1);
}

__global__ void k_cell_fill(const int* __restrict__ cell, int N, const int* __restrict__ cell_start,
                            int* __restrict__ cell_fill, int* __restrict__ cell_atoms) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  const int c = cell[a];
  cell_atoms[cell_start[c] + atomicAdd(cell_fill + c, 1)] = a;
}

// one warp per cell: each atom's rank among the cell's atoms (by index) is its place in
// the sorted list (cells hold tens of atoms; O(n^2 / 32) per cell)
__global__ void k_cell_sort(int ncell, const int* __restrict__ cell_start, const int* __restrict__ unsorted,
                            int* __restrict__ cell_atoms) {
  const int c = static_cast<int>((static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= ncell) return;
  const int b = cell_start[c], n = cell_start[c + 1] - b;
  for (int u = lane; u < n; u += 32) {
    const int v = unsorted[b + u];
    int rank = 0;
    for (int x = 0; x < n; ++x) rank += unsorted[b + x] < v;
    cell_atoms[b + rank] = v;
  }
}

// float32 copy of the positions for the neighbour search: the skin (1 A at the usual
// settings) absorbs its rounding, and the float64 pipe is slow on this part
__global__ void k_pos_to_float(int N, const double* __restrict__ pos, float4* __restrict__ posf) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  posf[a] = make_float4(static_cast<float>(pos[3 * a]), static_cast<float>(pos[3 * a + 1]),
                        static_cast<float>(pos[3 * a + 2]), 0.0f);
}

// Pass 0 counts, pass 1 fills.  Periodic images enter through the integer shift
// (sx, sy, sz) in box lengths; the list holds pairs with r < rl, excluding i itself.
template <bool FILL>
__global__ void k_neigh_cells(const float4* __restrict__ pos, const int* __restrict__ species, int N, float3 box,
                              int3 nc, int3 periodic, float rl2, const int* __restrict__ cell,
                              const int* __restrict__ cell_start, const int* __restrict__ cell_atoms,
                              int* __restrict__ num_neigh, const int* __restrict__ first, int* __restrict__ nidx,
                              int* __restrict__ ntype_e, int* __restrict__ edge_i, char4* __restrict__ shift,
                              long cap, int* __restrict__ cellseg) {
  // one warp per atom: the lanes test 32 candidates of a cell at a time and a ballot
  // keeps the hits in candidate order, so the list order is the sequential one; the fill
  // pass records where each of the 27 neighbour cells' hits start (cellseg, optional)
  const int i = static_cast<int>((static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= N) return;
  const unsigned below = (1u << lane) - 1u;
  const float4 pi = pos[i];
  const int ci = cell[i];
  const int cz = ci % nc.z, cy = (ci / nc.z) % nc.y, cx = ci / (nc.z * nc.y);
  long slot = FILL ? first[i] : 0;
  for (int dx = -1; dx <= 1; ++dx) {
    int qx = cx + dx, sx = 0;
    if (qx < 0) { if (!periodic.x) continue; qx += nc.x; sx = -1; }
    if (qx >= nc.x) { if (!periodic.x) continue; qx -= nc.x; sx = 1; }
    for (int dy = -1; dy <= 1; ++dy) {
      int qy = cy + dy, sy = 0;
      if (qy < 0) { if (!periodic.y) continue; qy += nc.y; sy = -1; }
      if (qy >= nc.y) { if (!periodic.y) continue; qy -= nc.y; sy = 1; }
      for (int dz = -1; dz <= 1; ++dz) {
        if (FILL && cellseg && lane == 0)
          cellseg[28L * i + ((dx + 1) * 3 + (dy + 1)) * 3 + (dz + 1)] = static_cast<int>(slot);
        int qz = cz + dz, sz = 0;
        if (qz < 0) { if (!periodic.z) continue; qz += nc.z; sz = -1; }
        if (qz >= nc.z) { if (!periodic.z) continue; qz -= nc.z; sz = 1; }
        const int q = (qx * nc.y + qy) * nc.z + qz;
        const float ox = sx * box.x, oy = sy * box.y, oz = sz * box.z;
        const int w1 = cell_start[q + 1];
        for (int w0 = cell_start[q]; w0 < w1; w0 += 32) {
          const int w = w0 + lane;
          int j = -1;
          bool hit = false;
          if (w < w1) {
            j = cell_atoms[w];
            if (!(j == i && sx == 0 && sy == 0 && sz == 0)) {
              const float4 pj = pos[j];
              const float ddx = pj.x + ox - pi.x, ddy = pj.y + oy - pi.y, ddz = pj.z + oz - pi.z;
              hit = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz)) < rl2;
            }
          }
          const unsigned ball = __ballot_sync(0xffffffffu, hit);
          if (FILL && hit) {
            const long sl = slot + __popc(ball & below);
            if (sl < cap) {
              nidx[sl] = j;
              ntype_e[sl] = species[j];
              edge_i[sl] = i;
              shift[sl] = make_char4(sx, sy, sz, 0);
            }
          }
          slot += __popc(ball);
        }
      }
    }
  }
  if (!FILL && lane == 0) num_neigh[i] = static_cast<int>(slot);
  if (FILL && cellseg && lane == 0) cellseg[28L * i + 27] = static_cast<int>(slot);
}

// Small or non-periodic systems: all pairs over the periodic images in range.
template <bool FILL>
__global__ void k_neigh_brute(const float4* __restrict__ pos, const int* __restrict__ species, int N, float3 box,
                              int3 nimg, float rl2, const int* __restrict__ seg_of, const int* __restrict__ seg_first,
                              int* __restrict__ num_neigh, const int* __restrict__ first, int* __restrict__ nidx,
                              int* __restrict__ ntype_e, int* __restrict__ edge_i, char4* __restrict__ shift,
                              long cap) {
  // one warp per atom, 32 candidates per ballot (order: candidate chunk, image, lane)
  const int i = static_cast<int>((static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= N) return;
  const unsigned below = (1u << lane) - 1u;
  const float4 pi = pos[i];
  long slot = FILL ? first[i] : 0;
  // with segments (a batch of molecules), only atoms of i's own segment are candidates
  const int j0 = seg_of ? seg_first[seg_of[i]] : 0, j1 = seg_of ? seg_first[seg_of[i] + 1] : N;
  for (int jb = j0; jb < j1; jb += 32) {
    const int j = jb + lane;
    const bool live = j < j1;
    for (int sx = -nimg.x; sx <= nimg.x; ++sx)
      for (int sy = -nimg.y; sy <= nimg.y; ++sy)
        for (int sz = -nimg.z; sz <= nimg.z; ++sz) {
          bool hit = false;
          if (live && !(j == i && sx == 0 && sy == 0 && sz == 0)) {
            const float4 pj = pos[j];
            const float ddx = pj.x + sx * box.x - pi.x, ddy = pj.y + sy * box.y - pi.y, ddz = pj.z + sz * box.z - pi.z;
            hit = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz)) < rl2;
          }
          const unsigned ball = __ballot_sync(0xffffffffu, hit);
          if (FILL && hit) {
            const long sl = slot + __popc(ball & below);
            if (sl < cap) {
              nidx[sl] = j;
              ntype_e[sl] = species[j];
              edge_i[sl] = i;
              shift[sl] = make_char4(sx, sy, sz, 0);
            }
          }
          slot += __popc(ball);
        }
  }
  if (!FILL && lane == 0) num_neigh[i] = static_cast<int>(slot);
}

// Wrap positions into the periodic box (done before each neighbour build; positions
// then move continuously until the next build, so stored image shifts stay valid).
__global__ void k_wrap(int N, double3 box, int3 periodic, double* __restrict__ pos) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  const double L[3] = {box.x, box.y, box.z};
  const int per[3] = {periodic.x, periodic.y, periodic.z};
  for (int d = 0; d < 3; ++d)
    if (per[d]) pos[3 * a + d] -= L[d] * floor(pos[3 * a + d] / L[d]);
}

// rev[e] = index of the reverse edge (j -> i, -shift) of e = (i -> j, shift); -1 if absent.
// One block per centre atom i, its warps taking every fourth edge: for each edge the
// lanes scan j's list 32 entries at a time (the first match in list order, as a
// sequential scan would find).
__global__ void k_reverse_edges(int N, const int* __restrict__ first, const int* __restrict__ nidx,
                                const char4* __restrict__ shift, int* __restrict__ rev) {
  const int i = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  if (i >= N) return;
  for (int e = first[i] + warp; e < first[i + 1]; e += nwarp) {
    const int j = nidx[e];
    const char4 sh = shift[e];
    const int w1 = first[j + 1];
    int found = -1;
    for (int w0 = first[j]; w0 < w1 && found < 0; w0 += 32) {
      const int w = w0 + lane;
      bool match = false;
      if (w < w1) {
        const char4 t = shift[w];
        match = nidx[w] == i && t.x == -sh.x && t.y == -sh.y && t.z == -sh.z;
      }
      const unsigned ball = __ballot_sync(0xffffffffu, match);
      if (ball) found = w0 + __ffs(ball) - 1;
    }
    if (lane == 0) rev[e] = found;
  }
}

// rev[e] for a cell-list build: the reverse of e = (i -> j, shift) lies in j's segment for
// the neighbour cell at the negated cell offset (cellseg), a few entries, scanned in order
// (the first match, as k_reverse_edges finds).  One thread per edge.
__global__ void k_reverse_edges_cells(long cap, int N, const int* __restrict__ first, const int* __restrict__ nidx,
                                      const int* __restrict__ edge_i, const char4* __restrict__ shift,
                                      const int* __restrict__ cell, int3 nc, const int* __restrict__ cellseg,
                                      int* __restrict__ rev) {
  const long E = first[N];
  for (long e = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; e < E && e < cap;
       e += static_cast<long>(gridDim.x) * blockDim.x) {
    const int i = edge_i[e], j = nidx[e];
    const char4 sh = shift[e];
    const int ci = cell[i], cj = cell[j];
    // offset of j's cell from i's in i's search: cell(j) + shift * nc - cell(i), each in [-1, 1]
    const int ox = (cj / (nc.z * nc.y)) + sh.x * nc.x - ci / (nc.z * nc.y);
    const int oy = (cj / nc.z) % nc.y + sh.y * nc.y - (ci / nc.z) % nc.y;
    const int oz = cj % nc.z + sh.z * nc.z - ci % nc.z;
    int found = -1;
    if (ox >= -1 && ox <= 1 && oy >= -1 && oy <= 1 && oz >= -1 && oz <= 1) {
      const int k = ((1 - ox) * 3 + (1 - oy)) * 3 + (1 - oz);  // in j's search the offset is negated
      const int w1 = cellseg[28L * j + k + 1];
      for (int w = cellseg[28L * j + k]; w < w1; ++w) {
        const char4 t = shift[w];
        if (nidx[w] == i && t.x == -sh.x && t.y == -sh.y && t.z == -sh.z) {
          found = w;
          break;
        }
      }
    }
    rev[e] = found;
  }
}

// xyz_e = x_j + shift_e * box - x_i, r_e = |xyz_e|
__global__ void k_edge_geometry(long cap, int N, const int* __restrict__ first, const double* __restrict__ pos,
                                double3 box, const int* __restrict__ nidx, const int* __restrict__ edge_i,
                                const char4* __restrict__ shift, double* __restrict__ xyz, double* __restrict__ r) {
  pdl_begin();
  const long e = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x;
  const long E = first[N] < cap ? first[N] : cap;
  if (e >= E) return;
  const int i = edge_i[e], j = nidx[e];
  const char4 s = shift[e];
  const double dx = pos[3 * j] + s.x * box.x - pos[3 * i];
  const double dy = pos[3 * j + 1] + s.y * box.y - pos[3 * i + 1];
  const double dz = pos[3 * j + 2] + s.z * box.z - pos[3 * i + 2];
  xyz[3 * e] = dx;
  xyz[3 * e + 1] = dy;
  xyz[3 * e + 2] = dz;
  r[e] = sqrt(dx * dx + dy * dy + dz * dz);
}

// velocity Verlet units: positions A, velocities A/fs, forces eV/A, masses amu, dt fs
constexpr double kAccel = 9.648533212331e-3;  // (eV/A)/amu in A/fs^2

// The in-cut-off edges of a skin list at the current positions, packed to the front of
// each centre atom's segment: one warp per atom, ballot ranks (list order kept,
// deterministic).  Atom a's packed edges are [first[a], last[a]) of the packed arrays;
// emap maps a packed edge to its skin-list index and pinv a skin-list edge to its packed
// index (-1 at or beyond r_cut).  The skin list's own geometry and forces are not
// written: only a state read-out needs them (launch_edge_geometry and the scatter below).
__global__ void k_edge_geometry_packed(int N, const int* __restrict__ first, const double* __restrict__ pos,
                                       double3 box, const int* __restrict__ nidx, const int* __restrict__ ntype_e,
                                       const char4* __restrict__ shift, double r_cut, int* __restrict__ pinv,
                                       int* __restrict__ last, int* __restrict__ emap, int* __restrict__ nidx_p,
                                       int* __restrict__ ntype_p, double* __restrict__ xyz_p, double* __restrict__ r_p) {
  pdl_begin();
  const int a = static_cast<int>((static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (a >= N) return;
  const int e0 = first[a], e1 = first[a + 1];
  const double px = pos[3 * a], py = pos[3 * a + 1], pz = pos[3 * a + 2];
  const float r_cut_f = static_cast<float>(r_cut);
  int count = 0;
  for (int base = e0; base < e1; base += 32) {
    const int e = base + lane;
    bool active = false;
    double dx = 0.0, dy = 0.0, dz = 0.0, re = 0.0;
    int j = 0;
    if (e < e1) {
      j = nidx[e];
      const char4 sh = shift[e];
      dx = pos[3 * j] + sh.x * box.x - px;
      dy = pos[3 * j + 1] + sh.y * box.y - py;
      dz = pos[3 * j + 2] + sh.z * box.z - pz;
      // the length in float32 (the evaluator reads r as a float; float64 arithmetic runs
      // on this part's slow float64 pipe)
      const float fx = static_cast<float>(dx), fy = static_cast<float>(dy), fz = static_cast<float>(dz);
      const float rf = sqrtf(fmaf(fx, fx, fmaf(fy, fy, fz * fz)));
      re = rf;
      active = rf < r_cut_f;
    }
    const unsigned ball = __ballot_sync(0xffffffffu, active);
    const int q = e0 + count + __popc(ball & ((1u << lane) - 1u));
    if (e < e1) pinv[e] = active ? q : -1;
    if (active) {
      emap[q] = e;
      nidx_p[q] = j;
      ntype_p[q] = ntype_e[e];
      xyz_p[3 * static_cast<long>(q)] = dx;
      xyz_p[3 * static_cast<long>(q) + 1] = dy;
      xyz_p[3 * static_cast<long>(q) + 2] = dz;
      r_p[q] = re;
    }
    count += __popc(ball);
  }
  if (lane == 0) last[a] = e0 + count;
}

// F_a = sum over a's packed edges q of (f[q'] - f[q]), q' the packed reverse edge
// pinv[rev[emap[q]]] (the reverse vector is the negated one up to the rounding of a
// periodic image shift, so only an edge within rounding of r_cut, where the forces
// vanish, can lack a packed reverse: it then adds nothing); one warp per atom, fixed lane
// assignment and reduction tree (deterministic).  With dt > 0 also the second
// velocity-Verlet half step of atom a, as k_vv_second.
__global__ void k_atom_forces_packed(int N, const int* __restrict__ first, const int* __restrict__ last,
                                     const int* __restrict__ emap, const int* __restrict__ rev,
                                     const int* __restrict__ pinv, const double* __restrict__ f,
                                     double* __restrict__ F, double dt, const double* __restrict__ inv_m,
                                     double* __restrict__ v) {
  pdl_begin();
  const int a = static_cast<int>((static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (a >= N) return;
  double s[3] = {0.0, 0.0, 0.0};
  for (int q = first[a] + lane; q < last[a]; q += 32) {
    const int er = rev[emap[q]];
    const int qr = er >= 0 ? pinv[er] : -1;
    for (int c = 0; c < 3; ++c)
      s[c] += (qr >= 0 ? f[3 * static_cast<long>(qr) + c] : 0.0) - f[3 * static_cast<long>(q) + c];
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int c = 0; c < 3; ++c) s[c] += __shfl_xor_sync(0xffffffffu, s[c], o);
  if (lane == 0) {
    for (int c = 0; c < 3; ++c) F[3 * a + c] = s[c];
    if (dt > 0.0) {
      const double h = 0.5 * dt * kAccel * inv_m[a];
      for (int c = 0; c < 3; ++c) v[3 * a + c] += h * s[c];
    }
  }
}

// skin-list forces of the packed edges: f_skin[emap[e]] = f_p[e]; one warp per atom
__global__ void k_scatter_packed_forces(int N, const int* __restrict__ first, const int* __restrict__ last,
                                        const int* __restrict__ emap, const double* __restrict__ f_p,
                                        double* __restrict__ f_skin) {
  pdl_begin();
  const int a = static_cast<int>((static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (a >= N) return;
  for (int e = first[a] + lane; e < last[a]; e += 32) {
    const long q = emap[e];
    for (int c = 0; c < 3; ++c) f_skin[3 * q + c] = f_p[3 * static_cast<long>(e) + c];
  }
}

// F_a = sum_{e in out(a)} (f[rev e] - f[e]); one thread per atom, no atomics
__global__ void k_atom_forces(int N, const int* __restrict__ first, const int* __restrict__ rev,
                              const double* __restrict__ f, double* __restrict__ F) {
  pdl_begin();
  // one warp per atom; fixed lane assignment and reduction tree: deterministic
  const int a = static_cast<int>((static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (a >= N) return;
  double s[3] = {0.0, 0.0, 0.0};
  for (int e = first[a] + lane; e < first[a + 1]; e += 32) {
    const int q = rev[e];
    for (int c = 0; c < 3; ++c) s[c] += (q >= 0 ? f[3 * static_cast<long>(q) + c] : 0.0) - f[3 * static_cast<long>(e) + c];
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int c = 0; c < 3; ++c) s[c] += __shfl_xor_sync(0xffffffffu, s[c], o);
  if (lane == 0)
    for (int c = 0; c < 3; ++c) F[3 * a + c] = s[c];
}

// Deterministic float64 reduction of the energy (slot 0) and the 9 virial
// components W_ab = sum_e xyz_e,a f_e,b (slots 1..9): per-block partials, then one
// block sums the partials in a fixed order.
__global__ void k_reduce_partials(int N, const int* __restrict__ first, const double* __restrict__ energies,
                                  const double* __restrict__ xyz, const double* __restrict__ f,
                                  double* __restrict__ partial) {
  __shared__ double sh[10][256];
  const long E = first[N];
  CompSum acc[10];
  const long stride = static_cast<long>(gridDim.x) * blockDim.x;
  for (long e = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x; e < E; e += stride)
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) acc[1 + 3 * a + b].add(xyz[3 * e + a] * f[3 * e + b]);
  for (long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) acc[0].add(energies[i]);
  for (int q = 0; q < 10; ++q) sh[q][threadIdx.x] = acc[q].value();
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 10; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 10) partial[blockIdx.x * 10 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_reduce_final(int nblocks, const double* __restrict__ partial, double* __restrict__ out) {
  if (threadIdx.x < 10) {
    CompSum s;
    for (int b = 0; b < nblocks; ++b) s.add(partial[b * 10 + threadIdx.x]);
    out[threadIdx.x] = s.value();
  }
}

// velocity Verlet halves

__global__ void k_vv_first(int N, double dt, const double* __restrict__ F, const double* __restrict__ inv_m,
                           double* __restrict__ v, double* __restrict__ x) {
  pdl_begin();
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  const double h = 0.5 * dt * kAccel * inv_m[a];
  for (int c = 0; c < 3; ++c) {
    v[3 * a + c] += h * F[3 * a + c];
    x[3 * a + c] += dt * v[3 * a + c];
  }
}

__global__ void k_vv_second(int N, double dt, const double* __restrict__ F, const double* __restrict__ inv_m,
                            double* __restrict__ v) {
  pdl_begin();
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  const double h = 0.5 * dt * kAccel * inv_m[a];
  for (int c = 0; c < 3; ++c) v[3 * a + c] += h * F[3 * a + c];
}

// ---- launchers ----
// atoms binned (atomic fill into cell_tmp), then each cell's atoms sorted by index into
// cell_atoms: the list order does not depend on the order of the atomics
void launch_cell_list(const double* pos, int N, double3 box, int3 nc, int* cell, int* cell_count, int* cell_start,
                      int* cell_fill, int* cell_tmp, int* cell_atoms, cudaStream_t s) {
  const int ncell = nc.x * nc.y * nc.z;
  cudaMemsetAsync(cell_count, 0, sizeof(int) * ncell, s);
  cudaMemsetAsync(cell_fill, 0, sizeof(int) * ncell, s);
  k_cell_assign<<<ceil_div(N, 256), 256, 0, s>>>(pos, N, box, nc, cell, cell_count);
  launch_scan_first(cell_count, ncell, cell_start, s);
  k_cell_fill<<<ceil_div(N, 256), 256, 0, s>>>(cell, N, cell_start, cell_fill, cell_tmp);
  k_cell_sort<<<ceil_div(ncell, 4), 128, 0, s>>>(ncell, cell_start, cell_tmp, cell_atoms);  // one warp per cell
}

// Spatial renumbering of the MD atoms: slot k takes atom perm[k] (the cell list's order),
// gathered into tmp_d [pos 3N | vel 3N | F 3N | inv_m N] and tmp_i [species N | orig N];
// the caller copies them back, so that device pointers (and captured graphs) stay valid.
__global__ void k_permute_atoms(int N, const int* __restrict__ perm, const double* __restrict__ pos,
                                const double* __restrict__ vel, const double* __restrict__ F,
                                const double* __restrict__ inv_m, const int* __restrict__ species,
                                const int* __restrict__ orig, double* __restrict__ tmp_d, int* __restrict__ tmp_i) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  const int a = perm[k];
  const long n3 = 3L * N;
  for (int c = 0; c < 3; ++c) {
    tmp_d[3L * k + c] = pos[3L * a + c];
    tmp_d[n3 + 3L * k + c] = vel[3L * a + c];
    tmp_d[2 * n3 + 3L * k + c] = F[3L * a + c];
  }
  tmp_d[3 * n3 + k] = inv_m[a];
  tmp_i[k] = species[a];
  tmp_i[N + k] = orig[a];
}

void launch_permute_atoms(int N, const int* perm, const double* pos, const double* vel, const double* F,
                          const double* inv_m, const int* species, const int* orig, double* tmp_d, int* tmp_i,
                          cudaStream_t s) {
  if (N <= 0) return;
  k_permute_atoms<<<ceil_div(N, 256), 256, 0, s>>>(N, perm, pos, vel, F, inv_m, species, orig, tmp_d, tmp_i);
}

void launch_neigh_pass(bool fill, bool brute, const double* pos_d, float4* pos, const int* species, int N,
                       double3 box_d, int3 nc, int3 periodic, int3 nimg, double rl, const int* cell,
                       const int* cell_start, const int* cell_atoms, const int* seg_of, const int* seg_first,
                       int* num_neigh, const int* first, int* nidx, int* ntype_e, int* edge_i, char4* shift, long cap,
                       cudaStream_t s, int* cellseg) {
  if (N <= 0) return;
  if (!fill) k_pos_to_float<<<ceil_div(N, 256), 256, 0, s>>>(N, pos_d, pos);  // the fill pass reuses it
  const float rl2 = static_cast<float>(rl * rl);
  const float3 box = make_float3(static_cast<float>(box_d.x), static_cast<float>(box_d.y), static_cast<float>(box_d.z));
  const int g = ceil_div(N, 4);  // 128-thread blocks, one warp per atom
  if (brute || seg_of) {
    if (fill)
      k_neigh_brute<true><<<g, 128, 0, s>>>(pos, species, N, box, nimg, rl2, seg_of, seg_first, num_neigh, first,
                                            nidx, ntype_e, edge_i, shift, cap);
    else
      k_neigh_brute<false><<<g, 128, 0, s>>>(pos, species, N, box, nimg, rl2, seg_of, seg_first, num_neigh, first,
                                             nidx, ntype_e, edge_i, shift, cap);
  } else {
    if (fill)
      k_neigh_cells<true><<<g, 128, 0, s>>>(pos, species, N, box, nc, periodic, rl2, cell, cell_start, cell_atoms,
                                            num_neigh, first, nidx, ntype_e, edge_i, shift, cap, cellseg);
    else
      k_neigh_cells<false><<<g, 128, 0, s>>>(pos, species, N, box, nc, periodic, rl2, cell, cell_start, cell_atoms,
                                             num_neigh, first, nidx, ntype_e, edge_i, shift, cap, nullptr);
  }
}

void launch_wrap(int N, double3 box, int3 periodic, double* pos, cudaStream_t s) {
  if (N > 0) k_wrap<<<ceil_div(N, 128), 128, 0, s>>>(N, box, periodic, pos);
}

void launch_reverse_edges(long cap, int N, const int* first, const int* nidx, const int* edge_i, const char4* shift,
                          int* rev, cudaStream_t s) {
  if (cap > 0 && N > 0) k_reverse_edges<<<N, 128, 0, s>>>(N, first, nidx, shift, rev);  // block per atom
}

void launch_reverse_edges_cells(long cap, int N, const int* first, const int* nidx, const int* edge_i,
                                const char4* shift, const int* cell, int3 nc, const int* cellseg, int* rev,
                                cudaStream_t s) {
  if (cap > 0 && N > 0)
    k_reverse_edges_cells<<<static_cast<int>(std::min<long>(ceil_div(cap, 256), 152L * 16)), 256, 0, s>>>(
        cap, N, first, nidx, edge_i, shift, cell, nc, cellseg, rev);
}

void launch_edge_geometry(long cap, int N, const int* first, const double* pos, double3 box, const int* nidx,
                          const int* edge_i, const char4* shift, double* xyz, double* r, cudaStream_t s) {
  if (cap > 0)
    launch_pdl(k_edge_geometry, ceil_div(cap, 256), 256, 0, s, cap, N, first, pos, box, nidx, edge_i, shift, xyz, r);
}

void launch_edge_geometry_packed(int N, const int* first, const double* pos, double3 box, const int* nidx,
                                 const int* ntype_e, const char4* shift, double r_cut, int* pinv, int* last, int* emap,
                                 int* nidx_p, int* ntype_p, double* xyz_p, double* r_p, cudaStream_t s) {
  if (N > 0)
    launch_pdl(k_edge_geometry_packed, ceil_div(N, 4), 128, 0, s, N, first, pos, box, nidx, ntype_e, shift, r_cut,
               pinv, last, emap, nidx_p, ntype_p, xyz_p, r_p);
}

void launch_atom_forces_packed(int N, const int* first, const int* last, const int* emap, const int* rev,
                               const int* pinv, const double* f_p, double* F, double dt, const double* inv_m, double* v,
                               cudaStream_t s) {
  if (N > 0)
    launch_pdl(k_atom_forces_packed, ceil_div(N, 4), 128, 0, s, N, first, last, emap, rev, pinv, f_p, F, dt, inv_m,
               v);  // one warp per atom
}

void launch_scatter_packed_forces(int N, const int* first, const int* last, const int* emap, const double* f_p,
                                  double* f_skin, cudaStream_t s) {
  if (N > 0) launch_pdl(k_scatter_packed_forces, ceil_div(N, 4), 128, 0, s, N, first, last, emap, f_p, f_skin);
}

void launch_atom_forces(int N, const int* first, const int* rev, const double* f, double* F, cudaStream_t s) {
  if (N > 0) launch_pdl(k_atom_forces, ceil_div(N, 4), 128, 0, s, N, first, rev, f, F);  // one warp per atom
}

void launch_reduce(int N, const int* first, const double* energies, const double* xyz, const double* f,
                   double* partial, int nblocks, double* out, cudaStream_t s) {
  k_reduce_partials<<<nblocks, 256, 0, s>>>(N, first, energies, xyz, f, partial);
  k_reduce_final<<<1, 32, 0, s>>>(nblocks, partial, out);
}

void launch_vv_first(int N, double dt, const double* F, const double* inv_m, double* v, double* x, cudaStream_t s) {
  if (N > 0) launch_pdl(k_vv_first, ceil_div(N, 128), 128, 0, s, N, dt, F, inv_m, v, x);
}

void launch_vv_second(int N, double dt, const double* F, const double* inv_m, double* v, cudaStream_t s) {
  if (N > 0) launch_pdl(k_vv_second, ceil_div(N, 128), 128, 0, s, N, dt, F, inv_m, v);
}

}  // namespace smx
