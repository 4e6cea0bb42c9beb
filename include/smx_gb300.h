/* smx_gb300.h — C ABI of the GB300-native MACE energy/force engine.
 *
 * Drop-in for libsymmetrix's evaluator path.  Each entry point names the
 * reference interface it replaces (paths are within the symmetrix repository):
 *
 *   smx_create / smx_destroy        MACE::MACE(std::string filename)
 *                                   (libsymmetrix/source/mace.hpp:16, mace.cpp:12-15)
 *   smx_compute_node_energies_forces
 *                                   MACE::compute_node_energies_forces
 *                                   (libsymmetrix/source/mace.hpp:29-35, mace.cpp:17-64);
 *                                   the results the reference leaves in the members
 *                                   node_energies / node_forces are written to caller
 *                                   buffers instead
 *   smx_compute_halo                the stage calls of the pair style's
 *                                   no-MPI-message-passing mode, layer 0 over local and
 *                                   halo nodes and layer 1 over the local ones
 *                                   (pair_symmetrix/pair_symmetrix_mace.cpp:672-698)
 *   smx_compute_node_energies_forces_device
 *                                   the same call on device-resident arrays, as the Kokkos
 *                                   pair style passes them (pair_symmetrix/
 *                                   pair_symmetrix_mace_kokkos.cpp:390-394)
 *   smx_sync                        no counterpart: the reference's calls are synchronous;
 *                                   it reports a timed-out device wait after the
 *                                   device-pointer call
 *   smx_num_elements, smx_num_channels, smx_r_cut, smx_l_max, smx_L_max, smx_num_LM,
 *   smx_atomic_numbers, smx_has_zbl public fields of class MACE (mace.hpp:18-25, :38)
 *   smx_get_stage, smx_set_stage    the stage buffers the Python binding exposes read/write
 *                                   (symmetrix/source/cpp/mace.cpp:14-34)
 *   smx_run_stage                   the binding's per-stage calls compute_H1 / reverse_H1,
 *                                   compute_Phi1 / reverse_Phi1 (with compute_R1 and
 *                                   compute_Y, fused), compute_A1 / reverse_A1
 *                                   (symmetrix/source/cpp/mace.cpp:152-179;
 *                                   libsymmetrix/source/mace.cpp:397-679)
 *   smx_compute_atoms               what the callers do around the evaluator: neighbour list,
 *                                   evaluation, F_j += f_e / F_i -= f_e and the virial
 *                                   (Symmetrix.calculate, symmetrix_calc.py:72-102;
 *                                   PairSymmetrixMACE::compute_no_domain_decomposition,
 *                                   pair_symmetrix/pair_symmetrix_mace.cpp:242-372)
 *   smx_pair_*                      pair_style symmetrix/mace's compute() in its three modes
 *                                   on one rank (pair_symmetrix/pair_symmetrix_mace.cpp:
 *                                   64-77, :242-748)
 *   smx_md_*                        a GPU-resident velocity-Verlet loop with a skin neighbour
 *                                   list, the role LAMMPS `fix nve` plays around the pair
 *                                   style (pair_symmetrix/test/test_pair_symmetrix_mace.py:253)
 *
 * Conventions (identical to the reference):
 *   - edges are a full directed list grouped by centre node: node i owns edges
 *     [sum(num_neigh[:i]), sum(num_neigh[:i+1])); neigh_indices[e] = j;
 *   - xyz[3e..3e+2] = x_j - x_i (periodic image included), r[e] = |xyz[e]|, 0 < r < r_cut;
 *   - node_types / neigh_types index the model's atomic_numbers list;
 *   - node_forces[3e..3e+2] = -dE/dxyz[e] (a per-edge "partial force"); atomic forces
 *     are F_j += f_e, F_i -= f_e and the virial is sum_e xyz[e] (x) f_e.
 *
 * Errors are status codes (the reference throws C++ exceptions); smx_last_error()
 * returns the message of the last failing call on the calling thread.
 * An engine is not thread-safe (like the reference's MACE object): one caller at a time.
 */
#ifndef SMX_GB300_H
#define SMX_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SMX_OK 0
#define SMX_ERR_INVALID 1   /* bad argument or input outside the model's domain */
#define SMX_ERR_MODEL 2     /* model file missing, malformed or unsupported */
#define SMX_ERR_CUDA 3      /* CUDA runtime error (message has the CUDA error string) */
#define SMX_ERR_CAPACITY 4  /* a fixed-capacity buffer is too small for the request */
#define SMX_ERR_TIMEOUT 5   /* a bounded device-side wait gave up */

#define SMX_PRECISION_FP32 0 /* plain form: float32 throughout, float64 outputs */
#define SMX_PRECISION_BF16 1 /* precision form: channel-mixing GEMMs in bf16 on the tensor cores
                                (tcgen05, float32 accumulation); everything else as the plain form */

typedef struct smx_engine smx_engine;

/* Parse a model (JSON, or a cache file) once and write it as a binary model cache:
 * the packed device-layout tables in one file that smx_create then loads in place of
 * the JSON without parsing it.  Host only (no GPU).  No counterpart in the reference,
 * whose MACE(std::string) parses the JSON on every construction
 * (libsymmetrix/source/mace.cpp:12-15, :905-1030). */
int smx_save_model_cache(const char* model_path, const char* cache_path);

/* Load a libsymmetrix JSON model (or a model cache written by smx_save_model_cache)
 * onto CUDA device `device`.  NULL on failure. */
smx_engine* smx_create(const char* model_path, int precision, int device);
void smx_destroy(smx_engine* eng);
const char* smx_last_error(void);

int smx_num_elements(const smx_engine* eng);
int smx_num_channels(const smx_engine* eng);
double smx_r_cut(const smx_engine* eng);
int smx_l_max(const smx_engine* eng);
int smx_L_max(const smx_engine* eng);
int smx_num_LM(const smx_engine* eng);
/* 1 when the model adds the ZBL pair repulsion (MACE::has_zbl, mace.hpp:38), else 0. */
int smx_has_zbl(const smx_engine* eng);
/* Copies up to cap atomic numbers (none when out is NULL); returns the number of species. */
int smx_atomic_numbers(const smx_engine* eng, int* out, int cap);

/* Host arrays in, host arrays out (node_energies[num_nodes], node_forces[3*num_edges]).
 * Inputs are validated (index ranges, 0 < r < r_cut, sum(num_neigh) == num_edges). */
int smx_compute_node_energies_forces(smx_engine* eng, int num_nodes, const int* node_types, const int* num_neigh,
                                     const int* neigh_indices, const int* neigh_types, long num_edges,
                                     const double* xyz, const double* r, double* node_energies,
                                     double* node_forces);

/* The evaluation the pair style's no-MPI-message-passing mode runs stage by stage
 * (pair_symmetrix/pair_symmetrix_mace.cpp:672-698): layer 0 (A0, M0, H1 and their
 * adjoints, density factor included) over all num_nodes nodes; ZBL, layer 1, the
 * readouts and their adjoints over the first num_local_nodes only.  The trailing nodes
 * are a halo: their H1 rows are read by the local nodes' layer-1 edges and the
 * H1_adj those edges scatter to them flows back through layer 0 into the halo's own
 * edges.  Arrays and checks as smx_compute_node_energies_forces over num_nodes nodes
 * (a halo node's neigh_indices must be in range but are never read); node_energies
 * receives num_local_nodes values, node_forces one triple per edge of every node.
 * num_local_nodes == num_nodes is smx_compute_node_energies_forces. */
int smx_compute_halo(smx_engine* eng, int num_local_nodes, int num_nodes, const int* node_types,
                     const int* num_neigh, const int* neigh_indices, const int* neigh_types, long num_edges,
                     const double* xyz, const double* r, double* node_energies, double* node_forces);

/* Same, with every pointer in device memory of the engine's device; runs on
 * `stream` (a cudaStream_t, or NULL for the engine's own stream) and returns
 * without synchronising.  Inputs are not validated; edges with r >= r_cut
 * contribute nothing.  A bounded device-side wait that gave up is reported by
 * the next smx_sync. */
int smx_compute_node_energies_forces_device(smx_engine* eng, int num_nodes, const int* node_types,
                                            const int* num_neigh, const int* neigh_indices, const int* neigh_types,
                                            long num_edges, const double* xyz, const double* r,
                                            double* node_energies, double* node_forces, void* stream);

/* Waits for `stream` (a cudaStream_t, or NULL for the engine's own stream) and
 * returns SMX_ERR_TIMEOUT if a bounded device-side wait of the engine gave up since
 * the last check (the results of that work are invalid), else SMX_OK.  The
 * host-pointer calls and the MD sync/state calls make this check themselves. */
int smx_sync(smx_engine* eng, void* stream);

/* Copies the last call's stage buffer `name` (A0, M0, H1, Phi1, A1, M1, H2, A0_adj,
 * M0_adj, H1_adj, Phi1_adj, A1_adj, M1_adj, H2_adj; reference layouts, see
 * libsymmetrix/source/mace.hpp) as float64, after waiting for the device.  Returns its
 * length (0 after an empty evaluation); -1 for an unknown name; -2 when the stage is
 * not available: no evaluation has run yet, or the BF16 form skipped the float32 rows
 * of M0, Phi1 or A1_adj (its tensor-core GEMMs read bf16 split rows instead), which it
 * writes only after smx_set_option(eng, "keep_stages", 1); -3 on a CUDA error.
 * smx_last_error() says which. */
long smx_get_stage(smx_engine* eng, const char* name, double* out, long cap);
/* "node_energies" (N) and "node_forces" (3E, the last host-pointer call's or stage call's
 * edges) are read the same way, as stored (float64). */

/* Writes stage buffer `name` (M0, H1, Phi1, A1, M0_adj, H1_adj, Phi1_adj, A1_adj: float32,
 * rounded from the float64 values; node_forces: float64) of the node count of the last
 * evaluation or stage call, in the layout smx_get_stage reads; n must be that stage's
 * length.  Returns n, or minus an SMX_ERR_* code.  The reference binding's buffers are
 * read-write attributes (symmetrix/source/cpp/mace.cpp:14-34). */
long smx_set_stage(smx_engine* eng, const char* name, const double* values, long n);

/* Runs one stage on the engine's stage buffers (what the reference's per-stage calls
 * do on its members, libsymmetrix/source/mace.cpp:397-679):
 *   "compute_H1"   H1 = M0 . H1_weights[L]              (mace.cpp:397-423)
 *   "reverse_H1"   M0_adj = H1_adj . H1_weights[L]^T      (mace.cpp:425-451)
 *   "compute_A1"   A1 = Phi1 . A1_weights[l]             (mace.cpp:607-642)
 *   "reverse_A1"   Phi1_adj = A1_adj . A1_weights[l]^T   (mace.cpp:644-679)
 *     node stages: num_nodes must be the last evaluation's; the edge arguments are
 *     ignored (NULL / 0);
 *   "compute_Phi1" R1, Y and Phi1 from H1 on the given edges (mace.cpp:92-148, 453-502)
 *   "reverse_Phi1" on the given edges: H1_adj += the Phi1_adj-contracted terms and
 *                  node_forces += -dPhi1/dxyz . Phi1_adj (mace.cpp:504-605); the flags
 *                  SMX_STAGE_ZERO_DXYZ / SMX_STAGE_ZERO_H1_ADJ start either from zero,
 *                  as the reference's zero_dxyz / zero_H1_adj arguments do.
 *     edge stages: the edge list is copied and checked as by the host-pointer call; a
 *     node count other than the last call's starts the buffers from zero.
 * The GEMMs run on the float32 SIMT kernel in both precision forms; the layer-1 stages
 * leave out the density normalisation (compute_A1_scaled / reverse_A1_scaled, fused
 * into the node tail with compute_M1, compute_H2, compute_readouts and their reverses,
 * which, like the layer-0 stages compute_Y, compute_R0, compute_A0(_scaled) and
 * compute_M0 and their reverses, run only inside a full evaluation).  Results are
 * read with smx_get_stage. */
#define SMX_STAGE_ZERO_DXYZ 1
#define SMX_STAGE_ZERO_H1_ADJ 2
int smx_run_stage(smx_engine* eng, const char* stage, int num_nodes, const int* node_types, const int* num_neigh,
                  const int* neigh_indices, const int* neigh_types, long num_edges, const double* xyz,
                  const double* r, int flags);

/* Options: "keep_stages" (the BF16 form also writes the float32 M0, Phi1 and A1_adj
 * rows for smx_get_stage), "profile" (record CUDA
 * events between the kernels of every evaluation); "autotune" (1, the default: the
 * first evaluation outside a stream capture picks, per per-atom kernel, one block per
 * atom or a persistent grid of resident blocks claiming atoms from a counter, and for
 * L_max = 2 models of 64 or more channels one or two channel slices per node in the
 * layer-1 kernels, by timing whole passes; in the BF16 form it times the candidate N-tile
 * widths and TMA ring depths of each tensor-core GEMM group on its own operands; setting
 * it again re-tunes; 0 keeps the defaults: one block per atom, two channel slices,
 * default GEMM schedule);
 * "persistent" (-1: tuned as above, 0: one block per atom, 1: persistent grids);
 * "species_order" (-1, the default: the edge kernels take the centre atoms sorted by
 * species when a layer's spline table exceeds 64 MB, so the rows in use stay in L2;
 * 0: input order; 1: always sorted; results do not depend on it);
 * "cg_padded" (1, the default: the layer-1 Clebsch-Gordan contractions read tables padded
 * to a fixed number of terms per row, with independent loads; 0: the compressed rows);
 * "pdl" (1, the default: the chained kernels of an evaluation and of an MD step are
 * launched with programmatic dependent launch, each waiting for its predecessor at its
 * first instruction; 0: plain launches; process-wide, read by later launches and graph
 * captures); BF16 form: "tc_terms" (1, 2 or 3 bf16 split products of the GEMMs: x_hi W_hi,
 * + x_hi W_lo, + x_lo W_hi; default 3; set before the first evaluation);
 * "test_gemm_timeout" (n in [0, 16]: a test of the timeout path, the next n tensor-core
 * GEMM launches issue no load so that their bounded wait gives up after 2 ms with
 * nothing in flight; the call that ran them, or smx_sync
 * after a device-pointer call, returns SMX_ERR_TIMEOUT and the results are invalid).
 * No counterpart in the reference (its MACE object has no options). */
int smx_set_option(smx_engine* eng, const char* key, long value);
/* Read an option or a tuned schedule entry ("tc_nt_<G>": the N-tile width, 0 when each
 * GEMM of the group is one N-tile of its whole width; "tc_stages_<G>",
 * "tc_tuned_ns_<G>" for G in H1, A1, Phi1_adj, M0_adj; "persistent": bit k set when
 * per-atom kernel k (layer0_fwd, contract0_rev, layer0_rev, layer1_fwd, layer1_rev,
 * node_tail) runs as a persistent grid; "species_order": 1 when the sorted order is in
 * effect; "poly_canon": 1 when the model's symmetric-contraction monomials are the
 * canonical sets and run as generated code, 0 for the data-driven path; "l2_split": channel
 * slices per node of the L_max = 2 layer-1 kernels, 1 or 2, picked by the autotuner); -1 if
 * unknown. */
long smx_get_option(const smx_engine* eng, const char* key);

/* The engine's own CUDA stream (a cudaStream_t): host-pointer calls and the MD driver
 * run on it, so callers can order their work or record CUDA events against it. */
void* smx_engine_stream(smx_engine* eng);

/* With "profile" on: device time (ms) of each stage of the last evaluation, in launch
 * order: layer0_fwd, gemm_H1, layer1_fwd, gemm_A1, node_tail, gemm_Phi1_adj,
 * layer1_rev, gemm_M0_adj, layer0_rev.  Returns the number of stages (0 if profiling
 * is off).  Blocks until the last evaluation has finished. */
int smx_stage_times(smx_engine* eng, double* out_ms, int cap);

/* Atom-level evaluation: positions[3n] (A), species[n] (indices into atomic_numbers),
 * box_lengths[3] of an orthorhombic periodic cell (NULL = non-periodic).  Builds the
 * full neighbour list (r < r_cut) on the GPU, evaluates, and returns the total energy,
 * optionally node_energies[n], atomic forces[3n] and the virial[9] W_ab = sum_e xyz_a f_b
 * (row-major, float64).  Host pointers; synchronous. */
int smx_compute_atoms(smx_engine* eng, int n_atoms, const double* positions, const int* species,
                      const double* box_lengths, double* energy, double* node_energies, double* forces,
                      double* virial);

/* Velocity-Verlet MD on the GPU.  Units: A, fs, amu, eV.  velocities may be NULL (zero).
 * The neighbour list (r_cut + skin) is rebuilt every rebuild_every steps; the steps in
 * between run as one captured CUDA graph.  NULL on failure (see smx_last_error). */
typedef struct smx_md smx_md;
smx_md* smx_md_create(smx_engine* eng, int n_atoms, const double* positions, const double* velocities,
                      const int* species, const double* masses, const double* box_lengths, double dt_fs, double skin,
                      int rebuild_every);
/* Enqueue `steps` steps on the engine's stream; returns without waiting for them
 * except at neighbour-list rebuilds. */
int smx_md_run(smx_md* md, int steps);
int smx_md_sync(smx_md* md);
/* Current state (any pointer may be NULL): positions[3n], velocities[3n] (A/fs),
 * forces[3n], potential energy, virial[9], step count.  Synchronous. */
int smx_md_state(smx_md* md, double* positions, double* velocities, double* forces, double* potential_energy,
                 double* virial, long* step);
long smx_md_num_edges(smx_md* md);
void smx_md_destroy(smx_md* md);

/* Energy and virial of one evaluation, summed on the GPU without allocating anything.
 * No counterpart in the reference: it serves callers that may not call cudaMalloc
 * where they need the sum (device memory owned by another framework's pools, such as
 * a Kokkos pair style, or a fixed memory budget).  All pointers are device memory of
 * the current device: node_energies[num_nodes], xyz[3*num_edges],
 * node_forces[3*num_edges] (as returned by smx_compute_node_energies_forces_device),
 * out[10] = {sum of node energies, W_xx, W_xy, ..., W_zz} with W_ab = sum_e xyz_e,a f_e,b.
 * Scratch is a fixed 1.25 MiB device array inside the library (one float64 partial per
 * 4096 nodes/edges), so at most 67,108,864 nodes and at most 67,108,864 edges are
 * accepted; larger inputs return SMX_ERR_CAPACITY without launching.  The first call on
 * each device looks up that array's device address; make it before any stream capture.
 * That address belongs to the device's primary context: a process that resets the
 * device (cudaDeviceReset) must not call this entry point on it afterwards.  Every call on a
 * device shares that array (it keeps the last call's partial sums; nothing in it needs
 * to start at zero), so calls that overlap on the same GPU, e.g. on two streams, race:
 * serialise them.  Enqueued on `stream`
 * (a cudaStream_t, NULL = legacy default stream); returns without synchronising.
 * Results are bitwise reproducible. */
int smx_energy_virial_device_noalloc(int num_nodes, long num_edges, const double* node_energies, const double* xyz,
                                     const double* node_forces, double* out, void* stream);

/* ---- batching form: many independent non-periodic molecules ---------------
 * Molecule m holds atoms [mol_first[m], mol_first[m+1]) (mol_first[0] = 0,
 * mol_first[n_mol] = number of atoms).  One neighbour build, one launch per engine
 * stage for the whole batch; edges only join atoms of the same molecule, wherever
 * the molecules sit in space.  Per-molecule energies, per-atom energies and forces.
 * The reference evaluates one structure per MACE::compute_node_energies_forces call
 * (libsymmetrix/source/mace.cpp:17-64); this batches what its callers would loop over. */
int smx_compute_molecules(smx_engine* eng, int n_mol, const int* mol_first, const double* positions,
                          const int* species, double* mol_energies, double* node_energies, double* forces);
/* velocity-Verlet MD of such a batch (as smx_md_create with no box) */
smx_md* smx_md_create_molecules(smx_engine* eng, int n_mol, const int* mol_first, const double* positions,
                                const double* velocities, const int* species, const double* masses, double dt_fs,
                                double skin, int rebuild_every);

/* ---- LAMMPS pair-style adapter -------------------------------------------
 * One compute() of pair_style symmetrix/mace in its no-domain-decomposition mode:
 * replaces PairSymmetrixMACE::compute_no_domain_decomposition
 * (pair_symmetrix/pair_symmetrix_mace.cpp:242-372), with the same inputs taken
 * straight from LAMMPS: the full neighbour list (list->inum, ilist, numneigh,
 * firstneigh, NEIGHMASK), atom->x[0] (x[nall][3] of local and ghost atoms),
 * atom->type (1-based, nall), local_of[j] = atom->map(atom->tag[j]) and the
 * LAMMPS-type -> model-species map mace_types[ntypes] set by pair_coeff.  Edges are
 * the candidates with r < r_cut; results are ADDED like the reference: f[nall][3]
 * (F_i -= f_e, F_local_of[j] += f_e), *eng_vdwl (eflag_global), eatom[inum]
 * (eflag_atom, overwritten), virial[6] = xx yy zz xy xz yz of sum_e xyz (x) f_e
 * (vflag_global).  neigh_changed != 0 re-uploads the list topology, types and owners
 * (LAMMPS re-neighbouring); otherwise only x moves.  Filtering, evaluation and force
 * scatter run on the GPU; synchronous.  One adapter per engine; not thread-safe. */
typedef struct smx_pair smx_pair;
smx_pair* smx_pair_create(smx_engine* eng);
void smx_pair_destroy(smx_pair* pair);
int smx_pair_compute(smx_pair* pair, int inum, int nall, const int* ilist, const int* numneigh,
                     const int* const* firstneigh, int neighmask, int neigh_changed, const double* x,
                     const int* type, const int* local_of, const int* mace_types, int ntypes, int eflag_global,
                     int eflag_atom, int vflag_global, double* f, double* eng_vdwl, double* eatom, double* virial);

/* The pair style's three modes (PairSymmetrixMACE::settings, pair_symmetrix/
 * pair_symmetrix_mace.cpp:95-113, and compute, :64-77), as they run on one rank.
 *   SMX_PAIR_NO_DOMAIN_DECOMPOSITION  smx_pair_compute above (:242-372).
 *   SMX_PAIR_MPI_MESSAGE_PASSING      :376-547.  On one rank LAMMPS's forward exchange of
 *       H1 to the ghosts (:462-470) gives each ghost its owner's H1 and the reverse
 *       exchange of H1_adj (:487-489) adds each ghost's to its owner's, which is the
 *       ghost -> owner map local_of itself, so the evaluation is the first mode's; the
 *       force of a ghost neighbour stays on its ghost row (F_j += f_e) for LAMMPS's own
 *       reverse communication of forces.
 *   SMX_PAIR_NO_MPI_MESSAGE_PASSING   :551-748.  The nodes are the local atoms, then the
 *       ghosts within r_cut of a local atom in ascending index order (found on the GPU
 *       each call); layer 0 runs over all of them, ZBL, layer 1 and the readouts over the
 *       local ones (smx_compute_halo), and each edge's force lands on its two atoms,
 *       ghosts included.  Needs LAMMPS's ghost neighbour list (the reference requests
 *       REQ_FULL | REQ_GHOST and a communication cutoff of 2 r_cut + skin, :175-190):
 *       ilist holds inum local then gnum ghost entries, numneigh and firstneigh cover
 *       them all; local_of may be NULL.  A ghost node without a list is an error.
 * gnum is ignored by the first two modes; every other argument is smx_pair_compute's. */
#define SMX_PAIR_NO_DOMAIN_DECOMPOSITION 0
#define SMX_PAIR_MPI_MESSAGE_PASSING 1
#define SMX_PAIR_NO_MPI_MESSAGE_PASSING 2
int smx_pair_compute_mode(smx_pair* pair, int mode, int inum, int gnum, int nall, const int* ilist,
                          const int* numneigh, const int* const* firstneigh, int neighmask, int neigh_changed,
                          const double* x, const int* type, const int* local_of, const int* mace_types, int ntypes,
                          int eflag_global, int eflag_atom, int vflag_global, double* f, double* eng_vdwl,
                          double* eatom, double* virial);

#ifdef __cplusplus
}
#endif

#endif /* SMX_GB300_H */
