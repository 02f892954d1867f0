/*
 * refeff_fms.h -- C ABI of the GB300 (sm_103a) full-multiple-scattering path.
 *
 * This library replaces the real-space FMS hot path of refeff (a Rust port of
 * FEFF10): the per-energy G0 / T assembly and the dense complex solve that
 * crates/refeff-engine/src/fms.rs hands to refeff-core and refeff-linalg.
 * A Rust caller binds these entry points through a thin FFI crate; the
 * signatures use plain C types only (no CUDA or torch types).
 *
 * Conventions
 *  - Complex numbers are two consecutive doubles (re, im): refeff_complex128.
 *  - Arrays are column-major ("Fortran order"), exactly like the reference's
 *    ndarray `.f()` tables.  Indices are zero-based.
 *  - Every entry point returns a refeff_fms_status; 0 is success.  Nothing
 *    aborts or throws across the ABI.  refeff_fms_last_error() returns a
 *    human-readable message for the last failure on a context.
 *  - The caller owns every host buffer; the library owns device memory and
 *    streams inside the context and plan handles.  Handles are not
 *    thread-safe: use one context per host thread (the reference configures
 *    faer's parallelism process-wide, docs/EMBEDDING_ROADMAP.md:88-92).
 *  - Lengths are Angstrom, wave numbers Angstrom^-1, sigma^2 Angstrom^2
 *    (crates/refeff-core/src/fms/internals/geometry.rs:19-24).
 */
#ifndef REFEFF_FMS_H
#define REFEFF_FMS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define REFEFF_FMS_ABI_VERSION 1

typedef struct {
  double re;
  double im;
} refeff_complex128;

/* Status codes.  They map onto the reference error variants the FMS path can
 * raise: crates/refeff-core/src/fms/types.rs:832 (FmsError) and
 * crates/refeff-linalg/src/error.rs (LinalgError::SingularMatrix). */
typedef enum {
  REFEFF_FMS_OK = 0,
  REFEFF_FMS_ERR_INVALID_ARGUMENT = 1,       /* null pointer, bad count, bad enum */
  REFEFF_FMS_ERR_EMPTY_CLUSTER = 2,          /* FmsError::EmptyCluster */
  REFEFF_FMS_ERR_POTENTIAL_OUT_OF_RANGE = 3, /* FmsError::PotentialOutOfRange */
  REFEFF_FMS_ERR_MISSING_REPRESENTATIVE = 4, /* FmsError::MissingRepresentativePotential */
  REFEFF_FMS_ERR_INVALID_ANGULAR_LIMIT = 5,  /* FmsError::InvalidAngularLimit */
  REFEFF_FMS_ERR_NONFINITE_INPUT = 6,        /* NonFiniteWaveNumber / NonFinitePhaseShift / NonFiniteRho */
  REFEFF_FMS_ERR_NONFINITE_COORDINATE = 7,   /* FmsError::NonFiniteCoordinate */
  REFEFF_FMS_ERR_ZERO_RHO = 8,               /* FmsError::ZeroRho */
  REFEFF_FMS_ERR_SINGULAR_MATRIX = 9,        /* LinalgError::SingularMatrix { pivot } */
  REFEFF_FMS_ERR_NOT_CONVERGED = 10,         /* refinement did not reach its tolerance */
  REFEFF_FMS_ERR_DUPLICATE_ABSORBER = 11,    /* FmsError::DuplicateAbsorber */
  REFEFF_FMS_ERR_MISSING_CENTRAL_ATOM = 12,  /* FmsError::MissingCentralAtom */
  REFEFF_FMS_ERR_UNSUPPORTED = 13,           /* valid input outside this library's scope */
  REFEFF_FMS_ERR_CUDA = 14,                  /* CUDA runtime error (message in last_error) */
  REFEFF_FMS_ERR_OUT_OF_MEMORY = 15,
  REFEFF_FMS_ERR_INVALID_TOLERANCE = 16,     /* FmsError::InvalidTolerance */
  REFEFF_FMS_ERR_INVALID_CLUSTER_RADIUS = 17, /* FmsError::InvalidClusterRadius */
  REFEFF_FMS_ERR_SCRATCH_LIMIT = 18,          /* request exceeds REFEFF_FMS_NOALLOC_SCRATCH_BYTES */
  REFEFF_FMS_ERR_ITERATIVE_BREAKDOWN = 19,    /* FmsError::IterativeSolverBreakdown (minv != 0) */
  REFEFF_FMS_ERR_DEBYE = 20                   /* DebyeError::IntegrationDidNotConverge / NonFiniteOutput, or a
                                                 pair sigma^2 that fails narrow_nonnegative_f64_to_f32 */
} refeff_fms_status;

/* Solver forms for the dense system (I - G0 T) X = G0[:, absorber]. */
/* For a plan with minv != 0 (the FEFF iterative forms, solvers.rs:225-357)
 * the form picks the arithmetic of the iterative solve instead: FP64_LU runs it
 * in FP64, FP32_REFINED in complex FP32 like the reference (no refinement). */
typedef enum {
  /* Plain FP64 blocked LU.  The drop-in for minv = 0 (FEFF gglu,
   * crates/refeff-core/src/fms/solvers.rs:366-484). */
  REFEFF_FMS_FORM_FP64_LU = 0,
  /* Complex FP32 LU, then FP64 iterative refinement of the full solution
   * against the FP64 system until the residual meets the plan tolerance. */
  REFEFF_FMS_FORM_FP32_REFINED = 1,
  /* BiCGSTAB on the complex FP32 system, all m absorber columns of a batch
   * together, right-preconditioned by the plan's learned diagonal
   * (refeff_fms_plan_set_preconditioner; none when unset), inside the same FP64
   * iterative refinement as FP32_REFINED.  Energies whose solve misses the
   * tolerance within the iteration cap are re-solved with the FP64 LU.  LU-form
   * plans (minv = 0) only.  No reference counterpart: the reference's
   * BiCGSTAB (minv = 1, iterative.rs:181-254) is unpreconditioned and
   * Complex32. */
  REFEFF_FMS_FORM_BICGSTAB = 2
} refeff_fms_form;

typedef struct refeff_fms_context refeff_fms_context;
typedef struct refeff_fms_plan refeff_fms_plan;
typedef struct refeff_fms_precond_model refeff_fms_precond_model;

/* ---- context ---------------------------------------------------------- */

/* Create a context on CUDA device `device` (one GPU per context). */
int refeff_fms_context_create(int device, refeff_fms_context** out);
void refeff_fms_context_destroy(refeff_fms_context* ctx);
/* Message of the last failing call on this context ("" if none). */
const char* refeff_fms_last_error(const refeff_fms_context* ctx);
int refeff_fms_abi_version(void);
/* Total GPU kernel launches issued by this library in the process so far
 * (launches replayed inside CUDA graphs included). */
unsigned long long refeff_fms_kernel_launches(void);

/* Context options; they apply to plans created and dense solves started
 * after the call.
 *   REFEFF_FMS_OPT_TENSOR_CORES: 1 (default) runs the trailing updates of the
 *     FP32 LU on the tcgen05 tensor cores (split TF32, FP32 accumulation);
 *     0 runs them on the CUDA cores.
 *   REFEFF_FMS_OPT_DENSE_REFINEMENT: corrections allowed in
 *     refeff_complex_lu_solve_batched with REFEFF_FMS_FORM_FP32_REFINED
 *     (default 10; 0 returns the plain FP32 LU solution, flagged NOT_CONVERGED).
 *   REFEFF_FMS_OPT_TC_WAIT_POLLS: poll budget of each wait between the
 *     roles of the tensor-core update (copy, MMA, epilogue); 0 restores the
 *     default 2^26 (each wait also gives up after one second).  A wait that
 *     gives up marks the call's tensor-core result void and every energy of
 *     the call is solved again with the FP64 LU (status 0, same results as
 *     REFEFF_FMS_FORM_FP64_LU; refeff_fms_last_error names the timeout).
 *     Applies from the next solve call of every plan of the context.
 *   REFEFF_FMS_OPT_PAIRED_BLOCKS: 1 (default) lets the FP32 LU on the tensor
 *     cores take its 64-column blocks in pairs, with one K = 128 trailing
 *     update per pair (half the trailing-matrix traffic); 0 updates after
 *     every block.  Same factors up to rounding.  Applies from the next solve
 *     call of every plan of the context. */
#define REFEFF_FMS_OPT_TENSOR_CORES 1
#define REFEFF_FMS_OPT_DENSE_REFINEMENT 2
#define REFEFF_FMS_OPT_TC_WAIT_POLLS 3
#define REFEFF_FMS_OPT_PAIRED_BLOCKS 4
/*   REFEFF_FMS_OPT_MULTI_STREAMS: streams that refeff_fms_real_space_spectrum_multi
 *     spreads its plans over (1..64, default 4); plans are packed onto them by
 *     estimated cost (energies x n^3), largest first, each to the least-loaded
 *     stream. */
#define REFEFF_FMS_OPT_MULTI_STREAMS 5
/*   REFEFF_FMS_OPT_DUAL_STREAMS: 1 (default) lets a single plan's spectrum of at
 *     least 8 energies run as batches alternating between two workspaces on two
 *     streams (the caller's and one of the plan's), so that the latency-bound
 *     phases of one batch overlap the arithmetic of the other, when device
 *     memory has room for the second workspace; 0 runs one batch after another
 *     on the caller's stream.  Same results. */
#define REFEFF_FMS_OPT_DUAL_STREAMS 6
/*   REFEFF_FMS_OPT_MULTI_GRAPH: 1 (default) runs the device work of a
 *     refeff_fms_real_space_spectrum_multi call that repeats the previous one
 *     (same plans in the same order, energy counts, batch sizes and form; the
 *     LU forms) as one CUDA graph: captured on the repeat, replayed by every
 *     later repeat until a buffer of any plan is reallocated or freed, or an
 *     option or plan setting changes; 0 keeps one launch sequence per plan. */
#define REFEFF_FMS_OPT_MULTI_GRAPH 7
/*   REFEFF_FMS_OPT_BICG_TENSOR: 1 (default) runs the BICGSTAB form's
 *     matrix-vector products on the tensor cores (split TF32, four real
 *     products, up to 32 right-hand sides); 2 the three-product (3M) form of
 *     the same; 0 on the FP32 CUDA cores.  A product whose bounded wait gives
 *     up hands its matrices to the refined LU. */
#define REFEFF_FMS_OPT_BICG_TENSOR 8
/*   REFEFF_FMS_OPT_RESIDUAL_TENSOR: 1 (default) computes the refinement
 *     residual r = b - A x of the FP32 LU forms on the tensor cores (exact
 *     products of 8-bit digits of A and x on the bf16 path, summed in
 *     double-float, one pass per 16 right-hand sides; with the tensor-core
 *     update on);
 *     0 in double-float on the FP32 CUDA cores.  The tensor-core residual
 *     reaches about 2^-48 of ||a_row||_1 ||x||_inf (2^-43 of sum |a||x|
 *     componentwise), the double-float one about 2^-47 of sum |a||x|.  A residual whose bounded wait gives up sends the call's
 *     energies to the FP64 LU. */
#define REFEFF_FMS_OPT_RESIDUAL_TENSOR 9
int refeff_fms_context_set_option(refeff_fms_context* ctx, int option, long long value);
/* How often the context captured and replayed the many-cluster graph. */
int refeff_fms_context_graph_stats(const refeff_fms_context* ctx, long long* captures, long long* replays);

/* ---- cluster preparation (host) -------------------------------------- */

/* FEFF yprep + sortat for one absorber: replaces fms_yprep_cluster
 * (crates/refeff-core/src/fms/cluster.rs:10-84) followed by
 * sort_representative_atoms (cluster.rs:115-195), as called from
 * fms_atoms_from_geom (crates/refeff-engine/src/fms.rs:4286-4322) and
 * build_fms_source_outputs (fms.rs:3578-3580).
 * positions_xyz: n_rows x 3 floats (row-major x,y,z); potentials: n_rows ints.
 * out_*: capacity n_rows.  The absorber ends up first, at the origin. */
int refeff_fms_yprep_cluster(int central_potential, int max_potential, int n_rows, const int* potentials,
                             const float* positions_xyz, float cluster_radius, int cluster_capacity,
                             float* out_positions_xyz, int* out_potentials, int* out_count);

/* ---- plan ------------------------------------------------------------- */

/* Energy-independent inputs; replaces FmsRealSpacePlanInput
 * (crates/refeff-core/src/fms/types.rs:166, driver.rs:105-140). */
typedef struct {
  int n_atoms;                      /* prepared cluster (absorber first) */
  const float* positions_xyz;       /* n_atoms x 3, Angstrom */
  const int* potentials;            /* n_atoms */
  int spin_channels;                /* nsp: 1 or 2 */
  int spin_selector;                /* global.inp ispin */
  int lfms;                         /* 0: absorber potential only; else all potentials (at most 64
                                       representative states in total) */
  int minv;                         /* FEFF minv: 0 LU, 1 ggbi, 2 ggrm (recursion), 3 gggm, other ggtf (TFQMR) */
  int max_potential;                /* nph */
  int global_lmax;                  /* max over lmaxph */
  const int* raw_potential_lmax;    /* lmaxph(0..nph), clamped like clamp_fms_lipotx */
  float direct_cutoff;              /* rdirec, Angstrom */
  const float* mean_square_displacements; /* N x N column-major [atom2 + N*atom1], or NULL */
  float sig2g;                      /* used for every i != j pair when the table is NULL */
  float convergence_tolerance;      /* toler1 (iterative forms) */
  float zero_tolerance;             /* toler2 */
} refeff_fms_plan_input;

int refeff_fms_real_space_plan_create(refeff_fms_context* ctx, const refeff_fms_plan_input* input,
                                      refeff_fms_plan** out);

/* The same plan with the full scattering matrix requested
 * (FmsRealSpacePlanInput::full_scattering_matrix_requested, set from fms.inp
 * save_gg_slice at crates/refeff-engine/src/fms.rs:3610): every column of G0
 * is a right-hand side, X = (I - G0 T)^-1 G0 (FmsLuResult::full_scattering,
 * crates/refeff-core/src/fms/solvers.rs:473-479).  Like the reference, the
 * request forces the LU form (fms_scattering_method_selection,
 * driver.rs:72-96): minv is taken as 0 and only REFEFF_FMS_FORM_FP64_LU is
 * accepted.  Every atom must carry b = nsp (L+1)^2 states (fixed-width atom
 * blocks, fms.rs:4164-4172), else UNSUPPORTED. */
int refeff_fms_real_space_plan_create_full(refeff_fms_context* ctx, const refeff_fms_plan_input* input,
                                           refeff_fms_plan** out);

/* The pair mean-square displacement table that feeds
 * refeff_fms_plan_input.mean_square_displacements, computed on the GPU.
 * Replaces fms_mean_square_displacements_with_metadata
 * (crates/refeff-engine/src/fms.rs:4345-4433) for idwopt < 0 (sig2g for every
 * i != j pair), 0 (correlated Debye: corrfn/sigms on the path atom1 -> atom2
 * -> atom1, crates/refeff-core/src/debye/models.rs:88-271) and 3 (classical
 * Debye: corrfn2/sigcl); other idwopt values return UNSUPPORTED.
 *   positions_xyz, potentials: the prepared cluster (refeff_fms_yprep_cluster)
 *   atomic_numbers: per potential 0..n_potentials-1 (phase.bin potential headers)
 *   temperature, debye_temperature: fms.inp tk, thetad (K)
 *   average_norman_radius: phase.bin rnrmav (Bohr)
 *   table_out: n_atoms x n_atoms floats, [atom2 + N*atom1], host memory
 *   debye_term_out: optional n_atoms x n_atoms doubles, the Debye term before
 *                   sig2g is added and the sum narrowed (NULL to skip)
 * Errors: INVALID_ARGUMENT (tk < 0, thetad <= 0, rnrmav <= 0, atomic number
 * outside 1..139, two atoms at one position), POTENTIAL_OUT_OF_RANGE,
 * NONFINITE_COORDINATE, DEBYE. */
int refeff_fms_debye_sigma2_table(refeff_fms_context* ctx, int idwopt, int n_atoms, const float* positions_xyz,
                                  const int* potentials, int n_potentials, const int* atomic_numbers,
                                  double temperature, double debye_temperature, double average_norman_radius,
                                  float sig2g, float* table_out, double* debye_term_out);
void refeff_fms_real_space_plan_destroy(refeff_fms_plan* plan);

/* Sizes of a plan: state count n, channel count C = nsp (L+1)^2 of the
 * scattering table, absorber block width m, potential count. */
int refeff_fms_plan_query(const refeff_fms_plan* plan, int* n_states, int* channel_count, int* absorber_block,
                          int* n_potentials);

/* Tuning: energies solved per device batch (0 = automatic from free memory)
 * and the refinement limits of REFEFF_FMS_FORM_FP32_REFINED: at most
 * max_iterations corrections; an energy has converged when its last
 * correction d_k, or the error it leaves, estimated as |d_k|^2 / |d_k-1| (the
 * initial solve counting as d_0 = x), is within tolerance * max|x| (max norms;
 * default 10, 1e-10).
 * Energies that reach the limit, or whose corrections stop halving, are
 * solved again with the FP64 LU. */
int refeff_fms_plan_set_batch(refeff_fms_plan* plan, int max_batch);
int refeff_fms_plan_set_refinement(refeff_fms_plan* plan, int max_iterations, double tolerance);

/* Per-phase device time (CUDA events on the solve stream) of the spectrum
 * calls made while profiling is on, accumulated in milliseconds:
 *   0 system build (G0, T, I - G0 T)   1 LU elimination
 *   2 triangular sweeps                3 FP64 residuals
 *   4 absorber extraction / small solves
 *   5 the tensor-core trailing-update kernels alone (part of 1)
 * Profiling runs batches without graph replay; enabling it resets the sums. */
#define REFEFF_FMS_PHASES 6
int refeff_fms_plan_set_profiling(refeff_fms_plan* plan, int enable);
int refeff_fms_plan_phase_times(const refeff_fms_plan* plan, double* ms_out, int n_phases);

/* ---- spectrum --------------------------------------------------------- */

/* Per-energy inputs; replaces FmsRealSpaceEnergyPoint (types.rs).
 * wave_numbers: n_energies x nsp (energy-major).
 * phase_shifts: n_energies blocks, each the FEFF xphase(spin, l + L, pot)
 *   table of shape (nsp, 2L+1, npot) in column-major order
 *   (built by fms_phase_shifts_for_energy, crates/refeff-engine/src/fms.rs:5002-5054). */
typedef struct {
  int n_energies;
  const refeff_complex128* wave_numbers;
  const refeff_complex128* phase_shifts;
} refeff_fms_energy_points;

typedef struct {
  double seconds;               /* wall time of the call */
  int refinement_iterations;    /* max corrections over energies (FP32_REFINED) */
  double residual_max;          /* max relative residual ||b - A x|| / ||b|| after refinement */
  int energies_failed;          /* energies with a non-zero status */
  int fp64_fallbacks;           /* energies re-solved with the FP64 LU because refinement missed */
} refeff_fms_report;

/* fms_real_space_spectrum (crates/refeff-core/src/fms/driver.rs:231-239):
 * solves every energy point and writes the scattering table of each, shape
 * (C, C, npot) column-major, C = nsp (L+1)^2 (FmsLuResult::scattering,
 * solvers.rs:415-471): entry (row, col, pot) = X[offset(pot) + row, col] with
 * X = (I - G0 T)^-1 G0[:, offset(pot) : offset(pot) + ipart].
 * status_out (optional): one refeff_fms_status per energy (the reference
 * returns Vec<Result<..>>).  Host buffers; the call copies inputs to the GPU
 * and results back. */
int refeff_fms_real_space_spectrum(refeff_fms_plan* plan, const refeff_fms_energy_points* points,
                                   refeff_fms_form form, refeff_complex128* scattering_out, int32_t* status_out,
                                   refeff_fms_report* report);

/* Spectrum of a full plan (refeff_fms_real_space_plan_create_full) with the
 * FP64 LU: the scattering table as refeff_fms_real_space_spectrum, plus the
 * two save_gg_slice outputs of build_saved_fms_scattering_outputs
 * (crates/refeff-engine/src/fms.rs:4154-4216), reference state order:
 *   slice_out: n_energies x (b x n) column-major, rows [0, b) (the absorber's
 *              states) of X over every column;
 *   diag_out:  n_energies x n_atoms x (b x b) column-major, the diagonal block
 *              of every atom.
 * Energies that failed hold zeros (status_out says which). */
int refeff_fms_real_space_spectrum_full(refeff_fms_plan* plan, const refeff_fms_energy_points* points,
                                        refeff_complex128* scattering_out, refeff_complex128* slice_out,
                                        refeff_complex128* diag_out, int32_t* status_out, refeff_fms_report* report);

/* Same solve for inputs already resident in device memory (same layouts as
 * above, device pointers); writes the solved blocks per energy: for lfms = 0
 * the absorber block, d_gg_out = n_energies x (m x m) complex128 (m from
 * refeff_fms_plan_query); for lfms != 0 the block of every potential
 * 0..max_potential in turn, each ipart(pot) x ipart(pot) column-major, packed
 * one after another per energy.  `stream` is a cudaStream_t (NULL = the
 * context stream).  Asynchronous: synchronise the stream before reading
 * results. */
int refeff_fms_real_space_spectrum_device(refeff_fms_plan* plan, int n_energies, const void* d_wave_numbers,
                                          const void* d_phase_shifts, refeff_fms_form form, void* d_gg_out,
                                          int32_t* d_status, void* stream);

/* Many clusters in one call (the batched form of fms_real_space_spectrum over
 * several plans, crates/refeff-core/src/fms/driver.rs:231-239): plans[i] with
 * points[i] writes scattering_out[i] (and status_out[i] when status_out is not
 * NULL), all plans of the same context.  Every plan's device work is put in
 * flight on a small pool of streams before any completes, so small clusters
 * overlap; the return code is the first failure, the report sums over plans. */
int refeff_fms_real_space_spectrum_multi(refeff_fms_context* ctx, int n_plans, refeff_fms_plan* const* plans,
                                         const refeff_fms_energy_points* points, refeff_fms_form form,
                                         refeff_complex128* const* scattering_out, int32_t* const* status_out,
                                         refeff_fms_report* report);

/* No reference counterpart: the autotuner of the batched form.  For the
 * clusters of one refeff_fms_real_space_spectrum_multi workload it times, on
 * up to sample_energies evenly spaced energies of every cluster (0 = all),
 * per size bucket (state counts rounded up to a multiple of 256) the FP32
 * elimination's inner panel width and block pairing (FP32_REFINED only), then
 * the number of streams the clusters are packed onto, and applies the fastest
 * (refeff_fms_plan_set_tuning on each plan, REFEFF_FMS_OPT_MULTI_STREAMS on
 * the context).  With cache_path, the choice is stored in that JSON file under
 * a key of the device name, the form and the clusters' sizes, and a later call
 * with the same key applies the stored choice without measuring
 * (out->from_cache = 1).  The results of the many-cluster call do not depend on
 * the choice beyond rounding. */
typedef struct {
  int streams;             /* streams chosen for the many-cluster call */
  int buckets;             /* size buckets tuned */
  double seconds_default;  /* sample time with the default choices */
  double seconds_tuned;    /* sample time with the chosen ones */
  int from_cache;          /* 1: applied from cache_path without measuring */
} refeff_fms_tuning;
int refeff_fms_autotune_multi(refeff_fms_context* ctx, int n_plans, refeff_fms_plan* const* plans,
                              const refeff_fms_energy_points* points, refeff_fms_form form, int sample_energies,
                              const char* cache_path, refeff_fms_tuning* out);
/* Per-plan choices of the FP32 elimination: inner_width 0 (by size: two-level
 * from n = 512 with 16-column inner panels first), 16 or 32 (two-level with
 * that inner panel width first, from n = 128) or 1 (single-level panels);
 * paired_blocks -1 (the context's REFEFF_FMS_OPT_PAIRED_BLOCKS), 0 or 1.
 * Applies from the plan's next solve. */
int refeff_fms_plan_set_tuning(refeff_fms_plan* plan, int inner_width, int paired_blocks);
int refeff_fms_plan_get_tuning(const refeff_fms_plan* plan, int* inner_width, int* paired_blocks);

/* Per-energy outcome of the last refeff_fms_real_space_spectrum call with
 * REFEFF_FMS_FORM_FP32_REFINED: relative residual max|b - A x| / max|b| of
 * the last residual evaluated (the one that produced the final correction),
 * corrections applied, and whether the energy was re-solved with the FP64 LU
 * because refinement did not converge (each pointer optional). */
int refeff_fms_plan_refinement_stats(const refeff_fms_plan* plan, int n_energies, double* rel_residual,
                                     int* iterations, int* fp64_fallback);

/* FEFF gg section for one energy (fms_gg_section_values,
 * crates/refeff-engine/src/fms.rs:2004-2047): the absorber block widened to
 * the output spin capacity nspu (>= nsp) of .dimensions.dat; out is
 * (nspu (lmax0+1)^2)^2 complex, column-major, zero-padded. */
int refeff_fms_gg_section(const refeff_fms_plan* plan, const refeff_complex128* scattering, int nspu,
                          refeff_complex128* out);

/* ---- FEFF file seam (module-level drop-in) ---------------------------- */

/* The `fms` stage on a FEFF work directory, replacing the generation path of
 * run_fms_in_dir (crates/refeff-engine/src/fms.rs:1102-1127, 1141-1219,
 * 3549-3695): reads fms.inp, global.inp, phase.bin, geom.dat and the optional
 * .dimensions.dat, solves every energy on the GPU, and writes gg.bin and
 * gg.dat (byte-compatible sectioned text, io/gg_dat.rs:174-233) and log3.dat
 * (fms.rs:5995-6058).  With save_gg_slice on, the full scattering matrix is
 * solved with the FP64 LU whatever `form` asks (the reference forces the LU
 * form) and gg_slice.bin and gg_diag.bin are written too (fms.rs:1113-1125).
 * Supported: idwopt < 0 (uniform sig2g), 0 and 3 (Debye models); other idwopt
 * values return REFEFF_FMS_ERR_UNSUPPORTED.  A work directory without
 * geom.dat but with feff.inp gets its cluster from feff.inp, through the same
 * geom.dat text FEFF's rdinp would have written (refeff_fms_write_geom_dat). */
int refeff_fms_run_dir(refeff_fms_context* ctx, const char* work_dir, refeff_fms_form form, refeff_fms_report* report);

/* The cluster of a feff.inp as FEFF's rdinp hands it to the FMS stage: the
 * ATOMS rows (x y z ipot, fields after '*' ignored) read with FEFF's line rules
 * (full-line comments ; * % #, inline comments ! # % outside delimiters,
 * BWORDS fields, block cards, INCLUDE / LOAD, END; crates/refeff-io/src/input.rs:64-372,
 * model.rs:626-676), scaled by RMULTIPLIER (model.rs:198-207), moved so the
 * absorber (the first atom of potential 0, else the first atom) sits at the
 * origin as row 0, coincident atoms dropped, and ordered by FEFF's strict
 * selection sort on the fused distance z*z + (x*x + y*y)
 * (crates/refeff-io/src/rdinp/geometry.rs:18-88).  model_atoms_out gets the
 * one-based first row of each potential (iatph, geometry.rs:90-119).
 * xyz_out: row_capacity x 3 doubles; ipot_out: row_capacity; model_atoms_out:
 * model_capacity.  With both capacities 0 only the counts are returned.
 * LATTICE / CIF clusters, OVERLAP shells and the NRIXS frame rotation return
 * REFEFF_FMS_ERR_UNSUPPORTED; the reason is in refeff_fms_feff_inp_last_error. */
int refeff_fms_geometry_from_feff_inp(const char* feff_inp_path, int row_capacity, double* xyz_out, int32_t* ipot_out,
                                      int32_t* n_rows, int model_capacity, int32_t* model_atoms_out,
                                      int32_t* n_model);
/* geom.dat for that cluster, byte-compatible with rdinp's write_geom_dat
 * (crates/refeff-io/src/rdinp/structure.rs:57-81). */
int refeff_fms_write_geom_dat(const char* feff_inp_path, const char* geom_dat_path);
/* Message of the last failing feff.inp call on this thread ("" if none). */
const char* refeff_fms_feff_inp_last_error(void);

/* gg.dat / gg.bin writer (gg_dat_bytes, crates/refeff-io/src/gg_dat.rs:174-202):
 * n_sections square dim x dim complex blocks (column-major), section numbers
 * 1..n, every value as Fortran E20.10 (crates/refeff-io/src/format.rs:174-209).
 * Host only; needs no GPU. */
int refeff_fms_write_gg_dat(const char* path, int n_sections, int dim, const refeff_complex128* values);

/* gg_slice.bin / gg_diag.bin writers (rhorrp_gg_slice_bin_bytes,
 * rhorrp_gg_diag_bin_bytes, crates/refeff-io/src/rhorrp_gg_bin.rs:138-160,
 * 228-252): Fortran sequential records, little-endian, values narrowed to
 * complex f32.  slice: ne blocks of rows x cols; diag: ne x n_atoms blocks of
 * dim x dim; column-major.  NONFINITE_INPUT when a narrowed value is not
 * finite.  Host only. */
int refeff_fms_write_gg_slice_bin(const char* path, int ne, int rows, int cols, const refeff_complex128* values);
int refeff_fms_write_gg_diag_bin(const char* path, int ne, int n_atoms, int dim, const refeff_complex128* values);

/* phase.bin reader (crates/refeff-io/src/phase_bin/parse.rs:18-130, PAD
 * decoding crates/refeff-io/src/pad.rs:102-127).  Host only.
 * dims: spin count, energy count, potential count (nph + 1), largest lmax.
 * read: energy grid (ne), reference energy (ne x nsp, energy fastest), lmax per
 * potential, and phase shifts (ne, 2*lmax_max+1, nsp, npot) column-major with
 * the signed-l axis centred on lmax_max (zero outside a potential's lmax);
 * any output pointer may be NULL. */
int refeff_fms_phase_bin_dims(const char* path, int* nsp, int* ne, int* npot, int* lmax_max);
int refeff_fms_phase_bin_read(const char* path, refeff_complex128* energy_grid, refeff_complex128* reference_energy,
                              int* potential_lmax, refeff_complex128* phase_shifts);

/* ---- MKGTR: gg -> trace spectrum ---------------------------------------- */

/* FEFF transition B matrix (bcoef; transition_b_matrix,
 * crates/refeff-core/src/angular/transition.rs:9-73), host only, FP64.
 * polarization_tensor: 3 x 3 complex, row-major (rows m = -1, 0, 1), may be
 * NULL when polarization == 0.  bmat_out (optional): (2L+1, 2, 8, 2L+1, 2, 8)
 * complex column-major, indexed [m2+L, s2, k2, m1+L, s1, k1] with transitions
 * zero-based; lind_out / kiind_out (optional): 8 orbital momenta (-1 = unused)
 * and final-state kappas. */
int refeff_fms_transition_matrix(int lmax, int initial_kappa, int polarization,
                                 const refeff_complex128* polarization_tensor, int multipole, int trace_orbital,
                                 int spin, int spin_channels, double spin_vector_angle, refeff_complex128* bmat_out,
                                 int32_t* lind_out, int32_t* kiind_out);

/* MKGTR trace on the GPU (mkgtr_green_trace, crates/refeff-core/src/fms/mkgtr.rs:790-952):
 * traces[sp + n_spectra*e] = sum over transitions k1,k2 (lind >= 0), spins s1,s2 < active_spin_channels and
 * m1, m2 of gg[e]((l1^2+l1+m1) nsp + s1, (l2^2+l2+m2) nsp + s2) * bmat[sp](m2,s2,k2,m1,s1,k1)
 * * rkk[e,k1,s1] * rkk[e,k2,s2].  lind: n_spectra x 8, bmat: n_spectra blocks as from
 * refeff_fms_transition_matrix with `lmax`.  Host buffers: gg (E, dim, dim) column-major per
 * energy, rkk (E, 8, rkk_spins) column-major, traces (n_spectra, E). */
int refeff_fms_mkgtr_trace(refeff_fms_context* ctx, int n_energies, int dim, int active_spin_channels, int lmax,
                           int n_spectra, const int32_t* lind, const refeff_complex128* bmat,
                           const refeff_complex128* gg, const refeff_complex128* rkk, int rkk_spins,
                           refeff_complex128* traces);

/* The same on device buffers, fusable after refeff_fms_real_space_spectrum_device: gg[e](r, c) =
 * d_gg[e*gg_energy_stride + r + gg_ld*c] (the scattering tables with gg_ld = C and energy stride
 * C*C*npot), d_rkk (E, 8, active spins) column-major, d_traces (n_spectra, E).  Synchronises
 * `stream` (NULL = the context's stream) before returning. */
int refeff_fms_mkgtr_trace_device(refeff_fms_context* ctx, int n_energies, int dim, int active_spin_channels,
                                  int lmax, int n_spectra, const int32_t* lind, const refeff_complex128* bmat,
                                  const refeff_complex128* d_gg, long long gg_ld, long long gg_energy_stride,
                                  const refeff_complex128* d_rkk, refeff_complex128* d_traces, void* stream);

/* The `mkgtr` stage on a FEFF work directory (run_mkgtr_in_dir + the ordinary
 * MKGTR outputs, crates/refeff-engine/src/fms.rs:559-600, 5255-5332, 5528-5608):
 * reads fms.inp, global.inp, phase.bin and gg.bin (else gg.dat); when fms.bin
 * or gtr.dat is missing, writes both (fms.bin PAD text, io/fms_bin.rs:77-98;
 * gtr.dat, io/gtr_dat.rs:60-71) from the GPU trace; then makes sure log3.dat
 * carries the MKGTR lines (fms.rs:5941-5963).  NRIXS (do_nrixs = 1) and EELS
 * (eels.inp) projections return REFEFF_FMS_ERR_UNSUPPORTED.  *written (optional)
 * receives the number of trace files written. */
int refeff_fms_run_mkgtr_dir(refeff_fms_context* ctx, const char* work_dir, int* written);

/* fms.bin writer (fms_bin_string, crates/refeff-io/src/fms_bin.rs:77-98): title
 * "FMS rfms=%7.4f", counts ne ne1 ne3 nph npadx 0 in I7, then one '$' PAD block
 * (pad.rs:142-161) per spectrum of traces (n_spectra x ne, column-major).
 * Host only. */
int refeff_fms_write_fms_bin(const char* path, double cluster_radius, int ne, int ne1, int ne3, int nph, int pad_width,
                             int n_spectra, const refeff_complex128* traces);

/* gtr.dat writer (gtr_dat_string, crates/refeff-io/src/gtr_dat.rs:60-71): per
 * energy Re E, Im E, Re gtr, Im gtr as F13.6.  Host only. */
/* FF2X XANES mu(E) from the MKGTR trace, host only: the stage after MKGTR
 * (ff2x_xanes_corrected_components, crates/refeff-engine/src/ff2x.rs:3186-3262;
 * ff2x_xscorr at zero electronic temperature, 4437-4641; the xmu.dat
 * normalisation and rows, 3309-3399).  chia = s02 * trace; per main row
 *   total  = Im(xsec + chia * background + xscorr(chia))
 *   atomic = Im(xsec + xscorr(0))       (0 when include_atomic == 0)
 *   mu0 = atomic / norm, chi = (total - atomic) / norm, mu = mu0 + chi,
 * norm = background interpolated (order 1) at fermi_photon_energy + 50 eV
 * (at fermi_photon_energy for ispec 2), or 1 when absolu == 1.
 *   ne, ne1: xsect.dat rows (ne1 horizontal rows, then the vertical contour
 *            whose last row lies at the Fermi level)
 *   fermi_index: 0-based Fermi row on the horizontal grid; ispec: +-1 or +-2
 *   energy (ne, complex Hartree), omega (ne1 photon energies, Hartree),
 *   cross_section (ne complex), background (ne), trace (ne complex gtr(E)),
 *   real_correction: vrcorr in Hartree (contour shift and rescale)
 *   imaginary_correction: the broadening in Hartree (vicorr, or half the core-hole width with
 *     i_gamma_ch = 1; ff2x.rs:5416-5425); above 1e-4 (total, atomic) are Lorentz-broadened over
 *     omega before normalisation (ff2x.rs:3265-3306, FMS-only spectra)
 *   mu, mu0, chi: ne1 each, optional.
 * The sig_gk Debye factor is applied by refeff_ff2x_debye_factor; this call
 * runs the zero-temperature xscorr (refeff_ff2x_xanes_mu_thermal takes the
 * electronic temperature). */
int refeff_ff2x_xanes_mu(int ne, int ne1, int fermi_index, int ispec, int absolu, int include_atomic,
                         const refeff_complex128* energy, const double* omega, const refeff_complex128* cross_section,
                         const double* background, const refeff_complex128* trace, double s02, double real_correction,
                         double imaginary_correction, double fermi_photon_energy, double* mu, double* mu0,
                         double* chi);
/* refeff_ff2x_xanes_mu with FEFF's electronic temperature (eV; 0 = the
 * zero-temperature xscorr, > 0 the thermal xscorr below). */
int refeff_ff2x_xanes_mu_thermal(int ne, int ne1, int fermi_index, int ispec, int absolu, int include_atomic,
                                 const refeff_complex128* energy, const double* omega,
                                 const refeff_complex128* cross_section, const double* background,
                                 const refeff_complex128* trace, double s02, double real_correction,
                                 double imaginary_correction, double fermi_photon_energy,
                                 double electronic_temperature_ev, double* mu, double* mu0, double* chi);
/* FF2X xscorr (ff2x_xscorr, crates/refeff-engine/src/ff2x.rs:4437-4641, and
 * at electronic_temperature_ev > 0 ff2x_thermal_xscorr, 4643-5050): the
 * correction cchi (ne1 rows) of xmu = cross_section + path_chi * background
 * over the xsect.dat rows.  The thermal form needs ne >= 2 ne1 + 11 rows (the
 * horizontal rows, ne1 loss rows, 10 auxiliary rows, the poles and a last row
 * at the Fermi level) and ignores fermi_index.  Host only.  Errors:
 * INVALID_ARGUMENT (layout, temperature < 0, a Fermi window outside the grid),
 * NONFINITE_INPUT. */
int refeff_ff2x_xscorr(int ne, int ne1, int fermi_index, int ispec, const refeff_complex128* energy,
                       const refeff_complex128* cross_section, const double* background,
                       const refeff_complex128* path_chi, double real_correction, double electronic_temperature_ev,
                       refeff_complex128* cchi_out);

/* FEFF xsect.dat, XSPH's cross-section table, read and handed to FF2X the way
 * FEFF's rdxbin does (parse_xsect_dat and xsect_dat_ff2x_handoff,
 * crates/refeff-io/src/xsect_dat.rs:394-760, 268-309): energies from eV to
 * Hartree, omega = Re(E) - edge + emu, the signed wave number of Re(E) - edge
 * (sqrt(2|x|) with the sign of x), and the effective S02 = the file's value when
 * mbconv > 0 or current_s02 <= 0.1, else current_s02.  The arrays feed
 * refeff_ff2x_xanes_mu / _thermal (energy, omega, cross_section, background).
 *   counts_out[4]: rows (nxsec), ne1, fermi_index (zero-based ik0 - 1), titles.
 *   scalars_out[7]: effective s02, the file's s02, erelax, wp, edge, emu
 *                   (both in Hartree as written), gamach in Hartree.
 *   energy_out, omega_out, wave_number_out, background_out, cross_section_out:
 *                   capacity rows each.
 * With capacity 0 only counts_out is written.  Errors: INVALID_ARGUMENT (file,
 * record or layout errors, ik0 outside 1..ne1, capacity below the row count),
 * NONFINITE_INPUT; the reason is in refeff_ff2x_xsect_last_error.  Host only. */
int refeff_ff2x_read_xsect_dat(const char* path, double current_s02, int mbconv, int capacity, int32_t* counts_out,
                               double* scalars_out, refeff_complex128* energy_out, double* omega_out,
                               double* wave_number_out, double* background_out, refeff_complex128* cross_section_out);
const char* refeff_ff2x_xsect_last_error(void);

/* FEFF conv (crates/refeff-core/src/convolution/lorentzian.rs:32-100): the
 * piecewise-linear spectrum (n >= 2 points over increasing omega) broadened by
 * a Lorentzian of half width `width`, divided by single-precision pi as FEFF
 * does.  Host only. */
int refeff_ff2x_lorentz_convolve(int n, const double* omega, const refeff_complex128* spectrum, double width,
                                 refeff_complex128* out);

/* FF2X's Debye factor sig_gk on the fine structure of the xmu.dat rows
 * (crates/refeff-engine/src/ff2x.rs:3388-3397): with sig_gk > 1e-4, chi[r] *=
 * exp(-(sig_gk * wave_number[r])^2) (wave numbers in 1/Angstrom), then mu[r] =
 * mu0[r] + chi[r] when mu and mu0 are given.  Host only. */
int refeff_ff2x_debye_factor(int n, const double* wave_number, double sig_gk, const double* mu0, double* chi,
                             double* mu);

int refeff_fms_write_gtr_dat(const char* path, int ne, const refeff_complex128* energy, const refeff_complex128* trace);

/* ---- learned preconditioner for the BiCGSTAB form ---------------------- */
/* No reference counterpart.  A small MLP (features -> 2 tanh layers of
 * `hidden` units -> outputs) predicts, per (energy, atom), the channel
 * diagonal of the atom's block of (I - G0 T)^-1 as a deviation from 1; the
 * BiCGSTAB form applies it as a right preconditioner.  Features per (energy,
 * atom): Re/Im k, the atom's t_l (l = 0..lmax), and for three neighbour shells
 * (< 2.9, < 3.7, < 4.6 Angstrom) the neighbour count / 12, the mean distance / 5
 * and the neighbours' mean t_l: 2 + 2(L+1) + 3 (2 + 2(L+1)) values.  Outputs:
 * 2 (L+1)^2 (Re, Im per channel l^2 + l + m).  Training (forward, backward,
 * Adam) and inference run on the GPU. */
int refeff_fms_precond_model_create(refeff_fms_context* ctx, int lmax, int hidden, unsigned long long seed,
                                    refeff_fms_precond_model** out);
/* Model kinds: the channel diagonal above (REFEFF_FMS_PRECOND_DIAGONAL, what
 * refeff_fms_precond_model_create makes) or the whole per-atom block
 * (REFEFF_FMS_PRECOND_BLOCK): 2 C^2 outputs, C = (L+1)^2, the block of
 * (I - G0 T)^-1 minus the identity, row-major, Re/Im interleaved; rows and
 * columns beyond an atom's own (lmax_atom+1)^2 channels are ignored.  The
 * BiCGSTAB form then applies the predicted block per atom (block Jacobi on the
 * inverse).  Block models need lmax <= 4 and plans with one spin channel
 * (refeff_fms_plan_set_preconditioner: UNSUPPORTED otherwise). */
enum { REFEFF_FMS_PRECOND_DIAGONAL = 0, REFEFF_FMS_PRECOND_BLOCK = 1 };
int refeff_fms_precond_model_create_kind(refeff_fms_context* ctx, int lmax, int hidden, int kind,
                                         unsigned long long seed, refeff_fms_precond_model** out);
void refeff_fms_precond_model_destroy(refeff_fms_precond_model* model);
int refeff_fms_precond_model_query(const refeff_fms_precond_model* model, int* n_features, int* hidden, int* n_outputs,
                                   long long* n_params);
/* Parameters as one float vector: W1[H][F], b1[H], W2[H][H], b2[H], W3[O][H], b3[O]. */
int refeff_fms_precond_get_params(const refeff_fms_precond_model* model, float* out);
int refeff_fms_precond_set_params(refeff_fms_precond_model* model, const float* in);
/* Mean squared error over n samples (X: n x F, T: n x O, row-major) and its
 * gradient with respect to the parameters (n_params floats). */
int refeff_fms_precond_loss_grad(refeff_fms_precond_model* model, int n_samples, const float* X, const float* T,
                                 double* loss, float* grad);
/* Adam (beta 0.9 / 0.999, eps 1e-8) on shuffled mini-batches; epoch_loss
 * (optional, `epochs` doubles) receives the full-set loss after each epoch. */
int refeff_fms_precond_train(refeff_fms_precond_model* model, int n_samples, const float* X, const float* T,
                             int epochs, int batch_size, float learning_rate, unsigned long long seed,
                             double* epoch_loss);
int refeff_fms_precond_predict(refeff_fms_precond_model* model, int n_samples, const float* X, float* Y);
/* Attach a model (built for the plan's global lmax) or detach it (NULL). The
 * plan does not own the model. */
int refeff_fms_plan_set_preconditioner(refeff_fms_plan* plan, refeff_fms_precond_model* model);
/* Energy gate of the attached model: it preconditions only the energies with
 * E - E_ref = Re((k a0)^2) / 2 Hartree (first spin's wave number) in
 * [e_lo_ev, e_hi_ev]; the others run unpreconditioned.  Default: all energies. */
int refeff_fms_plan_set_precond_window(refeff_fms_plan* plan, double e_lo_ev, double e_hi_ev);
/* BiCGSTAB controls: iteration cap per solve, relative residual tolerance of
 * each solve, and how often (iterations) the host checks for completion. */
int refeff_fms_plan_set_bicgstab(refeff_fms_plan* plan, int max_iterations, double tolerance, int poll_interval);
/* BiCGSTAB iterations per energy of the last BICGSTAB-form call (all solves;
 * 0 for energies outside the window below). */
int refeff_fms_plan_bicgstab_stats(const refeff_fms_plan* plan, int n_energies, int32_t* iterations);
/* Energy window of the BICGSTAB form (E - E_ref in eV, as the preconditioner
 * window): energies outside it are not iterated but solved by the refined LU
 * (REFEFF_FMS_FORM_FP32_REFINED), as are energies whose BiCGSTAB misses the
 * tolerance within the iteration cap; an energy the refined LU misses goes on
 * to the FP64 LU.  Default: all energies iterate. */
int refeff_fms_plan_set_bicgstab_window(refeff_fms_plan* plan, double e_lo_ev, double e_hi_ev);
/* Per energy of the last BICGSTAB-form call: 0 solved by BiCGSTAB, 1 missed
 * the tolerance and solved by the refined LU, 2 outside the window (refined LU). */
int refeff_fms_plan_bicgstab_lu_energies(const refeff_fms_plan* plan, int n_energies, int32_t* flags);
/* Features of every (energy, atom), atoms in device order (absorber last):
 * E * n_atoms rows of n_features floats. */
int refeff_fms_plan_precond_features(refeff_fms_plan* plan, const refeff_fms_energy_points* points,
                                     float* features_out);
/* Training targets from the FP64 LU: the diagonal of atom `atom`'s block of
 * (I - G0 T)^-1 per energy (atom: prepared-cluster index, 0 = absorber;
 * its state count must not exceed the absorber block width).  diag_out:
 * E x (states of the atom); status_out: per energy (optional). */
int refeff_fms_plan_inverse_diagonal(refeff_fms_plan* plan, const refeff_fms_energy_points* points, int atom,
                                     refeff_complex128* diag_out, int32_t* status_out);
/* Block-model targets: the whole block of atom `atom` in (I - G0 T)^-1,
 * block_out: E x cnt x cnt row-major (cnt = the atom's states),
 * block_out[(e cnt + r) cnt + c] = (A^-1)[s0 + r, s0 + c]. */
int refeff_fms_plan_inverse_block(refeff_fms_plan* plan, const refeff_fms_energy_points* points, int atom,
                                  refeff_complex128* block_out, int32_t* status_out);

/* ---- reciprocal-space FMS (KKR integration of given structure factors) -- */

/* One energy of FEFF kkrintegral (crates/refeff-core/src/fms/reciprocal.rs:67-223):
 * for every k-point X_k = (I - G(k) T)^-1 G(k) (FmsReciprocalPlan::solve_k_point,
 * solved on the GPU as one batch over the k-points), then the Brillouin-zone
 * average sum_k w_k X_k / sum_k w_k (FmsReciprocalAccumulator).
 *   structure_factors: n_kpoints x (order x order) complex, column-major (the
 *     KSPACE structure factors G(k); this library does not compute them)
 *   weights: n_kpoints positive finite weights
 *   t_matrix: order x order lattice T (zeros skipped, as the reference plan does)
 *   form: REFEFF_FMS_FORM_FP64_LU, or REFEFF_FMS_FORM_FP32_REFINED for order <= 64
 *   green_out: order x order; status_out (optional): per k-point status
 * Errors: INVALID_ARGUMENT (empty matrix, no k-point, a weight that is not
 * positive and finite), NONFINITE_INPUT, SINGULAR_MATRIX (first failing
 * k-point in last_error). */
int refeff_fms_reciprocal_integrate(refeff_fms_context* ctx, int order, int n_kpoints,
                                    const refeff_complex128* structure_factors, const double* weights,
                                    const refeff_complex128* t_matrix, refeff_fms_form form,
                                    refeff_complex128* green_out, int32_t* status_out);

/* FEFF kkrintegral core-hole method 1 (fms_reciprocal_apply_core_hole,
 * reciprocal.rs:236-302): G' = G - G[:, a] (I + C G_aa)^-1 C G[a, :] with
 * a = [absorber_offset, absorber_offset + block) and C = t_difference
 * (block x block, FEFF strength * (T_ground - T_core_hole)).  Host only, FP64.
 * Errors: INVALID_ARGUMENT (block outside the matrix), NONFINITE_INPUT,
 * SINGULAR_MATRIX (the Dyson matrix). */
int refeff_fms_reciprocal_core_hole(int order, const refeff_complex128* green, int absorber_offset, int block,
                                    const refeff_complex128* t_difference, refeff_complex128* out);

/* ---- dense solve (refeff-linalg boundary) ----------------------------- */

/* Batched dense complex solve A X = B, replacing complex32_faer_lu_factor +
 * complex32_faer_lu_solve (crates/refeff-linalg/src/lu.rs:385-397, 474-490)
 * for `batch` independent systems.  A: batch x (n x n), B/X: batch x (n x m),
 * column-major host buffers; X may alias B.  status_out (optional, batch
 * entries) reports REFEFF_FMS_ERR_SINGULAR_MATRIX with pivot_out (1-based
 * first zero pivot, optional). */
int refeff_complex_lu_solve_batched(refeff_fms_context* ctx, int n, int m, int batch, const refeff_complex128* A,
                                    const refeff_complex128* B, refeff_complex128* X, refeff_fms_form form,
                                    int32_t* status_out, int32_t* pivot_out);

/* ---- allocation-free dense solve ---------------------------------------- */

/* Device scratch reserved for refeff_complex_lu_solve_device_noalloc: one
 * static device array per device of this many bytes (24 MiB). */
#define REFEFF_FMS_NOALLOC_SCRATCH_BYTES (24u * 1024u * 1024u)

/* No counterpart in the reference: an allocation-free variant of
 * refeff_complex_lu_solve_batched (FP64 LU form) for callers that must not
 * allocate device memory -- a host whose device memory is fully reserved by
 * its own pool, or a multi-stream pipeline that cannot take the implicit
 * device-wide synchronisation of cudaFree.  Same elimination and results;
 * its scratch (padded systems, pivots, row moves, status words) is a static
 * device array of REFEFF_FMS_NOALLOC_SCRATCH_BYTES, never cudaMalloc.
 *
 * d_A: batch x (n x n), d_B / d_X: batch x (n x m), column-major device
 * buffers (d_X must not overlap d_A or d_B); d_status / d_pivot (optional,
 * device, batch entries) receive the per-system status code and 1-based
 * first zero pivot.  Per-system failures (a singular or non-finite system)
 * are reported through d_status only: the return code covers the arguments,
 * the scratch limit and the launches, so a caller that passes no d_status
 * gets no signal for a failed system.  Runs asynchronously on `stream` (NULL = legacy default
 * stream) on the calling thread's current device; results are ready when
 * the stream reaches them.  The scratch needed is about
 * batch * roundup(n, 32) * (n + m) * 16 bytes plus small pivot tables (one
 * system of n = 1200, m = 16 fits); a larger request returns
 * REFEFF_FMS_ERR_SCRATCH_LIMIT before anything runs.  m <= 64.
 * First call on each device: looks up the array's address
 * (cudaGetSymbolAddress) with that device current; make it before any
 * stream capture.  The array is shared by all calls on a device: calls whose
 * GPU work overlaps race on it, so order them on one stream or with events. */
int refeff_complex_lu_solve_device_noalloc(int n, int m, int batch, const refeff_complex128* d_A,
                                           const refeff_complex128* d_B, refeff_complex128* d_X, int32_t* d_status,
                                           int32_t* d_pivot, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* REFEFF_FMS_H */
