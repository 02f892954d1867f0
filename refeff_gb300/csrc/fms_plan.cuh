// Device-side plan of one FMS cluster (energy independent) and the launch
// entry points of the FMS kernels.
//
// Device state order: atoms are stored with the absorber (reference atom 0)
// moved to the END, so its states are the last m rows/columns of every
// system matrix.  Within an atom the reference order is kept
// (l = 0..lmax, m = -l..l, spin innermost; crates/refeff-core/src/state.rs:97-148).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

namespace rfx {

constexpr int kMaxL = 6;          // largest global lmax the kernels accept

// One solved block per potential of the range: rows [row, row + size) of the
// solution columns [col, col + size), packed at `pack` in each energy's output.
struct SolvedBlock {
  int row, col, size, pack;
};
constexpr int kBuildRowAtoms = 16;  // row atoms per build CTA

struct PlanDev {
  int N = 0;        // atoms
  int L = 0;        // global lmax
  int nsp = 1;      // spin channels
  int ispin = 0;    // spin selector (global.inp ispin)
  int npot = 0;     // potentials
  int n = 0;        // states
  int m = 0;        // absorber block width (states of the absorber atom)
  int ds = 0;       // small-d doubles per ordered pair (forward + backward)
  const float* pos = nullptr;        // [N][3] device order
  const int* atom_pot = nullptr;     // [N]
  const int* atom_off = nullptr;     // [N+1] first state of each atom (device order)
  const int* atom_lmax = nullptr;    // [N] per-atom l cutoff
  const double* sigsqr = nullptr;    // [N*N] (a2 + N*a1), device order
  double* pair_dist = nullptr;       // [N*N] (j + N*i), |R_i - R_j|        (written by launch_plan_geometry)
  double* pair_phi = nullptr;        // [N*N] azimuth of R_i - R_j           (written by launch_plan_geometry)
  double2* pair_eph = nullptr;       // [N*N*(4L+1)] e^{i mm (phi - pi)}, mm in [-2L, 2L] (launch_plan_geometry)
  double* pair_dsmall = nullptr;     // [N*N][ds] Wigner small-d tables      (written by launch_plan_geometry)
  // the same two tables as double-float pairs (hi, lo) for the refined form's
  // build, written by launch_plan_df_tables
  float2* pair_dsmall_df = nullptr;  // [N*N][ds]
  float4* pair_eph_df = nullptr;     // [N*N*(4L+1)] (re hi, im hi, re lo, im lo)
  const double* xnlm = nullptr;      // [(L+1)*(L+1)] xnlm(mu, l) at mu + (L+1)*l
  const double* xnlm_w = nullptr;    // [(L+1)*(L+1)] (2l+1) / xnlm(mu, l), same index
  const float2* xnlm_df = nullptr;   // the two tables above as double-float pairs (hi, lo)
  const float2* xnlm_w_df = nullptr;
  const double* t3p = nullptr;       // spin-orbit coefficients [l + (L+1)*((m+L) + (2L+1)*(s-1))]
  const double* t3m = nullptr;
  double rdirec2 = 0.0;              // direct-cutoff radius squared (Angstrom^2)
  // right-hand-side column of each device atom's states in B = G0[:, representatives]
  // (the representative of each potential in the solved range), -1 for other atoms
  const int* bcol = nullptr;         // [N]
};

// Per-batch matrix layout: [A | B] with A n x n and B n x m (column-major,
// leading dimension lda, matrix stride `stride` elements).
struct BatchLayout {
  int n = 0, m = 0, lda = 0;
  size_t stride = 0;
};

// status codes written by kernels (per matrix)
enum DevStatus : int {
  kDevOk = 0,
  kDevSingular = 1,      // exact zero pivot (info = 1 + pivot index in the aux word)
  kDevNonfinite = 2,     // non-finite wave number / phase / rho
  kDevZeroRho = 3,
  kDevNotConverged = 4,
  kDevTimeout = 5,
  kDevBreakdown = 6,     // iterative solver breakdown (zero divisor)
};

// Every kernel launch of the library calls this first; the total (including
// launches replayed inside CUDA graphs) is reported by refeff_fms_kernel_launches.
void count_launch();

// Kernel attributes set with cudaFuncSetAttribute apply to the calling
// thread's current device only, so every request is remembered per
// (device, kernel) under a lock.  The first request for a pair must come
// outside any stream capture: the library runs each batch shape un-captured
// once before it captures it.
// Raises the kernel's dynamic shared-memory limit to at least `bytes`.
cudaError_t ensure_smem_limit(const void* kernel, size_t bytes);
// Allows cluster sizes above the portable 8 CTAs for the kernel.
cudaError_t ensure_nonportable_clusters(const void* kernel);
// SM count of the current device (looked up once per device).
int current_sm_count();

// ---- geometry (once per plan) ----
void launch_plan_geometry(const PlanDev& P, cudaStream_t s);
// pair_dsmall_df / pair_eph_df from pair_dsmall / pair_eph (after launch_plan_geometry)
void launch_plan_df_tables(const PlanDev& P, cudaStream_t s);

// ---- system build (per energy batch) ----
// k: [E][nsp] double2; xphase: [E][nsp*(2L+1)*npot] double2 (column-major (nsp, 2L+1, npot)).
// Writes A (= I - G0 T) and B (= G0[:, absorber]) into M64 (and a float copy into M32 if non-null).
// With `scratch` (build_scratch_entries(P, E) entries of hank, E N^2 of hflag), the pair prefactors and
// Hankel tables are computed for the whole batch by one kernel first; without it, inside the build CTAs.
struct BuildScratch {
  double2* hank = nullptr;
  int* hflag = nullptr;
};
size_t build_scratch_entries(const PlanDev& P, int E);
void launch_build_system(const PlanDev& P, int E, const double2* k, const double2* xphase, const BatchLayout& lay,
                         double2* M64, float2* M32, int* status, cudaStream_t s, const BuildScratch* scratch = nullptr);
// Plain free propagator G0 (FP64, device state order) into G0[e * lay.stride + r + lay.lda * c].
void launch_build_g0(const PlanDev& P, int E, const double2* k, const BatchLayout& lay, double2* G0, int* status,
                     cudaStream_t s, const BuildScratch* scratch = nullptr);
// T table per state: t[(e * n + state) * 2 + band], band 0 = T(0, .), 1 = T(1, .).
void launch_t_table(const PlanDev& P, int E, const double2* xphase, double2* t, int* status, cudaStream_t s);

}  // namespace rfx
