// Batched blocked complex LU with partial pivoting on augmented systems
// [A | B] (column-major, B in columns n .. n+m-1 of the same buffer), and the
// blocked triangular sweeps that reuse the stored factors.
#pragma once
#include <cuda_runtime.h>

#include <utility>
#include <vector>
#include "cplx.cuh"
#include "fms_plan.cuh"

namespace rfx {

// Panel geometry picked on the host for a given n / precision.
struct PanelConfig {
  int nb = 32;       // panel width (the outer block width of a two-level elimination)
  int cluster = 1;   // CTAs per matrix (thread-block cluster)
  int rpc_max = 0;   // rows per CTA at k = 0
  int smem = 0;      // dynamic smem bytes per CTA
  int pos_global = 0;  // row-position bookkeeping in global scratch (large n) instead of shared memory
  // two-level elimination (FP32, nb = 64): the cluster panels are inner_nb wide
  int inner_nb = 0, inner_cluster = 0, inner_rpc = 0, inner_smem = 0, inner_pos_global = 0;
  // two-level elimination with tensor cores: 64-column blocks taken in pairs,
  // one K = 128 trailing update per pair (set by the workspace when the fused
  // forward sweep, which replays the paired row moves, serves the system)
  int pair128 = 0;
};

// inner_pref (FP32): 0 picks by n (two-level from n = 512, 16-column inner
// panels first); 16 or 32 asks for two-level with that inner width first
// (from n = 128); 1 asks for single-level panels.
template <typename T> PanelConfig choose_panel(int n, int inner_pref = 0);

inline int panel_count(int n, int nb) { return (n + nb - 1) / nb; }

// Tensor-core trailing update (tc_update.cu) for the FP32 elimination.
constexpr int kTcBM = 128, kTcBN = 64;
constexpr int kTcKMax = 128;  // deepest update: two 64-column blocks at once
// bytes of the operand tile images for a batch of systems of order n with m right-hand sides
size_t tc_image_bytes(int n, int m, int batch);
// CUDA events around every tensor-core update kernel of one plan while `on`
// (plan profiling); each plan's workspace owns its own list.
struct KernelSpans {
  bool on = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> spans;
};
// Default poll budget of each mbarrier wait in the tensor-core update (the
// waits also give up after one second of %globaltimer).
constexpr long long kTcWaitPolls = 1LL << 26;
// C -= L21 U12 for elimination step k with tcgen05 MMAs (split TF32, FP32 accumulation).
// wait_polls bounds the waits of the producer, MMA and epilogue roles on each
// other; the final waits for copies and MMAs still in flight keep the default
// budget, so nothing is outstanding when a CTA exits.  spans (nullable)
// records CUDA events around the kernel while spans->on.
void tc_trailing_update(const BatchLayout& lay, int batch, int k, int kb, int col_end, float2* M, uint8_t* images,
                        int* err_flag, const int* skip, long long wait_polls, KernelSpans* spans, cudaStream_t s);

struct LuWork {
  uint8_t* tc_images = nullptr;  // operand images for the tensor-core update (FP32 only); null = CUDA cores
  int* tc_err = nullptr;         // set when a tensor-core wait timed out
  long long tc_wait_polls = kTcWaitPolls;  // poll budget of the role waits in the tensor-core update
  KernelSpans* tc_spans = nullptr;         // events around the tensor-core update launches (profiling)
  int* ipiv = nullptr;    // [batch][n]  LAPACK-style: row k+j was swapped with row ipiv
  int2* perm = nullptr;   // [batch][npanels][2*nb] (dst, src) row moves per panel
  int* nperm = nullptr;   // [batch][npanels]
  int* status = nullptr;  // [batch] DevStatus (max-reduced)
  int* info = nullptr;    // [batch] first zero pivot (1-based, 0 = none)
  // Two-level FP32 elimination: row moves of the inner panels (width IW = 32 or
  // 16), [batch][ceil(n/IW)][2 IW] and [batch][ceil(n/IW)]; the outer 64-column
  // blocks keep their composed moves in perm / nperm.
  int2* perm_in = nullptr;
  int* nperm_in = nullptr;
  // [batch][64 x 64] inverse of the outer block's unit lower L11 (two-level FP32
  // elimination); null = the block row is solved column by column
  float2* linv = nullptr;
  // row-position bookkeeping of the panel kernel when it does not fit in
  // shared memory: [batch][2n] ints (row2pos, pos2row)
  int* pos_scratch = nullptr;
  int npanels = 0;
  int nb = 0;
  // the elimination paired its 64-column blocks (PanelConfig::pair128): the
  // second block's row moves were also applied to the first block's L, so a
  // forward sweep applies both blocks' moves before solving the pair
  int pair128 = 0;
};

// Elimination of the whole augmented system: after it, columns [0, n) hold
// L\U and columns [n, n+m) hold Y = L^-1 P B.
template <typename T>
cudaError_t lu_eliminate(const PanelConfig& pc, const BatchLayout& lay, int batch, cplx<T>* M, const LuWork& w,
                         cudaStream_t s);

// Forward sweep on the right-hand-side columns [n, n+m) only (new RHS):
// Y = L^-1 P R with the stored per-panel row moves.
// `skip` (nullable, per matrix): matrices with skip[b] != 0 are left untouched.
template <typename T>
void lu_forward_rhs(const PanelConfig& pc, const BatchLayout& lay, int batch, cplx<T>* M, const LuWork& w,
                    const int* skip, cudaStream_t s);

// Backward sweep on the RHS columns: X = U^-1 Y (in place).
template <typename T>
void lu_backward_rhs(const PanelConfig& pc, const BatchLayout& lay, int batch, cplx<T>* M, const int* skip,
                     cudaStream_t s);

// gg from the eliminated [U | Y]: solve U[n-m:, n-m:] X = Y[n-m:, :] (m x m,
// upper triangular) and write X (FP64, column-major m x m) per matrix.
template <typename T>
void launch_absorber_solve(const BatchLayout& lay, int batch, const cplx<T>* M, double2* gg, const int* status,
                           cudaStream_t s);

// FP64 refinement helpers.  X64 and R are n x m per matrix with leading
// dimension lay.lda and matrix stride lay.lda * m.
// The FP64 system [A | B] of the refined form is stored as hi/lo float pairs
// (float4 per entry, see split_hi_lo).
// R = B - A * X64 (double-float accumulation) and per matrix rnorm = max |R|,
// bnorm = max |B| (|re|+|im|); matrices with skip[b] != 0 are left untouched.
// Whole forward / backward sweeps of the right-hand-side columns in one launch
// (sweeps.cu); false when the right-hand sides do not fit in shared memory,
// in which case nothing was launched.
bool fused_forward_sweep(int nb, const BatchLayout& lay, int batch, float2* M, const LuWork& w, const int* skip,
                         cudaStream_t s);
bool fused_backward_sweep(int nb, const BatchLayout& lay, int batch, float2* M, const int* skip, cudaStream_t s);
// Whether the fused sweeps above serve systems of this layout (their right-hand
// sides fit in shared memory).
bool fused_sweep_available(int nb, const BatchLayout& lay);

// The refinement residual on the tensor cores (tc_residual.cu): scratch for the
// digit slots of X (the tensor-core update's operand images, unused while the
// residual runs), the error flag a timed-out wait raises, the role-wait budget.
struct ResidualTc {
  uint8_t* images = nullptr;
  size_t bytes = 0;
  int* err = nullptr;
  long long polls = kTcWaitPolls;
};
size_t residual_tc_image_bytes(int n, int batch);
// R = B - A X (A, B as hi/lo float4, X FP64) from exact digit products on the
// bf16 tensor path, one pass per 16 right-hand sides; false (nothing launched)
// when the scratch is short.
bool launch_residual_tc(const BatchLayout& lay, int batch, const float4* Ms, const double2* X64, const ResidualTc& tc,
                        double2* R, unsigned long long* rnorm_bits, unsigned long long* bnorm_bits, const int* skip,
                        cudaStream_t s);
// R = B - A X and max |r|, max |b| per system: on the tensor cores when tc is
// given and serves the shape, else in double-float (Dot2) on the FP32 pipes.
void launch_residual(const BatchLayout& lay, int batch, const float4* Ms, const double2* X64, float4* Xsplit,
                     double2* R, unsigned long long* rnorm_bits, unsigned long long* bnorm_bits, const int* skip,
                     cudaStream_t s, const ResidualTc* tc = nullptr);
// In place: M (double2 entries) -> hi/lo float4 entries, M32 <- hi (for the dense solve API).
void launch_split_system(const BatchLayout& lay, int batch, double2* M, float2* M32, cudaStream_t s);
// RHS columns of M32 <- float(R / rnorm_b)
void launch_residual_to_rhs32(const BatchLayout& lay, int batch, const double2* R,
                              const unsigned long long* rnorm_bits, float2* M32, const int* skip, cudaStream_t s);
// X64 += D32 * rnorm_b (D32 = RHS columns of M32); with init, X64 = D32.
// When dnorm/xnorm are given, max |correction| and max |X| are accumulated per matrix.
void launch_accumulate_correction(const BatchLayout& lay, int batch, const float2* M32,
                                  const unsigned long long* rnorm_bits, double2* X64, bool init, const int* skip,
                                  unsigned long long* dnorm_bits, unsigned long long* xnorm_bits, cudaStream_t s);
// Refinement stopping rule (see ir_check_kernel): done[b] = 1 converged, 2 stalled.
void launch_ir_check(int batch, const unsigned long long* rnorm_bits, const unsigned long long* bnorm_bits,
                     const unsigned long long* dnorm_bits, const unsigned long long* xnorm_bits, double tol,
                     int* done, int* iters, double* relres, double* dprev, cudaStream_t s);
// out[b][pack + r + size * c] = X64 block entries (zero where status[b] != 0);
// per_matrix = the packed size of one matrix's blocks.
void launch_extract_blocks(const BatchLayout& lay, int batch, const double2* X64, const SolvedBlock* blocks, int nblocks,
                           int per_matrix, double2* out, const int* status, cudaStream_t s);
// gg (m x m per matrix) = rows [n-m, n) of X64
void launch_extract_absorber(const BatchLayout& lay, int batch, const double2* X64, double2* gg, cudaStream_t s);
// X64 = RHS columns of M64 (for the FP64 full solve)
void launch_copy_rhs64(const BatchLayout& lay, int batch, const double2* M64, double2* X64, cudaStream_t s);

}  // namespace rfx
