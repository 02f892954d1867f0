// Pair mean-square displacement (sigma^2) table of the FMS stage under FEFF's
// correlated (idwopt 0, corrfn/sigms) and classical (idwopt 3, corrfn2/sigcl)
// Debye models, on the GPU: one thread per ordered atom pair.
//
// For the pair (atom1, atom2) the reference evaluates the path Debye-Waller
// factor of the closed path (atom1, atom2, atom1)
// (crates/refeff-engine/src/fms.rs:4849-4877), i.e. sigms over two legs
// (crates/refeff-core/src/debye/models.rs:181-271).  Its twelve correlation
// calls take three distinct values -- C(0; Z1, Z1), C(0; Z2, Z2) and
// C(r; Z1, Z2) -- because the path's rows 0 and 2 are the same atom and
// C(r; Za, Zb) is symmetric; each is one Richardson-extrapolated trapezoid
// integral over [0, 1] (models.rs:349-436).  The sums keep the reference's
// operation order, and every product that the compiler could fuse into an
// FMA is written with explicit round-to-nearest intrinsics, so the only
// difference from the reference's FP64 value is the last-place rounding of
// sin / exp; the table is then narrowed to f32 like the reference
// (fms.rs:4426-4427, 4950-4957).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/refeff_fms.h"
#include "fms_plan.cuh"
#include "host_internal.h"

namespace rfx {
namespace {

// FEFF pertab atwtd, Z = 1..139, single-precision data
// (crates/refeff-core/src/atomic/tables.rs:49-62).
__constant__ float c_atomic_weight[139] = {
    1.0079f, 4.0026f, 6.941f,  9.0122f, 10.81f,  12.01f,  14.007f, 15.999f, 18.998f, 20.18f,  22.9898f, 24.305f,
    26.982f, 28.086f, 30.974f, 32.064f, 35.453f, 39.948f, 39.09f,  40.08f,  44.956f, 47.90f,  50.942f,  52.00f,
    54.938f, 55.85f,  58.93f,  58.71f,  63.55f,  65.38f,  69.72f,  72.59f,  74.922f, 78.96f,  79.91f,   83.80f,
    85.47f,  87.62f,  88.91f,  91.22f,  92.91f,  95.94f,  98.91f,  101.07f, 102.90f, 106.40f, 107.87f,  112.40f,
    114.82f, 118.69f, 121.75f, 127.60f, 126.90f, 131.30f, 132.91f, 137.34f, 138.91f, 140.12f, 140.91f,  144.24f,
    145.0f,  150.35f, 151.96f, 157.25f, 158.92f, 162.50f, 164.93f, 167.26f, 168.93f, 173.04f, 174.97f,  178.49f,
    180.95f, 183.85f, 186.2f,  190.20f, 192.22f, 195.09f, 196.97f, 200.59f, 204.37f, 207.19f, 208.98f,  210.0f,
    210.0f,  222.0f,  223.0f,  226.0f,  227.0f,  232.04f, 231.0f,  238.03f, 237.05f, 244.0f,  243.0f,   247.0f,
    247.0f,  251.0f,  252.0f,  257.0f,  258.0f,  259.0f,  266.0f,  267.0f,  268.0f,  269.0f,  270.0f,   269.0f,
    278.0f,  281.0f,  282.0f,  285.0f,  286.0f,  289.0f,  289.0f,  293.0f,  294.0f,  294.0f,  315.0f,   320.0f,
    330.0f,  334.0f,  337.0f,  340.0f,  344.0f,  347.0f,  350.0f,  354.0f,  357.0f,  361.0f,  364.0f,   367.0f,
    371.0f,  374.0f,  378.0f,  381.0f,  385.0f,  388.0f,  392.0f};

constexpr double kBohrAngstrom = 0.529177249;
constexpr double kCorrelationFactor = double(48.50846f);
constexpr double kRombergTolerance = 1.0e-5;
constexpr int kRombergMaxIterations = 10;

// Per-pair failure codes, max-reduced into one word.
enum DebyeCode { kDebyeOk = 0, kDebyeZeroLeg = 1, kDebyeNotConverged = 2, kDebyeNonfinite = 3, kDebyeNarrow = 4 };

struct DebyeArgs {
  int n = 0;
  bool classical = false;
  const float* pos = nullptr;  // n x 3
  const int* pot = nullptr;    // n
  const int* z = nullptr;      // per potential
  double yinv = 0.0;           // tk / thetad
  double kd = 0.0;             // Debye wave number, 1/Angstrom
  double thetad = 0.0;
  float sig2g = 0.f;
  float* out = nullptr;        // n x n, [atom2 + n * atom1]
  double* pair64 = nullptr;    // optional: the Debye term before narrowing
  int* code = nullptr;
};

__device__ __forceinline__ double integrand(bool classical, double w, double x, double yinv) {
  if (w < 1.0e-20) return 2.0 * yinv;
  const double factor = x > 0.0 ? sin(__dmul_rn(w, x)) / x : w;
  if (classical) return __dmul_rn(__dmul_rn(factor, 2.0), yinv) / w;
  const double e = exp(-w / yinv);
  return __dmul_rn(factor, 1.0 + e) / (1.0 - e);
}

__device__ __forceinline__ double relative_error(double cur, double prev) {
  if (cur == 0.0) return prev == 0.0 ? 0.0 : __longlong_as_double(0x7ff0000000000000LL);
  return fabs((cur - prev) / cur);
}

// Debye correlation C(r; Z1, Z2): factor * integral (models.rs:349-383).
__device__ int correlation(const DebyeArgs& a, double r, double m1, double m2, double& out) {
  const double x = __dmul_rn(a.kd, r);
  long long intervals = 1;
  double delta = 1.0;
  double prev_trap = (integrand(a.classical, 0.0, x, a.yinv) + integrand(a.classical, 1.0, x, a.yinv)) / 2.0;
  double prev_ext = prev_trap;
  for (int it = 1; it <= kRombergMaxIterations; ++it) {
    delta /= 2.0;
    double mid = -0.0;
    for (long long i = 1; i <= intervals; ++i)
      mid = __dadd_rn(mid, integrand(a.classical, __dmul_rn(double(2 * i - 1), delta), x, a.yinv));
    const double trap = __dadd_rn(prev_trap / 2.0, __dmul_rn(delta, mid));
    const double ext = __dsub_rn(__dmul_rn(4.0, trap), prev_trap) / 3.0;
    if (relative_error(ext, prev_ext) < kRombergTolerance) {
      const double factor = __dmul_rn(1.5, kCorrelationFactor) / __dmul_rn(a.thetad, sqrt(__dmul_rn(m1, m2)));
      out = __dmul_rn(factor, ext);
      return isfinite(out) ? kDebyeOk : kDebyeNonfinite;
    }
    prev_trap = trap;
    prev_ext = ext;
    intervals *= 2;
  }
  return kDebyeNotConverged;
}

__device__ __forceinline__ double dot3(const double* u, const double* v) {
  double s = -0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) s = __dadd_rn(s, __dmul_rn(u[i], v[i]));
  return s;
}

__global__ void debye_table_kernel(DebyeArgs a) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long N = a.n;
  if (t >= N * N) return;
  const int a2 = int(t % N), a1 = int(t / N);
  if (a1 == a2) {
    a.out[t] = 0.f;
    if (a.pair64) a.pair64[t] = 0.0;
    return;
  }
  const double m1 = double(c_atomic_weight[a.z[a.pot[a1]] - 1]);
  const double m2 = double(c_atomic_weight[a.z[a.pot[a2]] - 1]);
  // path rows: P0 = atom1, P1 = atom2, P2 = atom1
  double leg[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) leg[c] = double(a.pos[3 * a2 + c]) - double(a.pos[3 * a1 + c]);
  const double r = sqrt(dot3(leg, leg));
  int code = kDebyeOk;
  double c11 = 0.0, c22 = 0.0, cr = 0.0;  // C(0; Z1, Z1), C(0; Z2, Z2), C(r; Z1, Z2)
  if (r == 0.0) code = kDebyeZeroLeg;
  if (!code) code = correlation(a, 0.0, m1, m1, c11);
  if (!code) code = correlation(a, 0.0, m2, m2, c22);
  if (!code) code = correlation(a, r, m1, m2, cr);
  double pair = 0.0;
  if (!code) {
    // legs: l1 = P1 - P0 = leg, l2 = P2 - P1 = -leg
    double neg[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) neg[c] = -leg[c];
    const double nrm = sqrt(dot3(leg, leg));
    const double p11 = dot3(leg, leg) / __dmul_rn(nrm, nrm);
    const double p12 = dot3(leg, neg) / __dmul_rn(nrm, nrm);
    const double p22 = dot3(neg, neg) / __dmul_rn(nrm, nrm);
    double total = 0.0;
    // (il, jl) = (1, 1): C(1,1) + C(0,0) - C(1,0) - C(0,1)
    total = __dadd_rn(total, __dmul_rn(c22 + c11 - cr - cr, p11));
    // (1, 2): 2 [C(1,2) + C(0,1) - C(1,1) - C(0,2)]
    total = __dadd_rn(total, __dmul_rn((cr + cr - c22 - c11) * 2.0, p12));
    // (2, 2): C(2,2) + C(1,1) - C(2,1) - C(1,2)
    total = __dadd_rn(total, __dmul_rn(c11 + c22 - cr - cr, p22));
    pair = total / 4.0;
    if (!isfinite(pair)) code = kDebyeNonfinite;
  }
  float v = 0.f;
  if (!code) {
    const double s = __dadd_rn(double(a.sig2g), pair);
    v = __double2float_rn(s);
    if (!(isfinite(s) && s >= 0.0 && isfinite(v))) code = kDebyeNarrow;
  }
  a.out[t] = v;
  if (a.pair64) a.pair64[t] = pair;
  if (code) atomicMax(a.code, code);
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, (n ? n : 1) * sizeof(T)); }
};

bool finite_nonneg(double v) { return std::isfinite(v) && v >= 0.0; }
bool finite_positive(double v) { return std::isfinite(v) && v > 0.0; }

}  // namespace
}  // namespace rfx

using namespace rfx;

extern "C" int refeff_fms_debye_sigma2_table(refeff_fms_context* ctx, int idwopt, int n_atoms,
                                             const float* positions_xyz, const int* potentials, int n_potentials,
                                             const int* atomic_numbers, double temperature, double debye_temperature,
                                             double average_norman_radius, float sig2g, float* table_out,
                                             double* debye_term_out) {
  if (!ctx || n_atoms < 0 || n_potentials < 1 || !table_out || (n_atoms > 0 && (!positions_xyz || !potentials)))
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (idwopt >= 0 && idwopt != 0 && idwopt != 3) {
    set_last_error(ctx, "only idwopt < 0, 0 (correlated Debye) and 3 (classical Debye) pair tables are built here");
    return REFEFF_FMS_ERR_UNSUPPORTED;
  }
  if (!(std::isfinite(sig2g) && sig2g >= 0.f)) {
    set_last_error(ctx, "FMS SIG2 is negative or non-finite");
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  const size_t N = size_t(n_atoms), NN = N * N;
  if (idwopt < 0) {  // fms.rs:4388: no Debye term, sig2g off the diagonal
    for (size_t a1 = 0; a1 < N; ++a1)
      for (size_t a2 = 0; a2 < N; ++a2) {
        table_out[a2 + N * a1] = a1 == a2 ? 0.f : sig2g;
        if (debye_term_out) debye_term_out[a2 + N * a1] = 0.0;
      }
    return REFEFF_FMS_OK;
  }
  // validate_fms_debye_damping_metadata (fms.rs:4879-4905), then the checks of
  // debye_waller_factor / debye_correlation (models.rs:190-193, 360-365)
  if (!atomic_numbers || !finite_positive(average_norman_radius)) {
    set_last_error(ctx, "FMS Debye damping requires a positive finite average Norman radius");
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  for (int p = 0; p < n_potentials; ++p)
    if (atomic_numbers[p] < 1 || atomic_numbers[p] > 139) {
      set_last_error(ctx, "FMS Debye damping requires an atomic number in 1..139 for potential " + std::to_string(p));
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    }
  if (!finite_nonneg(temperature) || !finite_positive(debye_temperature)) {
    set_last_error(ctx, "Debye model needs tk >= 0 and thetad > 0");
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  for (size_t i = 0; i < N; ++i) {
    if (potentials[i] < 0 || potentials[i] >= n_potentials) {
      set_last_error(ctx, "atom potential outside the potential table");
      return REFEFF_FMS_ERR_POTENTIAL_OUT_OF_RANGE;
    }
    for (int c = 0; c < 3; ++c)
      if (!std::isfinite(positions_xyz[3 * i + c])) return REFEFF_FMS_ERR_NONFINITE_COORDINATE;
  }
  if (N == 0) return REFEFF_FMS_OK;
  if (cudaSetDevice(context_device(ctx)) != cudaSuccess) return REFEFF_FMS_ERR_CUDA;
  cudaStream_t s = context_stream(ctx);
  DevBuf<float> dpos, dout;
  DevBuf<int> dpot, dz, dcode;
  DevBuf<double> dpair;
  if (dpos.alloc(3 * N) || dout.alloc(NN) || dpot.alloc(N) || dz.alloc(size_t(n_potentials)) || dcode.alloc(1) ||
      (debye_term_out && dpair.alloc(NN))) {
    set_last_error(ctx, "Debye table allocation failed");
    return REFEFF_FMS_ERR_OUT_OF_MEMORY;
  }
  DebyeArgs a;
  a.n = n_atoms;
  a.classical = idwopt == 3;
  a.pos = dpos.p;
  a.pot = dpot.p;
  a.z = dz.p;
  a.yinv = temperature / debye_temperature;
  a.kd = std::pow(9.0 * M_PI / 2.0, 1.0 / 3.0) / (average_norman_radius * kBohrAngstrom);
  a.thetad = debye_temperature;
  a.sig2g = sig2g;
  a.out = dout.p;
  a.pair64 = debye_term_out ? dpair.p : nullptr;
  a.code = dcode.p;
  if (cudaMemcpyAsync(dpos.p, positions_xyz, 3 * N * sizeof(float), cudaMemcpyHostToDevice, s) ||
      cudaMemcpyAsync(dpot.p, potentials, N * sizeof(int), cudaMemcpyHostToDevice, s) ||
      cudaMemcpyAsync(dz.p, atomic_numbers, size_t(n_potentials) * sizeof(int), cudaMemcpyHostToDevice, s) ||
      cudaMemsetAsync(dcode.p, 0, sizeof(int), s)) {
    set_last_error(ctx, "Debye table upload failed");
    return REFEFF_FMS_ERR_CUDA;
  }
  const int threads = 128;
  const unsigned blocks = unsigned((NN + threads - 1) / threads);
  count_launch();
  debye_table_kernel<<<blocks, threads, 0, s>>>(a);
  int code = 0;
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(table_out, dout.p, NN * sizeof(float), cudaMemcpyDeviceToHost, s) ||
      (debye_term_out && cudaMemcpyAsync(debye_term_out, dpair.p, NN * sizeof(double), cudaMemcpyDeviceToHost, s)) ||
      cudaMemcpyAsync(&code, dcode.p, sizeof(int), cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s)) {
    set_last_error(ctx, "Debye table kernel failed");
    return REFEFF_FMS_ERR_CUDA;
  }
  switch (code) {
    case kDebyeOk: return REFEFF_FMS_OK;
    case kDebyeZeroLeg:
      set_last_error(ctx, "two cluster atoms share a position (zero-length Debye path leg)");
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    case kDebyeNotConverged:
      set_last_error(ctx, "Debye correlation integral did not converge in 10 Richardson steps");
      return REFEFF_FMS_ERR_DEBYE;
    case kDebyeNonfinite:
      set_last_error(ctx, "Debye correlation produced a non-finite value");
      return REFEFF_FMS_ERR_DEBYE;
    default:
      set_last_error(ctx, "FMS pair sigsqr is negative, non-finite, or out of single-precision range");
      return REFEFF_FMS_ERR_DEBYE;
  }
}
