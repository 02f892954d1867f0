// TEST INFRASTRUCTURE ONLY -- the CPU oracle for the pair mean-square
// displacement (sigma^2) table of the FMS stage under the correlated (idwopt 0)
// and classical (idwopt 3) Debye models.  Restated in FP64 as the reference
// computes it, with -ffp-contract=off like the rest of the oracle:
//   FEFF atwtd atomic weights (f32 data)   crates/refeff-core/src/atomic/tables.rs:10-19, 49-62
//   corrfn / corrfn2 (Debye correlation)   crates/refeff-core/src/debye/models.rs:88-132, 349-436
//   sigms / sigcl (path Debye-Waller)      crates/refeff-core/src/debye/models.rs:134-271
//   pair table                             crates/refeff-engine/src/fms.rs:4345-4433, 4849-4877, 4950-4957
// Only tests, smoke() and the benchmark's CPU baseline use this file.
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

namespace {

// FEFF pertab atwtd, Z = 1..139, as single-precision data (tables.rs:49-62).
const float kAtomicWeight[139] = {
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

enum Code { OK = 0, INVALID = 1, NOT_CONVERGED = 2, NONFINITE = 3, NARROW = 4, ZERO_LEG = 5 };

bool weight(int z, double& w) {
  if (z < 1 || z > 139) return false;
  w = double(kAtomicWeight[z - 1]);
  return true;
}

double quantum_integrand(double w, double x, double yinv) {
  if (w < 1.0e-20) return 2.0 * yinv;
  const double factor = x > 0.0 ? std::sin(w * x) / x : w;
  const double e = std::exp(-w / yinv);
  return factor * (1.0 + e) / (1.0 - e);
}

double classical_integrand(double w, double x, double yinv) {
  if (w < 1.0e-20) return 2.0 * yinv;
  const double factor = x > 0.0 ? std::sin(w * x) / x : w;
  return factor * 2.0 * yinv / w;
}

double relative_error(double cur, double prev) {
  if (cur == 0.0) return prev == 0.0 ? 0.0 : std::numeric_limits<double>::infinity();
  return std::fabs((cur - prev) / cur);
}

// One Richardson step on successive trapezoid sums over [0, 1], stopping on
// the relative change of the extrapolated value (models.rs:402-436).
int romberg(bool classical, double x, double yinv, double& out, int& iters) {
  auto f = [&](double w) { return classical ? classical_integrand(w, x, yinv) : quantum_integrand(w, x, yinv); };
  long long intervals = 1;
  double delta = 1.0;
  double prev_trap = (f(0.0) + f(1.0)) / 2.0;
  double prev_ext = prev_trap;
  for (int it = 1; it <= kRombergMaxIterations; ++it) {
    delta /= 2.0;
    double mid = -0.0;
    for (long long i = 1; i <= intervals; ++i) mid += f(double(2 * i - 1) * delta);
    const double trap = prev_trap / 2.0 + delta * mid;
    const double ext = (4.0 * trap - prev_trap) / 3.0;
    if (relative_error(ext, prev_ext) < kRombergTolerance) {
      out = ext;
      iters = it;
      return OK;
    }
    prev_trap = trap;
    prev_ext = ext;
    intervals *= 2;
  }
  return NOT_CONVERGED;
}

bool nonneg(double v) { return std::isfinite(v) && v >= 0.0; }
bool positive(double v) { return std::isfinite(v) && v > 0.0; }

int correlation(bool classical, double r, double thetad, double tk, int z1, int z2, double rsavg, double& out,
                int& iters) {
  if (!nonneg(r) || !positive(thetad) || !nonneg(tk) || !positive(rsavg)) return INVALID;
  double m1, m2;
  if (!weight(z1, m1) || !weight(z2, m2)) return INVALID;
  const double yinv = tk / thetad;
  const double kd = std::pow(9.0 * M_PI / 2.0, 1.0 / 3.0) / (rsavg * kBohrAngstrom);
  const double x = kd * r;
  const double factor = double(1.5f) * kCorrelationFactor / (thetad * std::sqrt(m1 * m2));
  double integral = 0.0;
  const int rc = romberg(classical, x, yinv, integral, iters);
  if (rc) return rc;
  out = factor * integral;
  return std::isfinite(out) ? OK : NONFINITE;
}

double dot3(const double* a, const double* b) {
  double s = -0.0;
  for (int i = 0; i < 3; ++i) s += a[i] * b[i];
  return s;
}

// sigms / sigcl over a path of `rows` positions (row-major rows x 3).
int debye_waller(bool classical, double tk, double thetad, double rsavg, int rows, const double* pos, const int* z,
                 double& out) {
  if (rows < 2) return INVALID;
  for (int i = 0; i < 3 * rows; ++i)
    if (!std::isfinite(pos[i])) return INVALID;
  double w;
  for (int i = 0; i < rows; ++i)
    if (!weight(z[i], w)) return INVALID;
  if (!nonneg(tk) || !positive(thetad) || !positive(rsavg)) return INVALID;
  auto dist = [&](int a, int b) {
    const double d[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
    return std::sqrt(dot3(d, d));
  };
  auto corr = [&](int a, int b, double& c) {
    int it = 0;
    return correlation(classical, dist(a, b), thetad, tk, z[a], z[b], rsavg, c, it);
  };
  const int nleg = rows - 1;
  double total = 0.0;
  for (int il = 1; il <= nleg; ++il)
    for (int jl = il; jl <= nleg; ++jl) {
      double cij, cimjm, cijm, cimj;
      int rc;
      if ((rc = corr(il, jl, cij)) || (rc = corr(il - 1, jl - 1, cimjm)) || (rc = corr(il, jl - 1, cijm)) ||
          (rc = corr(il - 1, jl, cimj)))
        return rc;
      double l1[3], l2[3];
      for (int c = 0; c < 3; ++c) {
        l1[c] = pos[3 * il + c] - pos[3 * (il - 1) + c];
        l2[c] = pos[3 * jl + c] - pos[3 * (jl - 1) + c];
      }
      const double n1 = std::sqrt(dot3(l1, l1)), n2 = std::sqrt(dot3(l2, l2));
      if (n1 == 0.0 || n2 == 0.0) return ZERO_LEG;
      const double proj = dot3(l1, l2) / (n1 * n2);
      double contribution = cij + cimjm - cijm - cimj;
      if (jl != il) contribution *= 2.0;
      total += contribution * proj;
    }
  out = total / 4.0;
  return std::isfinite(out) ? OK : NONFINITE;
}

bool narrow_nonneg(double v, float& out) {
  const float f = float(v);
  if (!(std::isfinite(v) && v >= 0.0 && std::isfinite(f))) return false;
  out = f;
  return true;
}

}  // namespace

extern "C" {

double oracle_atomic_weight(int z) {
  double w = 0.0;
  return weight(z, w) ? w : -1.0;
}

int oracle_debye_correlation(int classical, double r, double thetad, double tk, int z1, int z2, double rsavg,
                             double* out, int* iterations) {
  int it = 0;
  double v = 0.0;
  const int rc = correlation(classical != 0, r, thetad, tk, z1, z2, rsavg, v, it);
  if (out) *out = v;
  if (iterations) *iterations = it;
  return rc;
}

int oracle_debye_waller(int classical, double tk, double thetad, double rsavg, int rows, const double* pos,
                        const int* z, double* out) {
  double v = 0.0;
  const int rc = debye_waller(classical != 0, tk, thetad, rsavg, rows, pos, z, v);
  if (out) *out = v;
  return rc;
}

// The (N, N) pair table [atom2 + N*atom1] of the FMS stage: idwopt < 0 gives
// sig2g for every i != j pair, 0 the correlated and 3 the classical Debye
// model on the path (atom1, atom2, atom1).  pair64 (optional) receives the
// Debye term before sig2g is added and the sum narrowed.
int oracle_debye_sigma2_table(int idwopt, int n_atoms, const float* pos_xyz, const int* potentials, int n_potentials,
                              const int* atomic_numbers, double tk, double thetad, double rsavg, float sig2g_in,
                              float* out, double* pair64) {
  if (n_atoms < 0 || (idwopt >= 0 && idwopt != 0 && idwopt != 3)) return INVALID;
  float sig2g;
  if (!narrow_nonneg(double(sig2g_in), sig2g)) return NARROW;
  if (idwopt >= 0) {
    if (!positive(rsavg)) return INVALID;
    for (int p = 0; p < n_potentials; ++p)
      if (atomic_numbers[p] == 0) return INVALID;
  }
  const size_t N = size_t(n_atoms);
  for (size_t a2 = 0; a2 < N; ++a2)
    for (size_t a1 = 0; a1 < N; ++a1) {
      const size_t idx = a2 + N * a1;
      out[idx] = 0.0f;
      if (pair64) pair64[idx] = 0.0;
      if (a1 == a2) continue;
      double pair = 0.0;
      if (idwopt >= 0) {
        const int p1 = potentials[a1], p2 = potentials[a2];
        if (p1 < 0 || p2 < 0 || p1 >= n_potentials || p2 >= n_potentials) return INVALID;
        double path[9];
        for (int c = 0; c < 3; ++c) {
          path[c] = double(pos_xyz[3 * a1 + c]);
          path[3 + c] = double(pos_xyz[3 * a2 + c]);
          path[6 + c] = double(pos_xyz[3 * a1 + c]);
        }
        const int z[3] = {atomic_numbers[p1], atomic_numbers[p2], atomic_numbers[p1]};
        const int rc = debye_waller(idwopt == 3, tk, thetad, rsavg, 3, path, z, pair);
        if (rc) return rc;
      }
      if (pair64) pair64[idx] = pair;
      if (!narrow_nonneg(double(sig2g) + pair, out[idx])) return NARROW;
    }
  return OK;
}

}  // extern "C"
