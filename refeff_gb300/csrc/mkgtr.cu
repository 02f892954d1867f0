// MKGTR: the step after the FMS solve that folds each energy's absorber block
// gg into the trace spectrum gtr(E).
//
//   transition B matrix (FEFF bcoef)   crates/refeff-core/src/angular/transition.rs:9-565
//     with cwig3j / rotwig             crates/refeff-core/src/angular/wigner.rs:7-184
//   trace (FEFF getgtr)                crates/refeff-core/src/fms/mkgtr.rs:790-952
//
// The B matrix is energy independent and tiny: it is built once on the host
// in FP64, exactly as the reference builds it.  Its non-zero entries are then
// compiled into a flat term list (row, column, transition/spin pair, value),
// and the GPU reduces, per energy and spectrum, the sum over the list of
// gg(row, col) * b * rkk(k1, s1) * rkk(k2, s2).  The kernel reads gg with an
// arbitrary leading dimension and energy stride, so it runs directly on the
// scattering tables the FMS solve leaves in device memory.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/refeff_fms.h"
#include "cplx.cuh"
#include "fms_plan.cuh"
#include "host_internal.h"

namespace rfx {
namespace {

using zc = std::complex<double>;

// ---------------------------------------------------------------------------
// angular algebra (host, FP64)
// ---------------------------------------------------------------------------

// Rust's f64::powi lowers to the integer power by squaring (compiler-rt
// __powidf2); the rotation matrices use it for cos/sin powers.
double powi_sq(double a, int b) {
  const bool recip = b < 0;
  double r = 1.0;
  while (true) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? 1.0 / r : r;
}

const double* log_factorials() {
  static const std::vector<double> t = [] {
    std::vector<double> v(59, 0.0);
    for (int i = 1; i <= 58; ++i) v[size_t(i)] = v[size_t(i) - 1] + std::log(double(i));
    return v;
  }();
  return t.data();
}

double parity(int e) { return (e % 2 == 0) ? 1.0 : -1.0; }

// Wigner 3j symbol by the Racah sum over log-factorials; arguments are
// multiplied by `sc` (1 for integers, 2 for half-integers).
double threej(int j1, int j2, int j3, int m1, int m2, int sc) {
  const double* lf = log_factorials();
  const int m3 = -m1 - m2;
  if (std::abs(m1) + std::abs(m2) == 0 && (j1 + j2 + j3) % (2 * sc) != 0) return 0.0;
  const int raw[12] = {j1 + j2 - j3, j2 + j3 - j1, j3 + j1 - j2, j1 + m1, j1 - m1, j2 + m2,
                       j2 - m2,      j3 + m3,      j3 - m3,      j1 + j2 + j3 + sc, j2 - j3 - m1, j1 - j3 + m2};
  int a[12];
  for (int i = 0; i < 12; ++i) {
    if (i < 10 && raw[i] < 0) return 0.0;
    a[i] = raw[i] / sc;
  }
  const int lo = std::max(0, std::max(a[10], a[11]));
  const int hi = std::min(a[0], std::min(a[4], a[5]));
  if (lo > hi) return 0.0;
  double half = -lf[a[9]];
  for (int i = 0; i < 9; ++i) half += lf[a[i]];
  half /= 2.0;
  double sum = 0.0, sg = parity(lo);
  for (int k = lo; k <= hi; ++k) {
    const double den = lf[k] + lf[a[0] - k] + lf[a[4] - k] + lf[a[5] - k] + lf[k - a[10]] + lf[k - a[11]];
    sum += sg * std::exp(half - den);
    sg = -sg;
  }
  return ((j1 - j2 - m3) % (2 * sc) != 0) ? -sum : sum;
}

// Wigner small-d d^{j}_{m1 m2}(beta) by the explicit sum, arguments scaled by `sc`;
// the four symmetry cases reduce to m1' >= |m2'|.
double small_d(double beta, int jj, int m1, int m2, int sc) {
  const double* lf = log_factorials();
  int a1 = m1, a2 = m2;
  double sg = 1.0;
  if (m1 >= 0 && std::abs(m1) >= std::abs(m2)) {
  } else if (m2 >= 0 && std::abs(m2) >= std::abs(m1)) {
    a1 = m2; a2 = m1; beta = -beta;
  } else if (m1 <= 0 && std::abs(m1) >= std::abs(m2)) {
    a1 = -m1; a2 = -m2; sg = parity((m1 - m2) / sc);
  } else {
    a1 = -m2; a2 = -m1; beta = -beta; sg = parity((m2 - m1) / sc);
  }
  const double c = std::cos(beta / 2.0), s = std::sin(beta / 2.0);
  double total = 0.0;
  for (int t = a1 - a2; t <= jj - a2; t += sc) {
    double f = (lf[(jj + a1) / sc] / 2.0 + lf[(jj - a1) / sc] / 2.0) + lf[(jj + a2) / sc] / 2.0 +
               lf[(jj - a2) / sc] / 2.0;
    f -= lf[(jj + a1 - t) / sc];
    f -= lf[(jj - a2 - t) / sc];
    f -= lf[t / sc];
    f -= lf[(a2 - a1 + t) / sc];
    const double coef = parity(t / sc) * std::exp(f);
    const int pc = (2 * jj + a1 - a2 - 2 * t) / sc, ps = (2 * t - a1 + a2) / sc;
    double term = coef;
    if (pc != 0 && ps != 0) term = coef * powi_sq(c, pc) * powi_sq(s, ps);
    else if (pc != 0) term = coef * powi_sq(c, pc);
    else if (ps != 0) term = coef * powi_sq(s, ps);
    total += term;
  }
  return sg * total;
}

zc i_pow(int e) {
  static const zc u[4] = {zc(1, 0), zc(0, 1), zc(-1, 0), zc(0, -1)};
  return u[((e % 4) + 4) % 4];
}

// B(m2, s2, k2, m1, s1, k1), magnetic numbers shifted by lmax, column-major
// like the reference's Array6 (2L+1, 2, 8, 2L+1, 2, 8).
struct TransitionMatrix {
  int lmax = 0, nm = 1;
  std::vector<zc> v;
  int jind[8], lind[8], kind[8];
  void resize(int L) {
    lmax = L;
    nm = 2 * L + 1;
    v.assign(size_t(nm) * 2 * 8 * nm * 2 * 8, zc(0.0, 0.0));
  }
  zc& operator()(int m2, int s2, int k2, int m1, int s1, int k1) {
    return v[size_t(m2 + lmax) + size_t(nm) * (s2 + 2 * (k2 + 8 * (size_t(m1 + lmax) + size_t(nm) * (s1 + 2 * k1))))];
  }
};

// Final-state channels of the core hole kappa: slots 1-3 the dipole
// (kappa' = kappa-1, -kappa, kappa+1), slots 4-8 the quadrupole / magnetic
// dipole ladder |kappa| - 2 .. |kappa| + 2; unused slots carry l = -1.
void transition_channels(int kinit, int multipole, int lmax, TransitionMatrix& T) {
  for (int d = -1; d <= 1; ++d) {
    int kappa = d == 0 ? -kinit : kinit + d;
    int j = std::abs(kappa), l = kappa <= 0 ? std::abs(kappa) - 1 : kappa;
    if (l > lmax) { j = 0; l = -1; kappa = 0; }
    T.jind[d + 1] = j; T.lind[d + 1] = l; T.kind[d + 1] = kappa;
  }
  for (int d = -2; d <= 2; ++d) {
    int j = std::max(0, std::abs(kinit) + d);
    int kappa = j;
    if ((kinit < 0 && std::abs(d) != 1) || (kinit > 0 && std::abs(d) == 1)) kappa = -j;
    int l = kappa <= 0 ? -kappa - 1 : kappa;
    if (l > lmax || multipole == 0 || (multipole == 1 && std::abs(d) == 2)) { j = 0; l = -1; kappa = 0; }
    T.jind[d + 5] = j; T.lind[d + 5] = l; T.kind[d + 5] = kappa;
  }
}

void polarized_matrix(TransitionMatrix& T, int kinit, int multipole, double angks, const zc ptz[3][3]) {
  const int L = T.lmax, nm = T.nm, ne = nm + 1;
  // tables indexed like the reference's flat scratch arrays (magnetic + lmax)
  std::vector<double> t3(size_t(8 * 2 * ne), 0.0), x3(size_t(8 * 3 * ne), 0.0), q(size_t(ne * nm * 2 * 8), 0.0);
  std::vector<zc> P(size_t(ne * 8 * ne * 8)), Tm(size_t(ne * 8 * nm * 2 * 8));
  auto T3 = [&](int k, int s, int m) -> double& { return t3[size_t((k * 2 + s) * ne + m + L)]; };
  auto X3 = [&](int k, int p, int m) -> double& { return x3[size_t((k * 3 + p + 1) * ne + m + L)]; };
  auto Q = [&](int mj, int ml, int s, int k) -> double& { return q[size_t((((mj + L) * nm + ml + L) * 2 + s) * 8 + k)]; };
  auto PM = [&](int m1, int k1, int m2, int k2) -> zc& { return P[size_t((((m1 + L) * 8 + k1) * ne + m2 + L) * 8 + k2)]; };
  auto TM = [&](int mj, int k2, int ml, int s, int k1) -> zc& {
    return Tm[size_t(((((mj + L) * 8 + k2) * nm + ml + L) * 2 + s) * 8 + k1)];
  };
  const int* J = T.jind;
  const int* Lk = T.lind;
  for (int k = 0; k < 8; ++k) {
    if (J[k] <= 0) continue;
    for (int mp = 1 - J[k]; mp <= J[k]; ++mp) {
      for (int s = 0; s < 2; ++s) {
        const int a = 2 * Lk[k], b = 1, c = 2 * J[k] - 1, ma = 2 * (mp - s), mb = 2 * s - 1;
        const double w = std::sqrt(double(c + 1)) * threej(a, b, c, ma, mb, 2);
        T3(k, s, mp) = (((b - a - ma - mb) / 2) % 2 != 0) ? -w : w;
      }
      const int jq = (k >= 3 && multipole == 2) ? 4 : 2;
      for (int p = -1; p <= 1; ++p) X3(k, p, mp) = threej(2 * J[k] - 1, jq, 2 * std::abs(kinit) - 1, 1 - 2 * mp, 2 * p, 2);
    }
  }
  for (int k = 0; k < 8; ++k) {
    if (Lk[k] < 0 || J[k] <= 0) continue;
    for (int s = 0; s < 2; ++s)
      for (int ml = -Lk[k]; ml <= Lk[k]; ++ml)
        for (int mj = 1 - J[k]; mj <= J[k]; ++mj)
          Q(mj, ml, s, k) = small_d(angks, 2 * J[k] - 1, 2 * mj - 1, 2 * (ml + s) - 1, 2) * T3(k, s, ml + s);
  }
  for (int k2 = 0; k2 < 8; ++k2) {
    if (J[k2] <= 0) continue;
    for (int m2 = 1 - J[k2]; m2 <= J[k2]; ++m2)
      for (int k1 = 0; k1 < 8; ++k1) {
        if (J[k1] <= 0) continue;
        for (int m1 = 1 - J[k1]; m1 <= J[k1]; ++m1) {
          if (std::abs(m2 - m1) > 2) continue;
          zc acc(0.0, 0.0);
          for (int pp = -1; pp <= 1; ++pp)
            for (int p = -1; p <= 1; ++p) {
              if (m1 - p != m2 - pp) continue;
              double sg = 1.0;
              if (multipole == 1 && p > 0 && k1 >= 3) sg = -sg;
              if (multipole == 1 && pp > 0 && k2 >= 3) sg = -sg;
              acc += ptz[p + 1][pp + 1] * (sg * X3(k1, p, m1) * X3(k2, pp, m2));
            }
          double sg = ((J[k1] - J[k2]) % 2 != 0) ? -1.0 : 1.0;
          if (k2 < 3) sg = -sg;
          acc *= sg * i_pow(Lk[k2] - Lk[k1]);
          PM(m1, k1, m2, k2) = acc;
        }
      }
  }
  for (int k1 = 0; k1 < 8; ++k1) {
    if (Lk[k1] < 0 || J[k1] <= 0) continue;
    for (int s = 0; s < 2; ++s)
      for (int ml = -Lk[k1]; ml <= Lk[k1]; ++ml)
        for (int k2 = 0; k2 < 8; ++k2) {
          if (J[k2] <= 0) continue;
          for (int mj = 1 - J[k2]; mj <= J[k2]; ++mj) {
            zc acc(0.0, 0.0);
            for (int mp = 1 - J[k1]; mp <= J[k1]; ++mp) acc += PM(mj, k2, mp, k1) * Q(mp, ml, s, k1);
            TM(mj, k2, ml, s, k1) = acc;
          }
        }
  }
  for (int k1 = 0; k1 < 8; ++k1) {
    if (Lk[k1] < 0) continue;
    for (int s1 = 0; s1 < 2; ++s1)
      for (int ml1 = -Lk[k1]; ml1 <= Lk[k1]; ++ml1)
        for (int k2 = 0; k2 < 8; ++k2) {
          if (Lk[k2] < 0 || J[k2] <= 0) continue;
          for (int s2 = 0; s2 < 2; ++s2)
            for (int ml2 = -Lk[k2]; ml2 <= Lk[k2]; ++ml2) {
              zc acc(0.0, 0.0);
              for (int mj = 1 - J[k2]; mj <= J[k2]; ++mj) acc += Q(mj, ml2, s2, k2) * TM(mj, k2, ml1, s1, k1);
              T(ml2, s2, k2, ml1, s1, k1) = acc;
            }
        }
  }
}

int build_transition_matrix(int lmax, int kinit, int polarization, const zc ptz[3][3], int multipole, bool trace,
                            int spin, int nsp, double angks, TransitionMatrix& T) {
  if (nsp <= 0 || lmax < 0 || lmax > 24) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      if (!std::isfinite(ptz[r][c].real()) || !std::isfinite(ptz[r][c].imag())) return REFEFF_FMS_ERR_NONFINITE_INPUT;
  T.resize(lmax);
  transition_channels(kinit, multipole, lmax, T);
  if (polarization == 0) {
    // isotropic average: diagonal, 1 / (2 (2l+1) degeneracy), dipole slots negative
    for (int k = 0; k < 8; ++k) {
      const int l = T.lind[k];
      if (l < 0) continue;
      double w = 0.5 / (2.0 * double(l) + 1.0) / ((multipole == 2 && k >= 3) ? 5.0 : 3.0);
      if (k < 3) w = -w;
      for (int s = 0; s < 2; ++s)
        for (int m = -l; m <= l; ++m) T(m, s, k, m, s, k) = zc(w, 0.0);
    }
  } else {
    polarized_matrix(T, kinit, multipole, angks, ptz);
  }
  if (trace) {
    for (int k1 = 0; k1 < 8; ++k1)
      for (int s1 = 0; s1 < 2; ++s1)
        for (int k2 = 0; k2 < 8; ++k2)
          for (int s2 = 0; s2 < 2; ++s2) {
            if (T.lind[k1] != T.lind[k2] || s1 != s2) {
              T(0, s2, k2, 0, s1, k1) = zc(0.0, 0.0);
              continue;
            }
            for (int m = 1; m <= T.lind[k1]; ++m) {
              const zc add = T(-m, s1, k2, -m, s1, k1) + T(m, s1, k2, m, s1, k1);
              T(0, s1, k2, 0, s1, k1) += add;
            }
          }
  }
  const bool add_up = spin == 0, copy_up = spin == 2 || (spin == 1 && nsp == 1);
  if (add_up || copy_up)
    for (int k1 = 0; k1 < 8; ++k1) {
      if (T.lind[k1] < 0) continue;
      for (int k2 = 0; k2 < 8; ++k2) {
        if (T.lind[k2] < 0) continue;
        for (int m1 = -T.lind[k1]; m1 <= T.lind[k1]; ++m1)
          for (int m2 = -T.lind[k2]; m2 <= T.lind[k2]; ++m2) {
            const zc up = T(m2, 1, k2, m1, 1, k1);
            zc& dn = T(m2, 0, k2, m1, 0, k1);
            dn = add_up ? dn + up : up;
          }
      }
    }
  return REFEFF_FMS_OK;
}

// ---------------------------------------------------------------------------
// trace on the GPU
// ---------------------------------------------------------------------------

struct TraceTerm {
  int row, col;
  int r1, r2;  // rkk slots (k + 8 s) of the two transitions
  double2 b;
};

constexpr int kTraceThreads = 256;

// One CTA per (energy, spectrum): sum over the spectrum's term list in FP64.
__global__ void __launch_bounds__(kTraceThreads) mkgtr_trace_kernel(
    int n_energies, const double2* __restrict__ gg, long long ld, long long energy_stride,
    const double2* __restrict__ rkk, const TraceTerm* __restrict__ terms,
    const int* __restrict__ term_off, int n_spectra, double2* __restrict__ traces, int* __restrict__ bad) {
  const int e = blockIdx.x, sp = blockIdx.y;
  const double2* g = gg + size_t(e) * size_t(energy_stride);
  const int t0 = term_off[sp], t1 = term_off[sp + 1];
  double sx = 0.0, sy = 0.0;
  int nonfinite = 0;
  for (int t = t0 + int(threadIdx.x); t < t1; t += kTraceThreads) {
    const TraceTerm tm = terms[t];
    const double2 gv = g[size_t(tm.row) + size_t(ld) * size_t(tm.col)];
    const double2 a = rkk[size_t(e) + size_t(n_energies) * size_t(tm.r1)];
    const double2 c = rkk[size_t(e) + size_t(n_energies) * size_t(tm.r2)];
    if (!cfinite(gv) || !cfinite(a) || !cfinite(c)) nonfinite = 1;
    const double2 v = cmul(cmul(cmul(gv, tm.b), a), c);
    sx += v.x;
    sy += v.y;
  }
  __shared__ double rx[kTraceThreads / 32], ry[kTraceThreads / 32];
  __shared__ int rb;
  if (threadIdx.x == 0) rb = 0;
  __syncthreads();
  if (nonfinite) atomicOr(&rb, 1);
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { rx[w] = sx; ry[w] = sy; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tx = 0.0, ty = 0.0;
    for (int i = 0; i < kTraceThreads / 32; ++i) { tx += rx[i]; ty += ry[i]; }
    traces[size_t(sp) + size_t(n_spectra) * e] = make_double2(tx, ty);
    if (rb || !isfinite(tx) || !isfinite(ty)) atomicExch(bad, 1);
  }
}

// Flattens the transition matrices into per-spectrum term lists.
int compile_terms(int n_spectra, int lmax, const int32_t* lind, const refeff_complex128* bmat, int dim, int nsp,
                  std::vector<TraceTerm>& terms, std::vector<int>& off) {
  const int nm = 2 * lmax + 1;
  const size_t bsz = size_t(nm) * 2 * 8 * nm * 2 * 8;
  terms.clear();
  off.assign(size_t(n_spectra) + 1, 0);
  for (int sp = 0; sp < n_spectra; ++sp) {
    const int32_t* li = lind + 8 * sp;
    const refeff_complex128* B = bmat + bsz * size_t(sp);
    for (int k1 = 0; k1 < 8; ++k1) {
      if (li[k1] < 0) continue;
      if (li[k1] > lmax) return REFEFF_FMS_ERR_INVALID_ANGULAR_LIMIT;
      for (int s1 = 0; s1 < nsp; ++s1)
        for (int k2 = 0; k2 < 8; ++k2) {
          if (li[k2] < 0) continue;
          if (li[k2] > lmax) return REFEFF_FMS_ERR_INVALID_ANGULAR_LIMIT;
          for (int s2 = 0; s2 < nsp; ++s2)
            for (int m1 = -li[k1]; m1 <= li[k1]; ++m1) {
              const int row = (li[k1] * li[k1] + li[k1] + m1) * nsp + s1;
              for (int m2 = -li[k2]; m2 <= li[k2]; ++m2) {
                const int col = (li[k2] * li[k2] + li[k2] + m2) * nsp + s2;
                if (row >= dim || col >= dim) return REFEFF_FMS_ERR_INVALID_ANGULAR_LIMIT;
                const refeff_complex128 b =
                    B[size_t(m2 + lmax) + size_t(nm) * (s2 + 2 * (k2 + 8 * (size_t(m1 + lmax) + size_t(nm) * (s1 + 2 * k1))))];
                if (!std::isfinite(b.re) || !std::isfinite(b.im)) return REFEFF_FMS_ERR_NONFINITE_INPUT;
                if (b.re == 0.0 && b.im == 0.0) continue;  // contributes exactly zero
                terms.push_back({row, col, k1 + 8 * s1, k2 + 8 * s2, make_double2(b.re, b.im)});
              }
            }
        }
    }
    off[size_t(sp) + 1] = int(terms.size());
  }
  return REFEFF_FMS_OK;
}

template <typename T>
struct Scratch {
  T* p = nullptr;
  ~Scratch() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
};

int run_trace(refeff_fms_context* ctx, int n_energies, const double2* d_gg, long long ld, long long energy_stride,
              const double2* d_rkk, int n_spectra, const std::vector<TraceTerm>& terms, const std::vector<int>& off,
              double2* d_traces, cudaStream_t s, bool sync_check) {
  Scratch<TraceTerm> dt;
  Scratch<int> doff, dbad;
  if (dt.alloc(terms.size()) || doff.alloc(off.size()) || dbad.alloc(1)) {
    set_last_error(ctx, "trace scratch allocation failed");
    return REFEFF_FMS_ERR_OUT_OF_MEMORY;
  }
  if (cudaMemcpyAsync(dt.p, terms.data(), terms.size() * sizeof(TraceTerm), cudaMemcpyHostToDevice, s) ||
      cudaMemcpyAsync(doff.p, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, s) ||
      cudaMemsetAsync(dbad.p, 0, sizeof(int), s)) {
    set_last_error(ctx, "trace upload failed");
    return REFEFF_FMS_ERR_CUDA;
  }
  count_launch();
  mkgtr_trace_kernel<<<dim3(unsigned(n_energies), unsigned(n_spectra)), kTraceThreads, 0, s>>>(
      n_energies, d_gg, ld, energy_stride, d_rkk, dt.p, doff.p, n_spectra, d_traces, dbad.p);
  int bad = 0;
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(&bad, dbad.p, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    set_last_error(ctx, "trace kernel failed");
    return REFEFF_FMS_ERR_CUDA;
  }
  if (sync_check && bad) {
    set_last_error(ctx, "non-finite gg, rkk or trace value");
    return REFEFF_FMS_ERR_NONFINITE_INPUT;
  }
  return bad ? REFEFF_FMS_ERR_NONFINITE_INPUT : REFEFF_FMS_OK;
}

}  // namespace

// shared with the file seam
int mkgtr_transition_matrix(int lmax, int kinit, int polarization, const refeff_complex128* ptz9, int multipole,
                            int trace_orbital, int spin, int nsp, double angks, refeff_complex128* out,
                            int32_t* lind, int32_t* kiind) {
  zc ptz[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) ptz[r][c] = ptz9 ? zc(ptz9[3 * r + c].re, ptz9[3 * r + c].im) : zc(0.0, 0.0);
  TransitionMatrix T;
  const int rc = build_transition_matrix(lmax, kinit, polarization, ptz, multipole, trace_orbital != 0, spin, nsp,
                                         angks, T);
  if (rc) return rc;
  if (out)
    for (size_t i = 0; i < T.v.size(); ++i) out[i] = {T.v[i].real(), T.v[i].imag()};
  for (int k = 0; k < 8; ++k) {
    if (lind) lind[k] = T.lind[k];
    if (kiind) kiind[k] = T.kind[k];
  }
  return REFEFF_FMS_OK;
}

}  // namespace rfx

using namespace rfx;

extern "C" int refeff_fms_transition_matrix(int lmax, int initial_kappa, int polarization,
                                            const refeff_complex128* polarization_tensor, int multipole,
                                            int trace_orbital, int spin, int spin_channels, double spin_vector_angle,
                                            refeff_complex128* bmat_out, int32_t* lind_out, int32_t* kiind_out) {
  return mkgtr_transition_matrix(lmax, initial_kappa, polarization, polarization_tensor, multipole, trace_orbital,
                                 spin, spin_channels, spin_vector_angle, bmat_out, lind_out, kiind_out);
}

extern "C" int refeff_fms_mkgtr_trace_device(refeff_fms_context* ctx, int n_energies, int dim, int active_spin_channels,
                                             int lmax, int n_spectra, const int32_t* lind,
                                             const refeff_complex128* bmat, const refeff_complex128* d_gg,
                                             long long gg_ld, long long gg_energy_stride,
                                             const refeff_complex128* d_rkk, refeff_complex128* d_traces,
                                             void* stream) {
  if (!ctx || n_energies <= 0 || dim <= 0 || active_spin_channels <= 0 || active_spin_channels > 2 || lmax < 0 ||
      n_spectra <= 0 || n_spectra > 65535 || !lind || !bmat || !d_gg || !d_rkk ||
      !d_traces || gg_ld < dim)
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  std::vector<TraceTerm> terms;
  std::vector<int> off;
  int rc = compile_terms(n_spectra, lmax, lind, bmat, dim, active_spin_channels, terms, off);
  if (rc) return rc;
  if (cudaSetDevice(context_device(ctx)) != cudaSuccess) return REFEFF_FMS_ERR_CUDA;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : context_stream(ctx);
  return run_trace(ctx, n_energies, reinterpret_cast<const double2*>(d_gg), gg_ld, gg_energy_stride,
                   reinterpret_cast<const double2*>(d_rkk), n_spectra, terms, off,
                   reinterpret_cast<double2*>(d_traces), s, true);
}

extern "C" int refeff_fms_mkgtr_trace(refeff_fms_context* ctx, int n_energies, int dim, int active_spin_channels,
                                      int lmax, int n_spectra, const int32_t* lind, const refeff_complex128* bmat,
                                      const refeff_complex128* gg, const refeff_complex128* rkk, int rkk_spins,
                                      refeff_complex128* traces) {
  if (!ctx || n_energies <= 0 || dim <= 0 || !gg || !rkk || !traces || rkk_spins < active_spin_channels ||
      rkk_spins > 2)
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(context_device(ctx)) != cudaSuccess) return REFEFF_FMS_ERR_CUDA;
  cudaStream_t s = context_stream(ctx);
  const size_t ng = size_t(n_energies) * dim * dim, nr = size_t(n_energies) * 8 * rkk_spins,
               nt = size_t(n_spectra) * n_energies;
  Scratch<double2> dg, dr, dtr;
  if (dg.alloc(ng) || dr.alloc(nr) || dtr.alloc(nt)) {
    set_last_error(ctx, "trace buffer allocation failed");
    return REFEFF_FMS_ERR_OUT_OF_MEMORY;
  }
  if (cudaMemcpyAsync(dg.p, gg, ng * sizeof(double2), cudaMemcpyHostToDevice, s) ||
      cudaMemcpyAsync(dr.p, rkk, nr * sizeof(double2), cudaMemcpyHostToDevice, s)) {
    set_last_error(ctx, "trace upload failed");
    return REFEFF_FMS_ERR_CUDA;
  }
  const int rc = refeff_fms_mkgtr_trace_device(ctx, n_energies, dim, active_spin_channels, lmax, n_spectra, lind, bmat,
                                               reinterpret_cast<const refeff_complex128*>(dg.p), dim,
                                               (long long)dim * dim, reinterpret_cast<const refeff_complex128*>(dr.p),
                                               reinterpret_cast<refeff_complex128*>(dtr.p), s);
  if (cudaMemcpyAsync(traces, dtr.p, nt * sizeof(double2), cudaMemcpyDeviceToHost, s) ||
      cudaStreamSynchronize(s)) {
    set_last_error(ctx, "trace download failed");
    return REFEFF_FMS_ERR_CUDA;
  }
  return rc;
}
