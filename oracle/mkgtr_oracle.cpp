// TEST INFRASTRUCTURE ONLY -- the CPU oracle for the MKGTR step that follows
// the FMS solve: FEFF's transition B matrix (bcoef) and the Green's-function
// trace (getgtr).  Restated from the reference, in FP64 as the reference
// computes them:
//   wigner_3j (cwig3j)          crates/refeff-core/src/angular/wigner.rs:7-92
//   wigner_rotation (rotwig)    crates/refeff-core/src/angular/wigner.rs:101-184
//   transition_b_matrix         crates/refeff-core/src/angular/transition.rs:9-565
//   mkgtr_green_trace           crates/refeff-core/src/fms/mkgtr.rs:790-952
// Only tests, smoke() and the benchmark's CPU baseline use this file.
#include <cmath>
#include <complex>
#include <cstdlib>
#include <vector>

namespace {

using cd = std::complex<double>;

// compiler-rt __powidf2 (what Rust's powi lowers to)
double powi(double a, int b) {
  const bool recip = b < 0;
  double r = 1.0;
  for (;;) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? 1.0 / r : r;
}

struct LogFact {
  double v[59];
  LogFact() {
    v[0] = 0.0;
    for (int i = 1; i <= 58; ++i) v[i] = v[i - 1] + std::log(double(i));
  }
};
const LogFact kLf;

// cwig3j with arguments scaled by `scale` (1 integer, 2 doubled half-integers).
double wigner_3j(int j1, int j2, int j3, int m1, int m2, int scale) {
  const int ds = 2 * scale, m3 = -m1 - m2;
  if (std::abs(m1) + std::abs(m2) == 0 && (j1 + j2 + j3) % ds != 0) return 0.0;
  int v[12] = {j1 + j2 - j3, j2 + j3 - j1, j3 + j1 - j2, j1 + m1, j1 - m1, j2 + m2,
               j2 - m2,      j3 + m3,      j3 - m3,      j1 + j2 + j3 + scale, j2 - j3 - m1, j1 - j3 + m2};
  for (int i = 0; i < 12; ++i) {
    if (i < 10 && v[i] < 0) return 0.0;
    v[i] /= scale;
  }
  const int kmin = std::max(std::max(v[10], v[11]), 0);
  const int kmax = std::min(std::min(v[0], v[4]), v[5]);
  if (kmin > kmax) return 0.0;
  double sign = (kmin % 2 == 0) ? 1.0 : -1.0;
  double c = -kLf.v[v[9]];
  for (int i = 0; i < 9; ++i) c += kLf.v[v[i]];
  c /= 2.0;
  double coef = 0.0;
  for (int k = kmin; k <= kmax; ++k) {
    const double b = kLf.v[k] + kLf.v[v[0] - k] + kLf.v[v[4] - k] + kLf.v[v[5] - k] + kLf.v[k - v[10]] +
                     kLf.v[k - v[11]];
    coef += sign * std::exp(c - b);
    sign = -sign;
  }
  if ((j1 - j2 - m3) % ds != 0) coef = -coef;
  return coef;
}

double alt(int e) { return e % 2 == 0 ? 1.0 : -1.0; }

// rotwig: Wigner small-d element d^{jj}_{m1 m2}(beta), arguments scaled by `scale`.
double wigner_rotation(double beta, int jj, int m1, int m2, int scale) {
  int m1p, m2p;
  double sign;
  if (m1 >= 0 && std::abs(m1) >= std::abs(m2)) { m1p = m1; m2p = m2; sign = 1.0; }
  else if (m2 >= 0 && std::abs(m2) >= std::abs(m1)) { m1p = m2; m2p = m1; beta = -beta; sign = 1.0; }
  else if (m1 <= 0 && std::abs(m1) >= std::abs(m2)) { m1p = -m1; m2p = -m2; sign = alt((m1 - m2) / scale); }
  else { m1p = -m2; m2p = -m1; beta = -beta; sign = alt((m2 - m1) / scale); }
  const double zeta = std::cos(beta / 2.0), eta = std::sin(beta / 2.0);
  double total = 0.0;
  for (int t = m1p - m2p; t <= jj - m2p; t += scale) {
    const int a[8] = {(jj + m1p) / scale,     (jj - m1p) / scale,     (jj + m2p) / scale, (jj - m2p) / scale,
                      (jj + m1p - t) / scale, (jj - m2p - t) / scale, t / scale,          (m2p - m1p + t) / scale};
    const int zp = (2 * jj + m1p - m2p - 2 * t) / scale, ep = (2 * t - m1p + m2p) / scale;
    double f = 0.0;
    for (int i = 0; i < 4; ++i) f += kLf.v[a[i]] / 2.0;
    for (int i = 4; i < 8; ++i) f -= kLf.v[a[i]];
    const double coefficient = alt(t / scale) * std::exp(f);
    double term;
    if (zp == 0 && ep == 0) term = coefficient;
    else if (ep == 0) term = coefficient * powi(zeta, zp);
    else if (zp == 0) term = coefficient * powi(eta, ep);
    else term = coefficient * powi(zeta, zp) * powi(eta, ep);
    total += term;
  }
  return sign * total;
}

cd ipow(int e) {
  switch (((e % 4) + 4) % 4) {
    case 0: return {1.0, 0.0};
    case 1: return {0.0, 1.0};
    case 2: return {-1.0, 0.0};
    default: return {0.0, -1.0};
  }
}

struct BMat {
  int L, ML, EL;
  std::vector<cd> a;  // (ML, 2, 8, ML, 2, 8) column-major
  cd& at(int m2, int s2, int k2, int m1, int s1, int k1) {
    return a[size_t((m2 + L) + ML * (s2 + 2 * (k2 + 8 * ((m1 + L) + ML * (s1 + 2 * k1)))))];
  }
};

void transition_indices(int kinit, int multipole, int lmax, int* jind, int* lind, int* kiind) {
  for (int k = -1; k <= 1; ++k) {
    int kappa = kinit + k;
    if (k == 0) kappa = -kappa;
    int jkap = std::abs(kappa);
    int lkap = kappa <= 0 ? std::abs(kappa) - 1 : kappa;
    if (lkap > lmax) { jkap = 0; lkap = -1; kappa = 0; }
    jind[k + 1] = jkap; lind[k + 1] = lkap; kiind[k + 1] = kappa;
  }
  for (int k = -2; k <= 2; ++k) {
    int jkap = std::abs(kinit) + k;
    if (jkap <= 0) jkap = 0;
    int kappa = jkap;
    if (kinit < 0 && std::abs(k) != 1) kappa = -jkap;
    if (kinit > 0 && std::abs(k) == 1) kappa = -jkap;
    int lkap = kappa <= 0 ? -kappa - 1 : kappa;
    if (lkap > lmax || multipole == 0 || (multipole == 1 && std::abs(k) == 2)) { jkap = 0; lkap = -1; kappa = 0; }
    jind[k + 5] = jkap; lind[k + 5] = lkap; kiind[k + 5] = kappa;
  }
}

void polarized(BMat& B, int kinit, int multipole, double angks, const cd ptz[3][3], const int* jind,
               const int* lind) {
  const int L = B.L, ML = B.ML, EL = B.EL;
  auto ext = [&](int m) { return m + L; };
  std::vector<double> t3j(size_t(8 * 2 * EL)), x3j(size_t(8 * 3 * EL)), qmat(size_t(EL * ML * 2 * 8));
  std::vector<cd> pmat(size_t(EL * 8 * EL * 8)), tmat(size_t(EL * 8 * ML * 2 * 8));
  auto t3i = [&](int k, int s, int mp) { return size_t((k * 2 + s) * EL + ext(mp)); };
  auto x3i = [&](int k, int p, int mp) { return size_t((k * 3 + p + 1) * EL + ext(mp)); };
  auto qi = [&](int mj, int ml, int s, int k) { return size_t(((ext(mj) * ML + (ml + L)) * 2 + s) * 8 + k); };
  auto pi = [&](int m1, int k1, int m2, int k2) { return size_t(((ext(m1) * 8 + k1) * EL + ext(m2)) * 8 + k2); };
  auto ti = [&](int mj, int k2, int ml, int s, int k1) {
    return size_t((((ext(mj) * 8 + k2) * ML + (ml + L)) * 2 + s) * 8 + k1);
  };
  for (int k = 0; k < 8; ++k) {
    const int j = jind[k];
    if (j <= 0) continue;
    for (int mp = -j + 1; mp <= j; ++mp) {
      for (int s = 0; s <= 1; ++s) {
        const int j1 = 2 * lind[k], j2 = 1, j3 = 2 * j - 1, m1 = 2 * (mp - s), m2 = 2 * s - 1;
        double v = std::sqrt(double(j3 + 1)) * wigner_3j(j1, j2, j3, m1, m2, 2);
        if (((j2 - j1 - m1 - m2) / 2) % 2 != 0) v = -v;
        t3j[t3i(k, s, mp)] = v;
      }
      for (int p = -1; p <= 1; ++p) {
        const int j1 = 2 * j - 1, j2 = (k >= 3 && multipole == 2) ? 4 : 2, j3 = 2 * std::abs(kinit) - 1;
        x3j[x3i(k, p, mp)] = wigner_3j(j1, j2, j3, -2 * mp + 1, 2 * p, 2);
      }
    }
  }
  for (int k = 0; k < 8; ++k) {
    const int l = lind[k], j = jind[k];
    if (l < 0 || j <= 0) continue;
    for (int s = 0; s <= 1; ++s)
      for (int ml = -l; ml <= l; ++ml)
        for (int mj = -j + 1; mj <= j; ++mj) {
          const int mp = ml + s;
          const double rot = wigner_rotation(angks, 2 * j - 1, 2 * mj - 1, 2 * mp - 1, 2);
          qmat[qi(mj, ml, s, k)] = rot * t3j[t3i(k, s, mp)];
        }
  }
  for (int k2 = 0; k2 < 8; ++k2) {
    const int j2 = jind[k2];
    if (j2 <= 0) continue;
    for (int m2 = -j2 + 1; m2 <= j2; ++m2)
      for (int k1 = 0; k1 < 8; ++k1) {
        const int j1 = jind[k1];
        if (j1 <= 0) continue;
        for (int m1 = -j1 + 1; m1 <= j1; ++m1) {
          if (std::abs(m2 - m1) > 2) continue;
          cd v(0.0, 0.0);
          for (int pp = -1; pp <= 1; ++pp)
            for (int p = -1; p <= 1; ++p) {
              if (m1 - p != m2 - pp) continue;
              double sg = 1.0;
              if (multipole == 1 && p > 0 && k1 >= 3) sg = -sg;
              if (multipole == 1 && pp > 0 && k2 >= 3) sg = -sg;
              v += ptz[p + 1][pp + 1] * (sg * x3j[x3i(k1, p, m1)] * x3j[x3i(k2, pp, m2)]);
            }
          double sg = 1.0;
          if ((jind[k1] - jind[k2]) % 2 != 0) sg = -sg;
          if (k2 < 3) sg = -sg;
          v *= sg * ipow(lind[k2] - lind[k1]);
          pmat[pi(m1, k1, m2, k2)] = v;
        }
      }
  }
  for (int k1 = 0; k1 < 8; ++k1) {
    const int l1 = lind[k1], j1 = jind[k1];
    if (l1 < 0 || j1 <= 0) continue;
    for (int s = 0; s <= 1; ++s)
      for (int ml = -l1; ml <= l1; ++ml)
        for (int k2 = 0; k2 < 8; ++k2) {
          const int j2 = jind[k2];
          if (j2 <= 0) continue;
          for (int mj = -j2 + 1; mj <= j2; ++mj) {
            cd v(0.0, 0.0);
            for (int mp = -j1 + 1; mp <= j1; ++mp) v += pmat[pi(mj, k2, mp, k1)] * qmat[qi(mp, ml, s, k1)];
            tmat[ti(mj, k2, ml, s, k1)] = v;
          }
        }
  }
  for (int k1 = 0; k1 < 8; ++k1) {
    const int l1 = lind[k1];
    if (l1 < 0) continue;
    for (int s1 = 0; s1 <= 1; ++s1)
      for (int ml1 = -l1; ml1 <= l1; ++ml1)
        for (int k2 = 0; k2 < 8; ++k2) {
          const int l2 = lind[k2], j2 = jind[k2];
          if (l2 < 0 || j2 <= 0) continue;
          for (int s2 = 0; s2 <= 1; ++s2)
            for (int ml2 = -l2; ml2 <= l2; ++ml2) {
              cd v(0.0, 0.0);
              for (int mj = -j2 + 1; mj <= j2; ++mj) v += qmat[qi(mj, ml2, s2, k2)] * tmat[ti(mj, k2, ml1, s1, k1)];
              B.at(ml2, s2, k2, ml1, s1, k1) = v;
            }
        }
  }
}

}  // namespace

extern "C" {

double oracle_wigner_3j(int j1, int j2, int j3, int m1, int m2, int scale) {
  return wigner_3j(j1, j2, j3, m1, m2, scale);
}

double oracle_wigner_rotation(double beta, int jj, int m1, int m2, int scale) {
  return wigner_rotation(beta, jj, m1, m2, scale);
}

// out: (2L+1, 2, 8, 2L+1, 2, 8) complex (interleaved doubles), column-major.
// ptz: 3 x 3 complex polarization tensor, row-major, interleaved.
int oracle_transition_b_matrix(int lmax, int initial_kappa, int polarization, const double* ptz18, int multipole,
                               int trace_orbital, int spin, int spin_channels, double angks, double* out, int* lind,
                               int* kiind) {
  if (spin_channels <= 0 || lmax < 0) return 1;
  BMat B;
  B.L = lmax;
  B.ML = 2 * lmax + 1;
  B.EL = B.ML + 1;
  B.a.assign(size_t(B.ML) * 2 * 8 * B.ML * 2 * 8, cd(0.0, 0.0));
  int jind[8], li[8], ki[8];
  transition_indices(initial_kappa, multipole, lmax, jind, li, ki);
  if (polarization == 0) {
    for (int k = 0; k < 8; ++k) {
      const int l = li[k];
      if (l < 0) continue;
      const double deg = (multipole == 2 && k >= 3) ? 5.0 : 3.0;
      double v = 0.5 / (2.0 * double(l) + 1.0) / deg;
      if (k < 3) v = -v;
      for (int s = 0; s <= 1; ++s)
        for (int m = -l; m <= l; ++m) B.at(m, s, k, m, s, k) = cd(v, 0.0);
    }
  } else {
    cd ptz[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) ptz[r][c] = cd(ptz18[2 * (3 * r + c)], ptz18[2 * (3 * r + c) + 1]);
    polarized(B, initial_kappa, multipole, angks, ptz, jind, li);
  }
  if (trace_orbital) {
    for (int k1 = 0; k1 < 8; ++k1)
      for (int s1 = 0; s1 <= 1; ++s1)
        for (int k2 = 0; k2 < 8; ++k2)
          for (int s2 = 0; s2 <= 1; ++s2) {
            if (li[k1] != li[k2] || s1 != s2) {
              B.at(0, s2, k2, 0, s1, k1) = cd(0.0, 0.0);
            } else {
              for (int m = 1; m <= li[k1]; ++m) {
                const cd add = B.at(-m, s1, k2, -m, s1, k1) + B.at(m, s1, k2, m, s1, k1);
                B.at(0, s1, k2, 0, s1, k1) += add;
              }
            }
          }
  }
  const bool fold_sum = spin == 0, fold_copy = spin == 2 || (spin == 1 && spin_channels == 1);
  if (fold_sum || fold_copy)
    for (int k1 = 0; k1 < 8; ++k1) {
      if (li[k1] < 0) continue;
      for (int k2 = 0; k2 < 8; ++k2) {
        if (li[k2] < 0) continue;
        for (int m1 = -li[k1]; m1 <= li[k1]; ++m1)
          for (int m2 = -li[k2]; m2 <= li[k2]; ++m2) {
            const cd up = B.at(m2, 1, k2, m1, 1, k1);
            if (fold_sum) B.at(m2, 0, k2, m1, 0, k1) += up;
            else B.at(m2, 0, k2, m1, 0, k1) = up;
          }
      }
    }
  for (size_t i = 0; i < B.a.size(); ++i) {
    out[2 * i] = B.a[i].real();
    out[2 * i + 1] = B.a[i].imag();
  }
  for (int k = 0; k < 8; ++k) {
    lind[k] = li[k];
    kiind[k] = ki[k];
  }
  return 0;
}

// gtr traces: traces[spec + nspec*e] = sum over transitions, spins and m of
// gg[e](row, col) bmat[spec](m2, s2, k2, m1, s1, k1) rkk[e, k1, s1] rkk[e, k2, s2],
// with gg as given (E blocks of dim x dim complex, column-major), bmat as from
// oracle_transition_b_matrix for lmax (per spectrum), lind per spectrum (8 ints),
// rkk (E, 8, nsp_rkk) complex column-major.  Returns 2 on a non-finite input or
// result (the reference's NonFiniteComplexValue), 4 when rkk has fewer spins.
int oracle_mkgtr_trace(int E, int dim, int nsp, int lmax, int nspec, const int* lind, const double* bmat,
                       const double* gg, const double* rkk, int nsp_rkk, double* traces) {
  if (nsp_rkk < nsp) return 4;  // the reference's SpinChannelCountMismatch
  const int ML = 2 * lmax + 1;
  const size_t bsz = size_t(ML) * 2 * 8 * ML * 2 * 8;
  for (int sp = 0; sp < nspec; ++sp) {
    const int* li = lind + 8 * sp;
    const double* bm = bmat + 2 * bsz * size_t(sp);
    for (int e = 0; e < E; ++e) {
      cd tr(0.0, 0.0);
      for (int k1 = 0; k1 < 8; ++k1) {
        if (li[k1] < 0) continue;
        for (int s1 = 0; s1 < nsp; ++s1) {
          const size_t r1 = size_t(e) + size_t(E) * (k1 + 8 * size_t(s1));
          const cd rk1(rkk[2 * r1], rkk[2 * r1 + 1]);
          if (!std::isfinite(rk1.real()) || !std::isfinite(rk1.imag())) return 2;
          for (int k2 = 0; k2 < 8; ++k2) {
            if (li[k2] < 0) continue;
            for (int s2 = 0; s2 < nsp; ++s2) {
              const size_t r2 = size_t(e) + size_t(E) * (k2 + 8 * size_t(s2));
              const cd rk2(rkk[2 * r2], rkk[2 * r2 + 1]);
              if (!std::isfinite(rk2.real()) || !std::isfinite(rk2.imag())) return 2;
              for (int m1 = -li[k1]; m1 <= li[k1]; ++m1) {
                const int row = (li[k1] * li[k1] + li[k1] + m1) * nsp + s1;
                for (int m2 = -li[k2]; m2 <= li[k2]; ++m2) {
                  const int col = (li[k2] * li[k2] + li[k2] + m2) * nsp + s2;
                  if (row >= dim || col >= dim) return 3;
                  const size_t gi = size_t(e) * dim * dim + size_t(row) + size_t(dim) * col;
                  const cd g(gg[2 * gi], gg[2 * gi + 1]);
                  if (!std::isfinite(g.real()) || !std::isfinite(g.imag())) return 2;
                  const size_t bi = size_t((m2 + lmax) + ML * (s2 + 2 * (k2 + 8 * ((m1 + lmax) + ML * (s1 + 2 * k1)))));
                  const cd b(bm[2 * bi], bm[2 * bi + 1]);
                  tr += g * b * rk1 * rk2;
                }
              }
            }
          }
        }
      }
      if (!std::isfinite(tr.real()) || !std::isfinite(tr.imag())) return 2;
      traces[2 * (size_t(sp) + size_t(nspec) * e)] = tr.real();
      traces[2 * (size_t(sp) + size_t(nspec) * e) + 1] = tr.imag();
    }
  }
  return 0;
}

}  // extern "C"
