// TEST INFRASTRUCTURE ONLY — the CPU oracle for the real-space FMS path.
//
// This file restates, in plain C++, the arithmetic of refeff's real-space
// full-multiple-scattering (FMS) path so that the GPU implementation in
// refeff_gb300/ can be checked against it.  It is never linked into, loaded
// by, or called from the product library; only tests/, the smoke check and
// bench.py's CPU-baseline leg load it.
//
// Every function is templated on the real type R:
//   R = float   "f32-faithful": the reference computes the whole path in
//               Complex32 / f32 (crates/refeff-core/src/fms/pairs.rs:290,
//               t_matrix.rs:149, crates/refeff-linalg/src/lu.rs:385); this
//               mode follows its operation order and the naive num-complex
//               formulas, and is pinned to the reference's known-answer tests.
//   R = double  "fp64": the same formulas evaluated in double precision; this
//               is the oracle for the FP64 GPU path (1e-10 relative gate).
// Parity pin: the f32-faithful mode is checked against the reference's own
// known-answer vectors (tests/golden/reference_kat.json, transcribed from the
// reference's #[test] functions).  Full-size gg parity against the reference
// binary itself is unpinned: the reference is Rust and no Rust toolchain is
// available here.
//
// Citations are to the reference project's files (paths within the project).
// Build: oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------------------
// Complex arithmetic with num-complex 0.4 semantics (naive formulas, no
// Annex-G special cases).  Rust never contracts a*b+c into an FMA, so this
// file is compiled with -ffp-contract=off.
// ---------------------------------------------------------------------------
template <typename R>
struct cx {
  R re, im;
  cx() : re(0), im(0) {}
  cx(R r, R i) : re(r), im(i) {}
};
template <typename R> inline cx<R> operator+(cx<R> a, cx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <typename R> inline cx<R> operator-(cx<R> a, cx<R> b) { return {a.re - b.re, a.im - b.im}; }
template <typename R> inline cx<R> operator-(cx<R> a) { return {-a.re, -a.im}; }
template <typename R> inline cx<R> operator*(cx<R> a, cx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename R> inline cx<R> operator*(cx<R> a, R s) { return {a.re * s, a.im * s}; }
template <typename R> inline cx<R> operator/(cx<R> a, R s) { return {a.re / s, a.im / s}; }
// num-complex Div: (a*conj(b)) / |b|^2 with the norm computed first.
template <typename R> inline cx<R> operator/(cx<R> a, cx<R> b) {
  R n = b.re * b.re + b.im * b.im;
  R re = a.re * b.re + a.im * b.im;
  R im = a.im * b.re - a.re * b.im;
  return {re / n, im / n};
}
template <typename R> inline cx<R>& operator+=(cx<R>& a, cx<R> b) { a = a + b; return a; }
template <typename R> inline cx<R>& operator-=(cx<R>& a, cx<R> b) { a = a - b; return a; }
template <typename R> inline cx<R>& operator*=(cx<R>& a, cx<R> b) { a = a * b; return a; }
template <typename R> inline bool is_zero(cx<R> a) { return a.re == R(0) && a.im == R(0); }
template <typename R> inline bool is_finite(cx<R> a) { return std::isfinite(a.re) && std::isfinite(a.im); }
// num-complex exp = from_polar(e^re, im).
template <typename R> inline cx<R> cexp(cx<R> a) {
  R r = std::exp(a.re);
  return {r * std::cos(a.im), r * std::sin(a.im)};
}
template <typename R> inline R cnorm(cx<R> a) { return std::hypot(a.re, a.im); }
template <typename R> inline R abs1(cx<R> a) { return std::fabs(a.re) + std::fabs(a.im); }

template <typename R> inline R pi_v();
template <> inline float pi_v<float>() { return 3.14159265358979323846f; }
template <> inline double pi_v<double>() { return 3.14159265358979323846; }

// Error codes (mirror the FmsError / LinalgError variants the tests reach).
enum : int {
  OK = 0,
  ERR_EMPTY_CLUSTER = -1,
  ERR_MISSING_CENTRAL_ATOM = -2,
  ERR_DUPLICATE_ABSORBER = -3,
  ERR_NONFINITE = -4,
  ERR_ZERO_RHO = -5,
  ERR_INVALID_LIMIT = -6,
  ERR_SINGULAR = -7,
  ERR_POTENTIAL_RANGE = -8,
  ERR_MISSING_REPRESENTATIVE = -9,
  ERR_CENTRAL_MISMATCH = -10,
  ERR_INVALID_ARGUMENT = -11,
  ERR_BREAKDOWN = -12,       // FmsError::IterativeSolverBreakdown
  ERR_NO_CONVERGENCE = -13,  // FmsError::IterativeSolverNoConvergence
};

struct Atom {
  float pos[3];
  int pot;
};

// ---------------------------------------------------------------------------
// Cluster preparation (FEFF yprep / athep / sortat / getang).
// ---------------------------------------------------------------------------

// crates/refeff-core/src/fms/internals/geometry.rs:30-36 (athep key) and
// cluster.rs:91-107: stable sort by r^2 + (index+1)*1e-6 evaluated in f64.
inline void sort_atoms_by_radius(std::vector<Atom>& atoms, std::vector<double>* keys_out) {
  std::vector<std::pair<double, size_t>> keyed(atoms.size());
  for (size_t i = 0; i < atoms.size(); ++i) {
    double x = atoms[i].pos[0], y = atoms[i].pos[1], z = atoms[i].pos[2];
    keyed[i] = {x * x + y * y + z * z + (double(i) + 1.0) * 1.0e-6, i};
  }
  std::stable_sort(keyed.begin(), keyed.end(),
                   [](const std::pair<double, size_t>& a, const std::pair<double, size_t>& b) {
                     return a.first < b.first;
                   });
  std::vector<Atom> sorted(atoms.size());
  for (size_t i = 0; i < atoms.size(); ++i) sorted[i] = atoms[keyed[i].second];
  atoms.swap(sorted);
  if (keys_out) {
    keys_out->resize(atoms.size());
    for (size_t i = 0; i < atoms.size(); ++i) (*keys_out)[i] = keyed[i].first;
  }
}

// crates/refeff-core/src/fms/cluster.rs:10-84 (fms_yprep_cluster).
inline int yprep_cluster(int central_potential, const int* pots, const float* positions, size_t rows,
                         float cluster_radius, size_t capacity, std::vector<Atom>& out,
                         size_t* central_atom, size_t* untruncated) {
  if (!std::isfinite(cluster_radius) || cluster_radius < 0.0f) return ERR_INVALID_ARGUMENT;
  if (capacity == 0) return ERR_INVALID_ARGUMENT;
  long central = -1;
  for (size_t i = 0; i < rows; ++i) {
    if (pots[i] == central_potential) {
      if (central_potential == 0 && central >= 0) return ERR_DUPLICATE_ABSORBER;
      if (central < 0) central = long(i);
    }
  }
  if (central < 0) return ERR_MISSING_CENTRAL_ATOM;
  const float* c = positions + 3 * central;
  for (int a = 0; a < 3; ++a)
    if (!std::isfinite(c[a])) return ERR_NONFINITE;
  out.resize(rows);
  for (size_t i = 0; i < rows; ++i) {
    for (int a = 0; a < 3; ++a) {
      out[i].pos[a] = positions[3 * i + a] - c[a];
      if (!std::isfinite(out[i].pos[a])) return ERR_NONFINITE;
    }
    out[i].pot = pots[i];
  }
  sort_atoms_by_radius(out, nullptr);
  float r2 = cluster_radius * cluster_radius;
  size_t first_outside = out.size();
  for (size_t i = 0; i < out.size(); ++i) {
    float x = out[i].pos[0], y = out[i].pos[1], z = out[i].pos[2];
    if (x * x + y * y + z * z > r2) { first_outside = i; break; }
  }
  size_t untr = first_outside == 0 ? out.size() : first_outside;
  out.resize(std::min(untr, capacity));
  if (central_atom) *central_atom = size_t(central);
  if (untruncated) *untruncated = untr;
  return OK;
}

// crates/refeff-core/src/fms/cluster.rs:115-195 (FEFF sortat).
inline int sort_representative_atoms(int central_potential, size_t max_potential, std::vector<Atom>& atoms,
                                     std::vector<long>& representative) {
  if (central_potential < 0 || size_t(central_potential) > max_potential) return ERR_POTENTIAL_RANGE;
  if (atoms.empty()) return ERR_EMPTY_CLUSTER;
  if (atoms[0].pot != central_potential) return ERR_CENTRAL_MISMATCH;
  for (auto& a : atoms) {
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(a.pos[k])) return ERR_NONFINITE;
    if (a.pot < 0 || size_t(a.pot) > max_potential) return ERR_POTENTIAL_RANGE;
  }
  representative.assign(max_potential + 1, -1);
  representative[size_t(central_potential)] = 0;
  for (size_t p = 0; p <= max_potential; ++p) {
    if (p == size_t(central_potential)) continue;
    for (size_t i = 1; i < atoms.size(); ++i)
      if (atoms[i].pot == int(p)) { representative[p] = long(i); break; }
  }
  for (size_t p = 0; p <= max_potential; ++p) {
    long point = representative[p];
    if (point < 0 || size_t(point) <= p) continue;
    std::swap(atoms[p], atoms[size_t(point)]);
    for (size_t q = p + 1; q <= max_potential; ++q)
      if (representative[q] == long(p)) representative[q] = point;
    representative[p] = long(p);
  }
  size_t prefix = std::min(atoms.size(), max_potential + 1);
  for (size_t p = 0; p <= max_potential; ++p) {
    long point = representative[p];
    if (point < 0) continue;
    long last = -1;
    for (size_t i = 0; i < prefix; ++i)
      if (atoms[i].pot == int(p)) last = long(i);
    if (last >= 0 && last != point) {
      float tmp[3];
      std::memcpy(tmp, atoms[size_t(last)].pos, sizeof tmp);
      std::memcpy(atoms[size_t(last)].pos, atoms[size_t(point)].pos, sizeof tmp);
      std::memcpy(atoms[size_t(point)].pos, tmp, sizeof tmp);
      representative[p] = last;
    }
  }
  return OK;
}

// crates/refeff-core/src/fms/cluster.rs:201-241 (FEFF getang): angles of
// positions[i] - positions[j]; computed in R (f32 in the reference).
template <typename R>
inline void pair_polar_angles(const float* pi, const float* pj, bool same, R* theta, R* phi) {
  if (same) { *theta = 0; *phi = 0; return; }
  R x = R(pi[0]) - R(pj[0]);
  R y = R(pi[1]) - R(pj[1]);
  R z = R(pi[2]) - R(pj[2]);
  R r = std::sqrt(x * x + y * y + z * z);
  const R tiny = R(1.0e-7f);
  const R half_pi = pi_v<R>() / R(2);
  R ph;
  if (std::fabs(x) < tiny) {
    if (std::fabs(y) < tiny) ph = 0;
    else if (y > tiny) ph = half_pi;
    else ph = -half_pi;
  } else {
    ph = std::atan2(y, x);
  }
  R th;
  if (r <= tiny) th = 0;
  else if (z <= -r) th = pi_v<R>();
  else if (z < r) th = std::acos(z / r);
  else th = 0;
  *theta = th;
  *phi = ph;
}

// ---------------------------------------------------------------------------
// Wigner rotations (FEFF rotxan).
// crates/refeff-core/src/fms/internals/rotation.rs:3-125, rotation.rs:89-117.
// The table is drix(m2+L, m1+L, l), column-major with dims (2L+1, 2L+1, L+1).
// ---------------------------------------------------------------------------
template <typename R>
inline void rotation_matrix(int lmax, int mmax, R beta, R phi, bool forward, cx<R>* drix) {
  const int D = 2 * lmax + 1;
  const int L1 = lmax + 1;
  // dri0(l, n, m) with l in 1..=lmax+1, n,m in 1..=2l-1 (1-based like FEFF).
  const int dl = lmax + 2, dn = 2 * lmax + 3;
  std::vector<R> dri0(size_t(dl) * dn * dn, R(0));
  auto d0 = [&](int l, int n, int m) -> R& { return dri0[size_t(l) + size_t(dl) * (size_t(n) + size_t(dn) * m)]; };
  const int lxp1 = lmax + 1, mxp1 = mmax + 1, ndm = lxp1 + mxp1 - 1;
  R xc = std::cos(beta / R(2));
  R xs = std::sin(beta / R(2));
  R s = std::sin(beta);
  d0(1, 1, 1) = 1;
  if (lxp1 >= 2) {
    d0(2, 1, 1) = xc * xc;
    d0(2, 1, 2) = s / std::sqrt(R(2));
    d0(2, 1, 3) = xs * xs;
    d0(2, 2, 1) = -d0(2, 1, 2);
    d0(2, 2, 2) = std::cos(beta);
    d0(2, 2, 3) = d0(2, 1, 2);
    d0(2, 3, 1) = d0(2, 1, 3);
    d0(2, 3, 2) = -d0(2, 2, 3);
    d0(2, 3, 3) = d0(2, 1, 1);
    for (int l = 3; l <= lxp1; ++l) {
      int ln = std::min(2 * l - 1, ndm);
      int lm = std::min(2 * l - 3, ndm);
      for (int n = 1; n <= ln; ++n) {
        for (int m = 1; m <= lm; ++m) {
          R t1 = R((2 * l - 1 - n) * (2 * l - 2 - n));
          R t = R((2 * l - 1 - m) * (2 * l - 2 - m));
          R f1 = std::sqrt(t1 / t);
          R f2 = std::sqrt(R((2 * l - 1 - n) * (n - 1)) / t);
          R t3 = R((n - 2) * (n - 1));
          R f3 = std::sqrt(t3 / t);
          R dlnm = f1 * xc * xc * d0(l - 1, n, m);
          if (n > 1) dlnm -= f2 * s * d0(l - 1, n - 1, m);
          if (n > 2) dlnm += f3 * xs * xs * d0(l - 1, n - 2, m);
          d0(l, n, m) = dlnm;
          if (n > 2 * l - 3) d0(l, m, n) = (((n - m) % 2) == 0 ? R(1) : R(-1)) * dlnm;
        }
        if (n > 2 * l - 3) {
          d0(l, 2 * l - 2, 2 * l - 2) = d0(l, 2, 2);
          d0(l, 2 * l - 1, 2 * l - 2) = -d0(l, 1, 2);
          d0(l, 2 * l - 2, 2 * l - 1) = -d0(l, 2, 1);
          d0(l, 2 * l - 1, 2 * l - 1) = d0(l, 1, 1);
        }
      }
    }
  }
  for (int i = 0; i < D * D * L1; ++i) drix[i] = cx<R>();
  auto dr = [&](int m2, int m1, int l) -> cx<R>& {
    return drix[size_t(m2 + lmax) + size_t(D) * (size_t(m1 + lmax) + size_t(D) * size_t(l))];
  };
  for (int il = 1; il <= lmax + 1; ++il) {
    int mmx = std::min(il - 1, mmax);
    for (int m1 = -mmx; m1 <= mmx; ++m1)
      for (int m2 = -mmx; m2 <= mmx; ++m2) dr(m2, m1, il - 1) = cx<R>(d0(il, m1 + il, m2 + il), R(0));
  }
  const R pi = pi_v<R>();
  for (int il = 0; il <= lmax; ++il) {
    for (int m1 = -il; m1 <= il; ++m1) {
      R angle = forward ? R(m1) * (phi - pi) : R(-m1) * (phi - pi);
      cx<R> phase = cexp(cx<R>(R(0), angle));
      for (int m2 = -il; m2 <= il; ++m2) {
        if (forward) dr(m1, m2, il) *= phase;
        else dr(m2, m1, il) *= phase;
      }
    }
  }
}

// crates/refeff-core/src/angular/harmonics.rs:51-75: xnlm(m, l) in f64.
inline double legendre_normalization(int l, int m) {
  if (m > l) return 0.0;
  double num = double(2 * l + 1);
  double den = 1.0;
  for (int k = l - m + 1; k <= l + m; ++k) den *= double(k);
  return std::sqrt(num / den);
}

// ---------------------------------------------------------------------------
// Hankel polynomial table (FEFF xclmz).  crates/refeff-core/src/fms/polynomial.rs:8-83.
// clm(il, im) stored column-major with dims (lx+2, 2lx+3).
// ---------------------------------------------------------------------------
template <typename R>
inline int rehr_albers_polynomials(int lx, int lmaxp1, int mmaxp1, cx<R> rho, cx<R>* clm) {
  if (lmaxp1 <= 0 || lmaxp1 > lx + 1 || mmaxp1 <= 0) return ERR_INVALID_LIMIT;
  if (!is_finite(rho)) return ERR_NONFINITE;
  if (is_zero(rho)) return ERR_ZERO_RHO;
  const int rows = lx + 2, cols = 2 * lx + 3;
  for (int i = 0; i < rows * cols; ++i) clm[i] = cx<R>();
  auto C = [&](int il, int im) -> cx<R>& { return clm[size_t(il) + size_t(rows) * size_t(im)]; };
  const cx<R> one(R(1), R(0));
  cx<R> z = cx<R>(R(0), R(-1)) / rho;
  auto odd = [](int index) { return cx<R>(R(2 * index - 1), R(0)); };
  C(0, 0) = one;
  C(1, 0) = one - z;
  int lmax = lmaxp1 - 1;
  for (int il = 2; il <= lmax; ++il) {
    cx<R> factor = odd(il) * z;
    C(il, 0) = C(il - 2, 0) - factor * C(il - 1, 0);
  }
  cx<R> cmm = one;
  int mmxp1 = std::min(lmaxp1, mmaxp1);
  for (int im = 2; im <= mmxp1; ++im) {
    int m = im - 1;
    cx<R> cmm_factor = odd(m) * z;
    cmm = (-cmm) * cmm_factor;
    C(im - 1, im - 1) = cmm;
    C(im, im - 1) = cmm * odd(im) * (one - cx<R>(R(im), R(0)) * z);
    for (int il = im + 1; il <= lmax; ++il) {
      cx<R> factor = odd(il) * z;
      C(il, im - 1) = C(il - 2, im - 1) - factor * (C(il - 1, im - 1) + C(il - 1, im - 2));
    }
  }
  return OK;
}

// crates/refeff-core/src/fms/internals/geometry.rs:14-28: e^{i rho}/rho * e^{-sigma^2 k^2}.
template <typename R>
inline cx<R> free_propagator_prefactor(cx<R> rho, cx<R> k, R msd) {
  cx<R> phase = cexp(cx<R>(R(0), R(1)) * rho) / rho;
  cx<R> damping_factor(-msd, R(0));
  cx<R> damping = cexp(damping_factor * k * k);
  return phase * damping;
}

// ---------------------------------------------------------------------------
// Spin-orbit tables t3jp/t3jm.  crates/refeff-core/src/angular/coupling.rs:4-40,
// wigner.rs:7-92 (Racah formula over log-factorials, doubled arguments).
// ---------------------------------------------------------------------------
inline double wigner_3j_doubled(int j1, int j2, int j3, int m1, int m2) {
  const int scale = 2, dscale = 4;
  int m3 = -m1 - m2;
  if (std::abs(m1) + std::abs(m2) == 0 && (j1 + j2 + j3) % dscale != 0) return 0.0;
  int v[12] = {j1 + j2 - j3, j2 + j3 - j1, j3 + j1 - j2, j1 + m1, j1 - m1, j2 + m2,
               j2 - m2,      j3 + m3,      j3 - m3,      j1 + j2 + j3 + scale, j2 - j3 - m1, j1 - j3 + m2};
  for (int i = 0; i < 12; ++i) {
    if (i < 10 && v[i] < 0) return 0.0;
    v[i] /= scale;
  }
  double lf[60];
  lf[0] = 0.0;
  for (int i = 1; i < 60; ++i) lf[i] = lf[i - 1] + std::log(double(i));
  int kmin = std::max(std::max(v[10], v[11]), 0);
  int kmax = std::min(std::min(v[0], v[4]), v[5]);
  if (kmin > kmax) return 0.0;
  double sign = (kmin % 2 == 0) ? 1.0 : -1.0;
  double c = -lf[v[9]];
  for (int i = 0; i < 9; ++i) c += lf[v[i]];
  c /= 2.0;
  double coef = 0.0;
  for (int k = kmin; k <= kmax; ++k) {
    double b = lf[k] + lf[v[0] - k] + lf[v[4] - k] + lf[v[5] - k] + lf[k - v[10]] + lf[k - v[11]];
    coef += sign * std::exp(c - b);
    sign = -sign;
  }
  if ((j1 - j2 - m3) % dscale != 0) coef = -coef;
  return coef;
}

// plus/minus(l, m, spin) for spin in {1,2}; returned in f64.
inline double spin_orbit_coefficient(bool plus, int l, int m, int spin) {
  int j1 = 2 * l, j2 = 1, j3 = plus ? j1 + 1 : j1 - 1;
  int m1 = 2 * m, m2 = 2 * spin - 3;
  int phase = (j2 - j1 - m1 - m2) / 2;
  double sign = (phase % 2 == 0) ? 1.0 : -1.0;
  return sign * std::sqrt(double(j3 + 1)) * wigner_3j_doubled(j1, j2, j3, m1, m2);
}

// ---------------------------------------------------------------------------
// State kets (FEFF getkts).  crates/refeff-core/src/state.rs:97-148.
// ---------------------------------------------------------------------------
struct Ket {
  int atom;  // zero-based
  int l, m, spin;  // spin 1-based
};

inline int construct_state_kets(int nsp, const std::vector<int>& atom_pots, const std::vector<int>& pot_lmax,
                                int global_lmax, std::vector<Ket>& kets, std::vector<long>& rep_offsets) {
  if (nsp <= 0) return ERR_INVALID_ARGUMENT;
  kets.clear();
  rep_offsets.assign(pot_lmax.size(), -1);
  for (size_t a = 0; a < atom_pots.size(); ++a) {
    int p = atom_pots[a];
    if (p < 0 || size_t(p) >= pot_lmax.size()) return ERR_POTENTIAL_RANGE;
    if (rep_offsets[size_t(p)] < 0) rep_offsets[size_t(p)] = long(kets.size());
    int lmax = std::min(global_lmax, pot_lmax[size_t(p)]);
    for (int l = 0; l <= lmax; ++l)
      for (int m = -l; m <= l; ++m)
        for (int s = 1; s <= nsp; ++s) kets.push_back({int(a), l, m, s});
  }
  return OK;
}

// crates/refeff-core/src/fms/internals/validation.rs:69-75.
inline int clamp_lipotx(int value, int global_lmax) { return value < 0 ? global_lmax : std::min(value, global_lmax); }

// ---------------------------------------------------------------------------
// Per-plan (energy independent) data, per-energy pipeline.
// ---------------------------------------------------------------------------
template <typename R>
struct Plan {
  int nsp = 1, ispin = 0, L = 0, npot = 0;
  std::vector<Atom> atoms;
  std::vector<int> pot_lmax;
  std::vector<Ket> kets;
  std::vector<long> rep_offsets;
  int pot_start = 0, pot_end = 0;
  R rdirec = 0;
  std::vector<R> sigsqr;       // (N,N) col-major, [atom2 + N*atom1]
  std::vector<cx<R>> rot;      // (D,D,L+1,2,N,N) col-major
  std::vector<R> xnlm;         // (L+1,L+1) [mu + (L+1)*l], narrowed like the reference
  // spin-orbit tables narrowed to f32 (reference narrows with `as f32`).
  std::vector<R> t3p, t3m;     // [(l) + (L+1)*((m+L) + (2L+1)*(s-1))]
  size_t n() const { return kets.size(); }
};

template <typename R>
inline size_t rot_index(const Plan<R>& P, int m2i, int m1i, int l, int k, int a2, int a1) {
  const size_t D = size_t(2 * P.L + 1), L1 = size_t(P.L + 1), N = P.atoms.size();
  return size_t(m2i) + D * (size_t(m1i) + D * (size_t(l) + L1 * (size_t(k) + 2 * (size_t(a2) + N * size_t(a1)))));
}

// crates/refeff-core/src/fms/rotation.rs:10-82 (fms_yprep_geometry).
template <typename R>
inline void build_rotations(Plan<R>& P) {
  const int L = P.L;
  const size_t D = size_t(2 * L + 1), L1 = size_t(L + 1), N = P.atoms.size();
  P.rot.assign(D * D * L1 * 2 * N * N, cx<R>());
  std::vector<cx<R>> tab(D * D * L1);
  for (size_t a1 = 0; a1 < N; ++a1)
    for (size_t a2 = 0; a2 < N; ++a2) {
      if (a1 == a2) continue;
      R beta, phi;
      pair_polar_angles<R>(P.atoms[a1].pos, P.atoms[a2].pos, false, &beta, &phi);
      for (int dir = 0; dir < 2; ++dir) {
        rotation_matrix<R>(L, L, dir == 0 ? beta : -beta, phi, dir == 0, tab.data());
        for (size_t l = 0; l < L1; ++l)
          for (size_t m1 = 0; m1 < D; ++m1)
            for (size_t m2 = 0; m2 < D; ++m2)
              P.rot[rot_index(P, int(m2), int(m1), int(l), dir, int(a2), int(a1))] = tab[m2 + D * (m1 + D * l)];
      }
    }
}

template <typename R>
inline int make_plan(Plan<R>& P, const Atom* atoms, int n_atoms, int nsp, int ispin, int lfms, int max_potential,
                     int global_lmax, const int* lmaxph, R rdirec, const float* sigsqr /* NxN col-major or null */,
                     float sig2g) {
  // crates/refeff-core/src/fms/driver.rs:4-65 (fms_driver_setup).
  if (n_atoms <= 0) return ERR_EMPTY_CLUSTER;
  if (nsp < 1 || nsp > 2) return ERR_INVALID_ARGUMENT;
  if (global_lmax < 0 || global_lmax > 24) return ERR_INVALID_LIMIT;
  P.nsp = nsp;
  P.ispin = ispin;
  P.atoms.assign(atoms, atoms + n_atoms);
  P.npot = max_potential + 1;
  int L = global_lmax;
  P.L = L;
  P.pot_lmax.resize(size_t(P.npot));
  for (int p = 0; p < P.npot; ++p) P.pot_lmax[size_t(p)] = clamp_lipotx(lmaxph[p], L);
  std::vector<int> atom_pots(static_cast<size_t>(n_atoms));
  for (int a = 0; a < n_atoms; ++a) {
    if (atoms[a].pot < 0 || atoms[a].pot > max_potential) return ERR_POTENTIAL_RANGE;
    atom_pots[size_t(a)] = atoms[a].pot;
  }
  int rc = construct_state_kets(nsp, atom_pots, P.pot_lmax, L, P.kets, P.rep_offsets);
  if (rc) return rc;
  int absorber = atom_pots[0];
  if (lfms == 0) { P.pot_start = absorber; P.pot_end = absorber; }
  else { P.pot_start = 0; P.pot_end = max_potential; }
  for (int p = P.pot_start; p <= P.pot_end; ++p)
    if (P.rep_offsets[size_t(p)] < 0) return ERR_MISSING_REPRESENTATIVE;
  P.rdirec = rdirec;
  size_t N = size_t(n_atoms);
  P.sigsqr.assign(N * N, R(0));
  for (size_t a1 = 0; a1 < N; ++a1)
    for (size_t a2 = 0; a2 < N; ++a2) {
      if (a1 == a2) continue;
      // engine/fms.rs:4394-4426: sigsqr(atom2, atom1) = sig2g + pair, narrowed to f32.
      float v = sigsqr ? sigsqr[a2 + N * a1] : float(double(sig2g) + 0.0);
      P.sigsqr[a2 + N * a1] = R(v);
    }
  build_rotations(P);
  P.xnlm.assign(size_t((L + 1) * (L + 1)), R(0));
  for (int l = 0; l <= L; ++l)
    for (int mu = 0; mu <= l; ++mu) P.xnlm[size_t(mu + (L + 1) * l)] = R(float(legendre_normalization(l, mu)));
  const size_t D = size_t(2 * L + 1);
  P.t3p.assign(size_t(L + 1) * D * 2, R(0));
  P.t3m.assign(size_t(L + 1) * D * 2, R(0));
  for (int l = 0; l <= L; ++l)
    for (int m = -l; m <= l; ++m)
      for (int s = 1; s <= 2; ++s) {
        size_t idx = size_t(l) + size_t(L + 1) * (size_t(m + L) + D * size_t(s - 1));
        P.t3p[idx] = R(float(spin_orbit_coefficient(true, l, m, s)));
        P.t3m[idx] = R(float(spin_orbit_coefficient(false, l, m, s)));
      }
  return OK;
}

// xphase(spin, l+L, pot) layout: [(spin) + nsp*((l+L) + (2L+1)*pot)] (column-major like ndarray .f()).
template <typename R>
struct EnergyInput {
  const cx<R>* k;       // nsp
  const cx<R>* xphase;  // nsp*(2L+1)*npot
};

template <typename R>
inline cx<R> phase_value(const Plan<R>& P, const cx<R>* xphase, int spin, int l, int pot) {
  const int D = 2 * P.L + 1;
  return xphase[size_t(spin - 1) + size_t(P.nsp) * (size_t(l + P.L) + size_t(D) * size_t(pot))];
}

// crates/refeff-core/src/fms/internals/t_matrix.rs:38-41.
template <typename R>
inline cx<R> t_matrix_phase(cx<R> phase) {
  cx<R> two_i(R(0), R(2));
  return (cexp(two_i * phase) - cx<R>(R(1), R(0))) / two_i;
}

template <typename R>
inline R so_coef(const Plan<R>& P, bool plus, int l, int m, int s) {
  const size_t D = size_t(2 * P.L + 1);
  size_t idx = size_t(l) + size_t(P.L + 1) * (size_t(m + P.L) + D * size_t(s - 1));
  return plus ? P.t3p[idx] : P.t3m[idx];
}

// crates/refeff-core/src/fms/t_matrix.rs:10-143 (fms_t_matrix_element) for a
// same-atom pair; callers handle the different-atom zero.
template <typename R>
inline cx<R> t_matrix_element(const Plan<R>& P, const cx<R>* xphase, const Ket& a, const Ket& b, int pot) {
  if (a.atom != b.atom) return cx<R>();
  int l1 = a.l;
  bool same = a.atom == b.atom && a.l == b.l && a.m == b.m && a.spin == b.spin;
  if (P.nsp == 1 && P.ispin == 0) {
    return same ? t_matrix_phase(phase_value(P, xphase, a.spin, l1, pot)) : cx<R>();
  }
  if (same) {
    int cs = P.nsp == 1 ? (P.ispin > 0 ? 2 : 1) : a.spin;
    R minus = so_coef(P, false, l1, a.m, cs);
    R plus = so_coef(P, true, l1, a.m, cs);
    cx<R> pm = phase_value(P, xphase, a.spin, l1, pot);
    cx<R> pp = phase_value(P, xphase, a.spin, -l1, pot);
    return t_matrix_phase(pm) * (minus * minus) + t_matrix_phase(pp) * (plus * plus);
  }
  if (P.nsp == 2 && a.l == b.l && a.m + a.spin == b.m + b.spin) {
    R mf = so_coef(P, false, l1, a.m, a.spin), ms = so_coef(P, false, l1, b.m, b.spin);
    R pf = so_coef(P, true, l1, a.m, a.spin), ps = so_coef(P, true, l1, b.m, b.spin);
    cx<R> minus_phase = (t_matrix_phase(phase_value(P, xphase, a.spin, l1, pot)) +
                         t_matrix_phase(phase_value(P, xphase, b.spin, l1, pot))) * R(0.5);
    cx<R> plus_phase = (t_matrix_phase(phase_value(P, xphase, a.spin, -l1, pot)) +
                        t_matrix_phase(phase_value(P, xphase, b.spin, -l1, pot))) * R(0.5);
    return minus_phase * mf * ms + plus_phase * pf * ps;
  }
  return cx<R>();
}

// crates/refeff-core/src/fms/internals/linear.rs:163-201.
inline long spin_partner_index(const Ket& s, long column, long n) {
  int projection = s.m + s.spin;
  if (projection <= -s.l + 1 || projection >= s.l + 2) return -1;
  long partner = s.spin == 1 ? column - 1 : column + 1;
  if (partner < 0 || partner >= n) return -1;
  return partner;
}

// crates/refeff-core/src/fms/t_matrix.rs:149-190: compact (nsp, n) table.
template <typename R>
inline void t_matrix_table(const Plan<R>& P, const cx<R>* xphase, std::vector<cx<R>>& t) {
  const size_t n = P.n();
  t.assign(size_t(P.nsp) * n, cx<R>());
  for (size_t c = 0; c < n; ++c) {
    const Ket& f = P.kets[c];
    int pot = P.atoms[size_t(f.atom)].pot;
    t[size_t(P.nsp) * c] = t_matrix_element(P, xphase, f, f, pot);
    if (P.nsp == 2) {
      long partner = spin_partner_index(f, long(c), long(n));
      if (partner >= 0) t[1 + 2 * c] = t_matrix_element(P, xphase, f, P.kets[size_t(partner)], pot);
    }
  }
}

// crates/refeff-core/src/fms/pairs.rs:242-323, 413-460, 519-553: the G0
// matrix (column-major n x n), with rho/xclm per spin (pairs.rs:9-98).
template <typename R>
inline int free_propagator_matrix(const Plan<R>& P, const cx<R>* k, std::vector<cx<R>>& g0, int threads = 1) {
  const size_t n = P.n(), N = P.atoms.size();
  const int L = P.L, L1 = L + 1, D = 2 * L + 1;
  g0.assign(n * n, cx<R>());
  // per spin, per unordered pair polynomial tables: xclm(m,l) = clm(l,m).
  const int rows = L + 2, cols = 2 * L + 3;
  std::vector<cx<R>> clm(static_cast<size_t>(rows * cols));
  std::vector<cx<R>> xclm(size_t(P.nsp) * N * N * size_t(L1 * L1));
  std::vector<cx<R>> rho(size_t(P.nsp) * N * N);
  for (int s = 0; s < P.nsp; ++s) {
    if (!is_finite(k[s])) return ERR_NONFINITE;
    for (size_t i = 0; i < N; ++i)
      for (size_t j = 0; j <= i; ++j) {
        R dx = R(P.atoms[i].pos[0]) - R(P.atoms[j].pos[0]);
        R dy = R(P.atoms[i].pos[1]) - R(P.atoms[j].pos[1]);
        R dz = R(P.atoms[i].pos[2]) - R(P.atoms[j].pos[2]);
        R dist = std::sqrt(dx * dx + dy * dy + dz * dz);
        cx<R> r = k[s] * dist;
        rho[size_t(s) * N * N + i + N * j] = r;
        rho[size_t(s) * N * N + j + N * i] = r;
        if (i == j) continue;
        int rc = rehr_albers_polynomials<R>(L, L1, L1, r, clm.data());
        if (rc) return rc;
        for (int l = 0; l <= L; ++l)
          for (int m = 0; m <= L; ++m) {
            cx<R> v = clm[size_t(l) + size_t(rows) * size_t(m)];
            xclm[((size_t(s) * N * N + j + N * i) * L1 + size_t(l)) * L1 + size_t(m)] = v;
            xclm[((size_t(s) * N * N + i + N * j) * L1 + size_t(l)) * L1 + size_t(m)] = v;
          }
      }
  }
  auto XC = [&](int s, size_t a2, size_t a1, int l, int m) -> cx<R> {
    return xclm[((size_t(s) * N * N + a2 + N * a1) * L1 + size_t(l)) * L1 + size_t(m)];
  };
  R cutoff2 = P.rdirec * P.rdirec;
  // Columns are independent; with threads > 1 they are shared out, and the
  // first error code in column order is returned.
  std::vector<int> col_err(n, OK);
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads > 0 ? threads : 1)
  for (long colv = 0; colv < long(n); ++colv) {
    const size_t col = size_t(colv);
    col_err[col] = [&]() -> int {
    const Ket& b = P.kets[col];
    for (size_t row = 0; row < n; ++row) {
      const Ket& a = P.kets[row];
      if (a.atom == b.atom || a.spin != b.spin) continue;
      const float* pa = P.atoms[size_t(a.atom)].pos;
      const float* pb = P.atoms[size_t(b.atom)].pos;
      R dx = R(pa[0]) - R(pb[0]), dy = R(pa[1]) - R(pb[1]), dz = R(pa[2]) - R(pb[2]);
      R d2 = dx * dx + dy * dy + dz * dz;
      if (d2 > cutoff2) continue;
      int s = a.spin - 1;
      size_t i = size_t(a.atom), j = size_t(b.atom);
      cx<R> r = rho[size_t(s) * N * N + j + N * i];
      R msd = P.sigsqr[j + N * i];
      if (!is_finite(r)) return ERR_NONFINITE;
      if (is_zero(r)) return ERR_ZERO_RHO;
      if (!std::isfinite(msd)) return ERR_NONFINITE;
      int l1 = a.l, l2 = b.l;
      cx<R> sum;
      for (int mu = -l1; mu <= l1; ++mu) {
        int amu = mu < 0 ? -mu : mu;
        cx<R> g;
        if (amu <= l2) {
          R n1 = P.xnlm[size_t(amu + L1 * l1)], n2 = P.xnlm[size_t(amu + L1 * l2)];
          cx<R> w(R(2 * l1 + 1), R(0));
          R sign = (amu % 2 == 0) ? R(1) : R(-1);
          int numax = std::min(l1, l2 - amu);
          for (int nu = 0; nu <= numax; ++nu) {
            cx<R> gamtl = w * XC(s, j, i, l1, nu) / n1;
            cx<R> gam = XC(s, j, i, l2, amu + nu) * (sign * n2);
            g += gamtl * gam;
          }
        }
        cx<R> back = P.rot[rot_index(P, mu + L, a.m + L, l1, 1, int(j), int(i))];
        cx<R> fwd = P.rot[rot_index(P, b.m + L, mu + L, l2, 0, int(j), int(i))];
        sum += back * g * fwd;
      }
      (void)D;
      g0[row + n * col] = free_propagator_prefactor(r, k[s], msd) * sum;
    }
    return OK;
    }();
  }
  for (size_t col = 0; col < n; ++col)
    if (col_err[col] != OK) return col_err[col];
  return OK;
}

// crates/refeff-core/src/fms/internals/linear.rs:102-135: A = I - G0*T (compact T, spin partner).
template <typename R>
inline void lu_system_matrix(const Plan<R>& P, const std::vector<cx<R>>& g0, const std::vector<cx<R>>& t,
                             std::vector<cx<R>>& A) {
  const size_t n = P.n();
  A.assign(n * n, cx<R>());
  for (size_t c = 0; c < n; ++c) {
    for (size_t r = 0; r < n; ++r) A[r + n * c] = (-g0[r + n * c]) * t[size_t(P.nsp) * c];
    if (P.nsp == 2) {
      long partner = spin_partner_index(P.kets[c], long(c), long(n));
      if (partner >= 0)
        for (size_t r = 0; r < n; ++r) A[r + n * c] -= g0[r + n * size_t(partner)] * t[1 + 2 * c];
    }
    A[c + n * c] += cx<R>(R(1), R(0));
  }
}

// crates/refeff-linalg/src/lu.rs:328-377 (FEFF cgetrf-compatible LU, pivot
// norm |re|+|im|), operating on a column-major n x n matrix in place.
template <typename R>
inline int lu_factor(cx<R>* A, size_t n, std::vector<size_t>& piv, long* singular_pivot) {
  piv.resize(n);
  for (size_t p = 0; p < n; ++p) {
    size_t pr = p;
    R best = abs1(A[p + n * p]);
    for (size_t r = p + 1; r < n; ++r) {
      R cand = abs1(A[r + n * p]);
      if (cand > best) { pr = r; best = cand; }
    }
    piv[p] = pr;
    if (is_zero(A[pr + n * p])) {
      if (singular_pivot) *singular_pivot = long(p);
      return ERR_SINGULAR;
    }
    if (pr != p)
      for (size_t c = 0; c < n; ++c) std::swap(A[p + n * c], A[pr + n * c]);
    cx<R> pv = A[p + n * p];
    for (size_t r = p + 1; r < n; ++r) A[r + n * p] = A[r + n * p] / pv;
    for (size_t c = p + 1; c < n; ++c) {
      cx<R> u = A[p + n * c];
      if (is_zero(u)) continue;
      cx<R>* colc = A + n * c;
      const cx<R>* colp = A + n * p;
      for (size_t r = p + 1; r < n; ++r) colc[r] = colc[r] - colp[r] * u;
    }
  }
  return OK;
}

// crates/refeff-linalg/src/lu.rs:400-465 (complex32_lu_solve): B is n x m column-major.
template <typename R>
inline void lu_solve(const cx<R>* LU, size_t n, const std::vector<size_t>& piv, cx<R>* B, size_t m) {
  for (size_t p = 0; p < n; ++p)
    if (piv[p] != p)
      for (size_t c = 0; c < m; ++c) std::swap(B[p + n * c], B[piv[p] + n * c]);
  for (size_t c = 0; c < m; ++c) {
    cx<R>* b = B + n * c;
    for (size_t p = 0; p < n; ++p) {
      cx<R> v = b[p];
      const cx<R>* col = LU + n * p;
      for (size_t r = p + 1; r < n; ++r) b[r] = b[r] - col[r] * v;
    }
    for (size_t p = n; p-- > 0;) {
      b[p] = b[p] / LU[p + n * p];
      cx<R> v = b[p];
      const cx<R>* col = LU + n * p;
      for (size_t r = 0; r < p; ++r) b[r] = b[r] - col[r] * v;
    }
  }
}

// crates/refeff-core/src/fms/solvers.rs:366-484 (fms_lu_scattering): returns
// the (C, C, npot) scattering table, C = nsp (L+1)^2, column-major.
template <typename R>
inline int lu_scattering(const Plan<R>& P, const std::vector<cx<R>>& g0, const std::vector<cx<R>>& t,
                         std::vector<cx<R>>& scat, long* singular_pivot) {
  const size_t n = P.n();
  std::vector<cx<R>> A;
  lu_system_matrix(P, g0, t, A);
  std::vector<size_t> piv;
  int rc = lu_factor(A.data(), n, piv, singular_pivot);
  if (rc) return rc;
  const size_t C = size_t(P.nsp) * size_t((P.L + 1) * (P.L + 1));
  scat.assign(C * C * size_t(P.npot), cx<R>());
  for (int p = P.pot_start; p <= P.pot_end; ++p) {
    int lm = std::min(P.pot_lmax[size_t(p)], P.L);
    size_t ipart = size_t(P.nsp) * size_t((lm + 1) * (lm + 1));
    size_t off = size_t(P.rep_offsets[size_t(p)]);
    std::vector<cx<R>> rhs(n * ipart);
    for (size_t c = 0; c < ipart; ++c)
      for (size_t r = 0; r < n; ++r) rhs[r + n * c] = g0[r + n * (off + c)];
    lu_solve(A.data(), n, piv, rhs.data(), ipart);
    for (size_t c = 0; c < ipart; ++c)
      for (size_t r = 0; r < ipart; ++r) scat[r + C * (c + C * size_t(p))] = rhs[off + r + n * c];
  }
  return OK;
}

// crates/refeff-core/src/fms/solvers.rs:10-78 (iterative system 1 - T*G0 with toler2 cutoff).
template <typename R>
inline void iterative_system_matrix(const Plan<R>& P, const std::vector<cx<R>>& g0, const std::vector<cx<R>>& t,
                                    R toler2, std::vector<cx<R>>& A) {
  const size_t n = P.n();
  A.assign(n * n, cx<R>());
  const cx<R> factor(R(-1), R(0));
  for (size_t c = 0; c < n; ++c) {
    for (size_t r = 0; r < n; ++r) {
      cx<R> g = g0[r + n * c];
      if (cnorm(g) > toler2) A[r + n * c] += factor * t[size_t(P.nsp) * r] * g;
      if (P.nsp == 2) {
        long partner = spin_partner_index(P.kets[r], long(r), long(n));
        if (partner >= 0) {
          cx<R> gf = g0[size_t(partner) + n * c];
          if (cnorm(gf) > toler2) A[r + n * c] += factor * t[1 + 2 * size_t(partner)] * gf;
        }
      }
    }
    A[c + n * c] += cx<R>(R(1), R(0));
  }
}

// ---------------------------------------------------------------------------
// Iterative FMS solvers (minv != 0).  crates/refeff-core/src/fms/solvers.rs:10-78,
// 225-357 and internals/iterative.rs:24-612, with the vector helpers of
// internals/linear.rs:3-101.  Each solver returns the solution of W x = e_src.
// ---------------------------------------------------------------------------
template <typename R>
inline cx<R> conj(cx<R> a) { return {a.re, -a.im}; }

// num-complex sqrt: special cases on the axes, else the polar form.
template <typename R>
inline cx<R> csqrt(cx<R> z) {
  if (z.im == R(0)) {
    if (!std::signbit(z.re)) return {std::sqrt(z.re), z.im};
    const R r = std::sqrt(-z.re);
    return {R(0), std::signbit(z.im) ? -r : r};
  }
  if (z.re == R(0)) {
    const R x = std::sqrt(std::fabs(z.im) / R(2));
    return {x, std::signbit(z.im) ? -x : x};
  }
  const R r = std::hypot(z.re, z.im), th = std::atan2(z.im, z.re);
  const R sr = std::sqrt(r), h = th / R(2);
  return {sr * std::cos(h), sr * std::sin(h)};
}

template <typename R>
inline cx<R> cdot(const std::vector<cx<R>>& a, const std::vector<cx<R>>& b) {
  cx<R> s;
  for (size_t i = 0; i < a.size(); ++i) s = s + conj(a[i]) * b[i];
  return s;
}

template <typename R>
inline std::vector<cx<R>> matvec(const std::vector<cx<R>>& W, const std::vector<cx<R>>& v) {
  const size_t n = v.size();
  std::vector<cx<R>> y(n);
  for (size_t c = 0; c < n; ++c)
    for (size_t r = 0; r < n; ++r) y[r] += W[r + n * c] * v[c];
  return y;
}

template <typename R>
inline std::vector<cx<R>> adj_matvec(const std::vector<cx<R>>& W, const std::vector<cx<R>>& v) {
  const size_t n = v.size();
  std::vector<cx<R>> y(n);
  for (size_t c = 0; c < n; ++c)
    for (size_t r = 0; r < n; ++r) y[c] += conj(W[r + n * c]) * v[r];
  return y;
}

template <typename R>
inline bool within(const std::vector<cx<R>>& v, R tol) {
  for (const auto& x : v)
    if (!(std::fabs(x.re) <= tol && std::fabs(x.im) <= tol)) return false;
  return true;
}

struct Breakdown {};
template <typename R> inline void nz(cx<R> v) { if (is_zero(v)) throw Breakdown{}; }
template <typename R> inline cx<R> cdivc(cx<R> a, cx<R> b) { nz(b); return a / b; }
template <typename R> inline R pos(R v) { if (!(std::isfinite(v) && v > R(0))) throw Breakdown{}; return v; }
template <typename R> inline R nonneg(R v) { if (!(std::isfinite(v) && v >= R(0))) throw Breakdown{}; return v; }
template <typename R> inline R scaled(R tol, R scale) {
  const R s = tol * scale;
  if (!(std::isfinite(s) && s >= R(0))) throw Breakdown{};
  return s;
}

// FEFF ggbi: one BiCGSTAB step that returns after the first update.
template <typename R>
int bicgstab(const std::vector<cx<R>>& W, size_t src, R tol, std::vector<cx<R>>& x, int& ord) {
  ord = 0;
  const size_t n = x.size();
  const cx<R> zero;
  std::fill(x.begin(), x.end(), zero);
  std::vector<cx<R>> r(n);
  r[src] = cx<R>(R(1), R(0));
  if (within(r, tol)) return OK;
  std::vector<cx<R>> p = r, a = matvec(W, p);
  ++ord;
  cx<R> aa = cdot(a, a), wa = cdot(r, a), aw = conj(wa), ww = cdot(r, r);
  nz(aa);
  nz(ww);
  const cx<R> dd = aa * ww - aw * wa;
  const cx<R> sdd = cdivc(cdivc(dd, aa), ww);
  std::vector<cx<R>> y(n);
  if (cnorm(sdd) < R(1.0e-8)) {
    for (size_t i = 0; i < n; ++i) y[i] = r[i] / ww;
  } else {
    nz(dd);
    ww = (ww - aw) / dd;
    aa = (wa - aa) / dd;
    for (size_t i = 0; i < n; ++i) y[i] = r[i] * aa + a[i] * ww;
  }
  const cx<R> del = cdot(y, r), delp = cdot(y, a);
  const cx<R> omega = cdivc(del, delp);
  std::vector<cx<R>> sv(n);
  for (size_t i = 0; i < n; ++i) sv[i] = r[i] - omega * a[i];
  if (within(sv, tol)) {
    for (size_t i = 0; i < n; ++i) x[i] += omega * p[i];
    return OK;
  }
  const std::vector<cx<R>> as = matvec(W, sv);
  ++ord;
  const cx<R> a2 = cdot(as, as), w2 = cdot(as, sv);
  const cx<R> chi = cdivc(w2, a2);
  for (size_t i = 0; i < n; ++i) x[i] += omega * p[i] + chi * sv[i];
  return OK;
}

// FEFF ggrm: two-sided Lanczos recursion with restarts.
template <typename R>
int recursion(const std::vector<cx<R>>& W, size_t src, R tol, std::vector<cx<R>>& x, int& ord) {
  ord = 0;
  const size_t n = x.size();
  const cx<R> zero, one(R(1), R(0));
  std::fill(x.begin(), x.end(), zero);
  for (int restart = 0; restart < 128; ++restart) {
    std::vector<cx<R>> r = restart > 0 ? matvec(W, x) : std::vector<cx<R>>(n);
    r[src] -= one;
    std::vector<cx<R>> xket(n);
    for (size_t i = 0; i < n; ++i) xket[i] = -r[i];
    const cx<R> rn = cdot(xket, xket);
    if (is_zero(rn)) return OK;
    const R xf = R(1) / pos(rn.re);
    std::vector<cx<R>> xbra(n);
    for (size_t i = 0; i < n; ++i) xbra[i] = xket[i] * xf;
    std::vector<cx<R>> tket = matvec(W, xket);
    ++ord;
    cx<R> aa = cdot(xbra, tket), aac = conj(aa), bb, bbc, betac = aa;
    nz(betac);
    cx<R> yy = one;
    std::vector<cx<R>> xketp(n), xbrap(n), z = xket, sv = tket;
    for (size_t i = 0; i < n; ++i) x[i] += z[i] / betac;
    for (size_t i = 0; i < n; ++i) r[i] += sv[i] / betac;
    for (int it = 0; it < 100; ++it) {
      for (size_t i = 0; i < n; ++i) tket[i] -= aa * xket[i] + bb * xketp[i];
      std::vector<cx<R>> tbra = adj_matvec(W, xbra);
      for (size_t i = 0; i < n; ++i) tbra[i] -= aac * xbra[i] + bbc * xbrap[i];
      const cx<R> rnorm = cdot(tbra, tket);
      if (is_zero(rnorm)) return OK;
      bb = csqrt(rnorm);
      bbc = conj(bb);
      nz(bb);
      nz(bbc);
      xketp = xket;
      xbrap = xbra;
      for (size_t i = 0; i < n; ++i) xket[i] = tket[i] / bb;
      for (size_t i = 0; i < n; ++i) xbra[i] = tbra[i] / bbc;
      tket = matvec(W, xket);
      ++ord;
      aa = cdot(xbra, tket);
      aac = conj(aa);
      const cx<R> alphac = cdivc(bb, betac);
      for (size_t i = 0; i < n; ++i) {
        z[i] = xket[i] - alphac * z[i];
        sv[i] = tket[i] - alphac * sv[i];
      }
      betac = aa - alphac * bb;
      nz(betac);
      yy = -alphac * yy;
      const cx<R> gamma = cdivc(yy, betac);
      for (size_t i = 0; i < n; ++i) {
        x[i] += gamma * z[i];
        r[i] += gamma * sv[i];
      }
      if (within(r, tol)) return OK;
    }
  }
  return ERR_NO_CONVERGENCE;
}

// FEFF gggm: Graves-Morris on W = T G0 (no identity), restarted.
template <typename R>
int graves_morris(const std::vector<cx<R>>& W, size_t src, R tol, std::vector<cx<R>>& x, int& ord) {
  ord = 0;
  const size_t n = x.size();
  const cx<R> zero, one(R(1), R(0));
  std::fill(x.begin(), x.end(), zero);
  std::vector<cx<R>> b(n), x0(n);
  cx<R> q0 = one;
  b[src] = one;
  for (int restart = 0; restart < 128; ++restart) {
    if (restart > 0) {
      nz(q0);
      for (size_t i = 0; i < n; ++i) x[i] += x0[i] / q0;
      const std::vector<cx<R>> av = matvec(W, x);
      for (size_t i = 0; i < n; ++i) b[i] = av[i] - x[i];
      b[src] += one;
    }
    std::vector<cx<R>> r0 = b;
    std::fill(x0.begin(), x0.end(), zero);
    std::vector<cx<R>> x1 = b, r1 = matvec(W, b);
    ++ord;
    cx<R> ww = cdot(r0, r0), aa = cdot(r1, r1);
    const cx<R> wa = cdot(r0, r1), aw = conj(wa);
    nz(aa);
    nz(ww);
    const cx<R> dd = aa * ww - aw * wa;
    const cx<R> sdd = cdivc(cdivc(dd, aa), ww);
    std::vector<cx<R>> wv(n);
    if (cnorm(sdd) < R(1.0e-8)) {
      for (size_t i = 0; i < n; ++i) wv[i] = r0[i] / ww;
    } else {
      nz(dd);
      ww = (ww - aw) / dd;
      aa = (wa - aa) / dd;
      for (size_t i = 0; i < n; ++i) wv[i] = r0[i] * aa + r1[i] * ww;
    }
    cx<R> e0 = cdot(wv, r0), e1 = cdot(wv, r1);
    q0 = one;
    cx<R> q1 = one;
    for (int it = 0; it < 10; ++it) {
      R t1 = scaled(tol, cnorm(q1) / R(10));
      if (within(r1, t1)) {
        nz(q1);
        for (size_t i = 0; i < n; ++i) x[i] += x1[i] / q1;
        return OK;
      }
      const cx<R> alpha = cdivc(e1, e0);
      std::vector<cx<R>> t0(n);
      for (size_t i = 0; i < n; ++i) t0[i] = r1[i] - alpha * r0[i];
      const std::vector<cx<R>> tv = matvec(W, t0);
      ++ord;
      const cx<R> wa2 = cdot(t0, tv), ww2 = cdot(t0, t0), aa2 = cdot(tv, tv), aw2 = conj(wa2);
      const cx<R> theta = cdivc(wa2 - aa2, ww2 - aw2);
      for (size_t i = 0; i < n; ++i) r0[i] = tv[i] - theta * t0[i];
      const cx<R> d1 = one - theta;
      for (size_t i = 0; i < n; ++i) x0[i] = t0[i] + d1 * (x1[i] - alpha * x0[i]);
      q0 = d1 * (q1 - alpha * q0);
      R t0l = scaled(tol, cnorm(q0));
      if (within(r0, t0l)) {
        nz(q0);
        for (size_t i = 0; i < n; ++i) x[i] += x0[i] / q0;
        return OK;
      }
      e0 = cdot(wv, r0);
      const cx<R> beta = cdivc(e0, e1);
      for (size_t i = 0; i < n; ++i) t0[i] = r0[i] - beta * r1[i];
      const std::vector<cx<R>> av = matvec(W, t0);
      ++ord;
      const cx<R> d2 = beta * theta;
      for (size_t i = 0; i < n; ++i) r1[i] = av[i] + d2 * r1[i];
      e1 = cdot(wv, r1);
      const cx<R> d3 = beta * (one - theta);
      for (size_t i = 0; i < n; ++i) x1[i] = x0[i] - d3 * x1[i] + t0[i];
      q1 = q0 - (one - theta) * beta * q1;
    }
  }
  return ERR_NO_CONVERGENCE;
}

// FEFF ggtf: transpose-free QMR, 21 half-steps per restart.
template <typename R>
int tfqmr(const std::vector<cx<R>>& W, size_t src, R tol, std::vector<cx<R>>& x, int& ord) {
  ord = 0;
  const size_t n = x.size();
  const cx<R> zero;
  std::fill(x.begin(), x.end(), zero);
  std::vector<cx<R>> a(n);
  for (int restart = 0; restart < 128; ++restart) {
    if (restart > 0) a = matvec(W, x);
    std::vector<cx<R>> u(n);
    for (size_t i = 0; i < n; ++i) u[i] = -a[i];
    u[src] += cx<R>(R(1), R(0));
    a = matvec(W, u);
    ++ord;
    std::vector<cx<R>> w = u, v = a, d(n);
    const cx<R> aa0 = cdot(u, u);
    nz(aa0);
    R tau = std::sqrt(pos(aa0.re));
    R nu = R(0);
    cx<R> eta, alpha, rho(R(1), R(0));
    std::vector<cx<R>> rv(n);
    for (size_t i = 0; i < n; ++i) rv[i] = u[i] / aa0;
    for (int nit = 0; nit <= 20; ++nit) {
      if (nit % 2 == 0) alpha = cdivc(rho, cdot(rv, v));
      else {
        a = matvec(W, u);
        ++ord;
      }
      for (size_t i = 0; i < n; ++i) w[i] -= alpha * a[i];
      const cx<R> f = cdivc(eta * (nu * nu), alpha);
      const std::vector<cx<R>> dp = d;
      for (size_t i = 0; i < n; ++i) d[i] = u[i] + f * dp[i];
      const cx<R> wn = cdot(w, w);
      const R norm = std::sqrt(nonneg(wn.re));
      nu = norm / tau;
      const R cm = R(1) / std::sqrt(R(1) + nu * nu);
      tau *= nu * cm;
      eta = alpha * (cm * cm);
      for (size_t i = 0; i < n; ++i) x[i] += eta * d[i];
      const R err = tau * std::sqrt((R(1) + R(nit)) / R(n)) * R(10);
      if (std::fabs(err) < tol) return OK;
      if (nit % 2 != 0) {
        const cx<R> prho = rho;
        rho = cdot(rv, w);
        const cx<R> beta = cdivc(rho, prho);
        for (size_t i = 0; i < n; ++i) u[i] = w[i] + beta * u[i];
        for (size_t i = 0; i < n; ++i) v[i] = beta * (a[i] + beta * v[i]);
        a = matvec(W, u);
        ++ord;
        for (size_t i = 0; i < n; ++i) v[i] += a[i];
      } else {
        for (size_t i = 0; i < n; ++i) u[i] -= alpha * v[i];
      }
    }
  }
  return ERR_NO_CONVERGENCE;
}

// fms_iterative_scattering_with_system (iterative.rs:38-179): absorber-range
// potentials, every source column of the representative block, gg = G0 x rows.
template <typename R>
inline int iterative_scattering(const Plan<R>& P, const std::vector<cx<R>>& g0, const std::vector<cx<R>>& t, int minv,
                                R toler1, R toler2, std::vector<cx<R>>& scat, std::vector<cx<R>>* system_out = nullptr,
                                int* order_out = nullptr) {
  const size_t n = P.n();
  std::vector<cx<R>> W(n * n);
  if (minv == 3) {
    // fms_graves_morris_system_matrix: + T G0, no identity
    for (size_t c = 0; c < n; ++c)
      for (size_t r = 0; r < n; ++r) {
        const cx<R> g = g0[r + n * c];
        if (cnorm(g) > toler2) W[r + n * c] += cx<R>(R(1), R(0)) * t[size_t(P.nsp) * r] * g;
        if (P.nsp == 2) {
          const long partner = spin_partner_index(P.kets[r], long(r), long(n));
          if (partner >= 0) {
            const cx<R> gf = g0[size_t(partner) + n * c];
            if (cnorm(gf) > toler2) W[r + n * c] += cx<R>(R(1), R(0)) * t[1 + 2 * size_t(partner)] * gf;
          }
        }
      }
  } else {
    iterative_system_matrix(P, g0, t, toler2, W);
  }
  const size_t C = size_t(P.nsp) * size_t((P.L + 1) * (P.L + 1));
  scat.assign(C * C * size_t(P.npot), cx<R>());
  if (system_out) *system_out = W;
  std::vector<cx<R>> x(n);
  int ord = 0;
  for (int p = P.pot_start; p <= P.pot_end; ++p) {
    const int lm = std::min(P.pot_lmax[size_t(p)], P.L);
    const size_t ipart = size_t(P.nsp) * size_t((lm + 1) * (lm + 1));
    const size_t off = size_t(P.rep_offsets[size_t(p)]);
    for (size_t c = 0; c < ipart; ++c) {
      int rc;
      try {
        switch (minv) {
          case 1: rc = bicgstab(W, off + c, toler1, x, ord); break;
          case 2: rc = recursion(W, off + c, toler1, x, ord); break;
          case 3: rc = graves_morris(W, off + c, toler1, x, ord); break;
          default: rc = tfqmr(W, off + c, toler1, x, ord); break;
        }
      } catch (const Breakdown&) {
        rc = ERR_BREAKDOWN;
      }
      if (rc != OK) return rc;
      for (size_t r = 0; r < ipart; ++r) {
        cx<R> v;
        for (size_t s = 0; s < n; ++s) v = v + g0[off + r + n * s] * x[s];
        scat[r + C * (c + C * size_t(p))] = v;
      }
      if (order_out) *order_out = ord;
    }
  }
  return OK;
}

}  // namespace oracle

// ===========================================================================
// C API for the tests (ctypes).  mode: 0 = f32-faithful, 1 = fp64.
// Complex values cross as interleaved doubles.
// ===========================================================================
using namespace oracle;

template <typename R>
static cx<R> ld(const double* p) { return cx<R>(R(p[0]), R(p[1])); }
template <typename R>
static void st(double* p, cx<R> v) { p[0] = double(v.re); p[1] = double(v.im); }

extern "C" {

int oracle_sort_atoms_by_radius(int n, float* pos, int* pots, double* keys) {
  std::vector<Atom> a(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) { std::memcpy(a[size_t(i)].pos, pos + 3 * i, 12); a[size_t(i)].pot = pots[i]; }
  for (auto& at : a)
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(at.pos[k])) return ERR_NONFINITE;
  std::vector<double> k;
  sort_atoms_by_radius(a, &k);
  for (int i = 0; i < n; ++i) { std::memcpy(pos + 3 * i, a[size_t(i)].pos, 12); pots[i] = a[size_t(i)].pot; keys[i] = k[size_t(i)]; }
  return OK;
}

int oracle_yprep_cluster(int central_potential, int n, const int* pots, const float* pos, float radius, int capacity,
                         float* out_pos, int* out_pots, int* out_n, int* central_atom, int* untruncated) {
  std::vector<Atom> out;
  size_t ca = 0, un = 0;
  int rc = yprep_cluster(central_potential, pots, pos, size_t(n), radius, size_t(capacity), out, &ca, &un);
  if (rc) return rc;
  for (size_t i = 0; i < out.size(); ++i) { std::memcpy(out_pos + 3 * i, out[i].pos, 12); out_pots[i] = out[i].pot; }
  *out_n = int(out.size());
  *central_atom = int(ca);
  *untruncated = int(un);
  return OK;
}

int oracle_sort_representative_atoms(int central_potential, int max_potential, int n, float* pos, int* pots,
                                     long* representative) {
  std::vector<Atom> a(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) { std::memcpy(a[size_t(i)].pos, pos + 3 * i, 12); a[size_t(i)].pot = pots[i]; }
  std::vector<long> rep;
  int rc = sort_representative_atoms(central_potential, size_t(max_potential), a, rep);
  if (rc) return rc;
  for (int i = 0; i < n; ++i) { std::memcpy(pos + 3 * i, a[size_t(i)].pos, 12); pots[i] = a[size_t(i)].pot; }
  for (int p = 0; p <= max_potential; ++p) representative[p] = rep[size_t(p)];
  return OK;
}

int oracle_pair_polar_angles(int mode, const float* pi, const float* pj, int same, double* theta, double* phi) {
  if (mode == 0) {
    float t, p;
    pair_polar_angles<float>(pi, pj, same != 0, &t, &p);
    *theta = t; *phi = p;
  } else {
    double t, p;
    pair_polar_angles<double>(pi, pj, same != 0, &t, &p);
    *theta = t; *phi = p;
  }
  return OK;
}

int oracle_rotation_matrix(int mode, int lmax, int mmax, double beta, double phi, int forward, double* out) {
  if (lmax < 0 || lmax > 24 || mmax < 0 || mmax > lmax) return ERR_INVALID_LIMIT;
  if (!std::isfinite(beta) || !std::isfinite(phi)) return ERR_NONFINITE;
  size_t sz = size_t(2 * lmax + 1) * size_t(2 * lmax + 1) * size_t(lmax + 1);
  if (mode == 0) {
    std::vector<cx<float>> t(sz);
    rotation_matrix<float>(lmax, mmax, float(beta), float(phi), forward != 0, t.data());
    for (size_t i = 0; i < sz; ++i) st(out + 2 * i, t[i]);
  } else {
    std::vector<cx<double>> t(sz);
    rotation_matrix<double>(lmax, mmax, beta, phi, forward != 0, t.data());
    for (size_t i = 0; i < sz; ++i) st(out + 2 * i, t[i]);
  }
  return OK;
}

int oracle_polynomials(int mode, int lx, int lmaxp1, int mmaxp1, const double* rho, double* out) {
  size_t sz = size_t(lx + 2) * size_t(2 * lx + 3);
  if (mode == 0) {
    std::vector<cx<float>> t(sz);
    int rc = rehr_albers_polynomials<float>(lx, lmaxp1, mmaxp1, ld<float>(rho), t.data());
    if (rc) return rc;
    for (size_t i = 0; i < sz; ++i) st(out + 2 * i, t[i]);
  } else {
    std::vector<cx<double>> t(sz);
    int rc = rehr_albers_polynomials<double>(lx, lmaxp1, mmaxp1, ld<double>(rho), t.data());
    if (rc) return rc;
    for (size_t i = 0; i < sz; ++i) st(out + 2 * i, t[i]);
  }
  return OK;
}

double oracle_legendre_normalization(int l, int m) { return legendre_normalization(l, m); }
double oracle_spin_orbit_coefficient(int plus, int l, int m, int spin) {
  return spin_orbit_coefficient(plus != 0, l, m, spin);
}

int oracle_t_matrix_phase(int mode, const double* phase, double* out) {
  if (mode == 0) st(out, t_matrix_phase(ld<float>(phase)));
  else st(out, t_matrix_phase(ld<double>(phase)));
  return OK;
}

int oracle_prefactor(int mode, const double* rho, const double* k, double msd, double* out) {
  if (mode == 0) st(out, free_propagator_prefactor(ld<float>(rho), ld<float>(k), float(msd)));
  else st(out, free_propagator_prefactor(ld<double>(rho), ld<double>(k), msd));
  return OK;
}

// Dense LU factor + solve (column-major), for the linalg known-answer test
// and for the GPU LU parity tests.
int oracle_lu_factor_solve(int mode, int n, double* A, int m, double* B, long* piv_out, long* singular_pivot) {
  size_t N = size_t(n);
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    std::vector<cx<R>> a(N * N), b(N * size_t(m));
    for (size_t i = 0; i < N * N; ++i) a[i] = ld<R>(A + 2 * i);
    for (size_t i = 0; i < N * size_t(m); ++i) b[i] = ld<R>(B + 2 * i);
    std::vector<size_t> piv;
    int rc = lu_factor(a.data(), N, piv, singular_pivot);
    if (rc) return rc;
    lu_solve(a.data(), N, piv, b.data(), size_t(m));
    for (size_t i = 0; i < N * N; ++i) st(A + 2 * i, a[i]);
    for (size_t i = 0; i < N * size_t(m); ++i) st(B + 2 * i, b[i]);
    for (size_t i = 0; i < N; ++i) piv_out[i] = long(piv[i]);
    return OK;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

// Plan-level entry: the cluster is already yprep-prepared (absorber first).
// positions: 3N floats; pots: N ints; lmaxph: npot ints; sigsqr: NxN col-major (may be null).
// wave_numbers: E*nsp complex; xphase: E * nsp*(2L+1)*npot complex (per-energy blocks).
// Outputs (may be null): scattering E*(C*C*npot) complex; g0/system/t for energy 0 only.
int oracle_fms_spectrum(int mode, int n_atoms, const float* positions, const int* pots, int nsp, int ispin,
                        int lfms, int max_potential, int global_lmax, const int* lmaxph, double rdirec,
                        const float* sigsqr, double sig2g, int n_energies, const double* wave_numbers, const double* xphase,
                        double* scattering_out, int* status_out, int n_threads) {
  std::vector<Atom> atoms(static_cast<size_t>(n_atoms));
  for (int i = 0; i < n_atoms; ++i) { std::memcpy(atoms[size_t(i)].pos, positions + 3 * i, 12); atoms[size_t(i)].pot = pots[i]; }
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    Plan<R> P;
    int rc = make_plan<R>(P, atoms.data(), n_atoms, nsp, ispin, lfms, max_potential, global_lmax, lmaxph, R(float(rdirec)),
                          sigsqr, float(sig2g));
    if (rc) return rc;
    const size_t C = size_t(P.nsp) * size_t((P.L + 1) * (P.L + 1));
    const size_t scat_sz = C * C * size_t(P.npot);
    const size_t xph_sz = size_t(P.nsp) * size_t(2 * P.L + 1) * size_t(P.npot);
    int first_error = OK;
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads > 0 ? n_threads : 1)
    for (int e = 0; e < n_energies; ++e) {
      std::vector<cx<R>> k(static_cast<size_t>(P.nsp)), xp(xph_sz), g0, t, scat;
      for (int s = 0; s < P.nsp; ++s) k[size_t(s)] = ld<R>(wave_numbers + 2 * (size_t(e) * size_t(P.nsp) + size_t(s)));
      for (size_t i = 0; i < xph_sz; ++i) xp[i] = ld<R>(xphase + 2 * (size_t(e) * xph_sz + i));
      int erc = free_propagator_matrix(P, k.data(), g0);
      if (erc == OK) {
        t_matrix_table(P, xp.data(), t);
        long sp = -1;
        erc = lu_scattering(P, g0, t, scat, &sp);
      }
      if (status_out) status_out[e] = erc;
      if (erc != OK) {
#pragma omp critical
        if (first_error == OK) first_error = erc;
        continue;
      }
      if (scattering_out)
        for (size_t i = 0; i < scat_sz; ++i) st(scattering_out + 2 * (size_t(e) * scat_sz + i), scat[i]);
    }
    return first_error;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

// Iterative forms (minv != 0) of oracle_fms_spectrum: toler1 = convergence,
// toler2 = G0 drop tolerance, both narrowed to f32 like the reference.
int oracle_fms_spectrum_iterative(int mode, int minv, double toler1, double toler2, int n_atoms, const float* positions,
                                  const int* pots, int nsp, int ispin, int lfms, int max_potential, int global_lmax,
                                  const int* lmaxph, double rdirec, const float* sigsqr, double sig2g, int n_energies,
                                  const double* wave_numbers, const double* xphase, double* scattering_out,
                                  int* status_out, int n_threads) {
  std::vector<Atom> atoms(static_cast<size_t>(n_atoms));
  for (int i = 0; i < n_atoms; ++i) { std::memcpy(atoms[size_t(i)].pos, positions + 3 * i, 12); atoms[size_t(i)].pot = pots[i]; }
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    Plan<R> P;
    int rc = make_plan<R>(P, atoms.data(), n_atoms, nsp, ispin, lfms, max_potential, global_lmax, lmaxph, R(float(rdirec)),
                          sigsqr, float(sig2g));
    if (rc) return rc;
    const size_t C = size_t(P.nsp) * size_t((P.L + 1) * (P.L + 1));
    const size_t scat_sz = C * C * size_t(P.npot);
    const size_t xph_sz = size_t(P.nsp) * size_t(2 * P.L + 1) * size_t(P.npot);
    int first_error = OK;
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads > 0 ? n_threads : 1)
    for (int e = 0; e < n_energies; ++e) {
      std::vector<cx<R>> k(static_cast<size_t>(P.nsp)), xp(xph_sz), g0, t, scat;
      for (int s = 0; s < P.nsp; ++s) k[size_t(s)] = ld<R>(wave_numbers + 2 * (size_t(e) * size_t(P.nsp) + size_t(s)));
      for (size_t i = 0; i < xph_sz; ++i) xp[i] = ld<R>(xphase + 2 * (size_t(e) * xph_sz + i));
      int erc = free_propagator_matrix(P, k.data(), g0);
      if (erc == OK) {
        t_matrix_table(P, xp.data(), t);
        erc = iterative_scattering(P, g0, t, minv, R(float(toler1)), R(float(toler2)), scat);
      }
      if (status_out) status_out[e] = erc;
      if (erc != OK) {
#pragma omp critical
        if (first_error == OK) first_error = erc;
        continue;
      }
      if (scattering_out)
        for (size_t i = 0; i < scat_sz; ++i) st(scattering_out + 2 * (size_t(e) * scat_sz + i), scat[i]);
    }
    return first_error;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

// fms_driver_setup for the known-answer test (driver.rs:4-65): returns the
// clamped potential lmax, active potential range, representative offsets and kets.
int oracle_driver_setup(int n_atoms, const int* pots, int nsp, int lfms, int max_potential, int global_lmax,
                        const int* raw_lmax, int* pot_lmax_out, int* range_out, long* rep_out, int* n_states,
                        int* kets4_out, int kets_capacity) {
  std::vector<Atom> atoms(static_cast<size_t>(n_atoms));
  for (int i = 0; i < n_atoms; ++i) { atoms[size_t(i)].pos[0] = atoms[size_t(i)].pos[1] = atoms[size_t(i)].pos[2] = 0.f; atoms[size_t(i)].pot = pots[i]; }
  Plan<double> P;
  if (n_atoms <= 0) return ERR_EMPTY_CLUSTER;
  if (nsp < 1 || nsp > 2) return ERR_INVALID_ARGUMENT;
  P.nsp = nsp;
  P.L = global_lmax;
  P.npot = max_potential + 1;
  P.pot_lmax.resize(size_t(P.npot));
  for (int p = 0; p < P.npot; ++p) P.pot_lmax[size_t(p)] = clamp_lipotx(raw_lmax[p], global_lmax);
  std::vector<int> ap(static_cast<size_t>(n_atoms));
  for (int a = 0; a < n_atoms; ++a) {
    if (pots[a] < 0 || pots[a] > max_potential) return ERR_POTENTIAL_RANGE;
    ap[size_t(a)] = pots[a];
  }
  int rc = construct_state_kets(nsp, ap, P.pot_lmax, global_lmax, P.kets, P.rep_offsets);
  if (rc) return rc;
  int start = lfms == 0 ? ap[0] : 0, end = lfms == 0 ? ap[0] : max_potential;
  for (int p = start; p <= end; ++p)
    if (P.rep_offsets[size_t(p)] < 0) return ERR_MISSING_REPRESENTATIVE;
  for (int p = 0; p < P.npot; ++p) { pot_lmax_out[p] = P.pot_lmax[size_t(p)]; rep_out[p] = P.rep_offsets[size_t(p)]; }
  range_out[0] = start;
  range_out[1] = end;
  *n_states = int(P.kets.size());
  for (size_t i = 0; i < P.kets.size() && int(i) < kets_capacity; ++i) {
    kets4_out[4 * i] = P.kets[i].atom; kets4_out[4 * i + 1] = P.kets[i].l;
    kets4_out[4 * i + 2] = P.kets[i].m; kets4_out[4 * i + 3] = P.kets[i].spin;
  }
  return OK;
}

// Single-energy intermediates for tests: G0 (n x n), compact T (nsp x n),
// LU system matrix (n x n), iterative system matrix (n x n, toler2 cutoff).
int oracle_fms_energy_intermediates(int mode, int n_atoms, const float* positions, const int* pots, int nsp,
                                    int ispin, int lfms, int max_potential, int global_lmax, const int* lmaxph,
                                    double rdirec,
                                    const float* sigsqr, double sig2g, const double* wave_numbers,
                                    const double* xphase, double toler2, int* n_states, double* g0_out,
                                    double* t_out, double* a_out, double* ait_out) {
  std::vector<Atom> atoms(static_cast<size_t>(n_atoms));
  for (int i = 0; i < n_atoms; ++i) { std::memcpy(atoms[size_t(i)].pos, positions + 3 * i, 12); atoms[size_t(i)].pot = pots[i]; }
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    Plan<R> P;
    int rc = make_plan<R>(P, atoms.data(), n_atoms, nsp, ispin, lfms, max_potential, global_lmax, lmaxph, R(float(rdirec)),
                          sigsqr, float(sig2g));
    if (rc) return rc;
    *n_states = int(P.n());
    if (!g0_out) return OK;
    const size_t xph_sz = size_t(P.nsp) * size_t(2 * P.L + 1) * size_t(P.npot);
    std::vector<cx<R>> k(static_cast<size_t>(P.nsp)), xp(xph_sz), g0, t, A, Ait;
    for (int s = 0; s < P.nsp; ++s) k[size_t(s)] = ld<R>(wave_numbers + 2 * size_t(s));
    for (size_t i = 0; i < xph_sz; ++i) xp[i] = ld<R>(xphase + 2 * i);
    rc = free_propagator_matrix(P, k.data(), g0);
    if (rc) return rc;
    t_matrix_table(P, xp.data(), t);
    lu_system_matrix(P, g0, t, A);
    iterative_system_matrix(P, g0, t, R(float(toler2)), Ait);
    const size_t n = P.n();
    for (size_t i = 0; i < n * n; ++i) st(g0_out + 2 * i, g0[i]);
    if (t_out)
      for (size_t i = 0; i < t.size(); ++i) st(t_out + 2 * i, t[i]);
    if (a_out)
      for (size_t i = 0; i < n * n; ++i) st(a_out + 2 * i, A[i]);
    if (ait_out)
      for (size_t i = 0; i < n * n; ++i) st(ait_out + 2 * i, Ait[i]);
    return OK;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

// The dense system of one energy as the LU form solves it
// (crates/refeff-core/src/fms/internals/linear.rs:102-135 and
// solvers.rs:434-446): A = I - G0 T (n x n, column-major) and the absorber's
// right-hand sides B = G0[:, off .. off + ipart) (n x ipart), for an
// independent host solve.  With a_out null only n, off and ipart are set.
// G0 columns are built on `threads` OpenMP threads.
int oracle_fms_lu_system(int mode, int n_atoms, const float* positions, const int* pots, int nsp, int ispin,
                         int global_lmax, const int* lmaxph, int npot, double rdirec, const float* sigsqr, double sig2g,
                         const double* wave_numbers, const double* xphase, int threads, long* n_states,
                         long* absorber_offset, long* absorber_width, double* a_out, double* b_out) {
  std::vector<Atom> atoms(static_cast<size_t>(n_atoms));
  for (int i = 0; i < n_atoms; ++i) { std::memcpy(atoms[size_t(i)].pos, positions + 3 * i, 12); atoms[size_t(i)].pot = pots[i]; }
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    Plan<R> P;
    int rc = make_plan<R>(P, atoms.data(), n_atoms, nsp, ispin, 0, npot - 1, global_lmax, lmaxph, R(float(rdirec)),
                          sigsqr, float(sig2g));
    if (rc) return rc;
    const size_t n = P.n();
    const int lm = std::min(P.pot_lmax[0], P.L);
    const size_t ipart = size_t(P.nsp) * size_t((lm + 1) * (lm + 1));
    const size_t off = size_t(P.rep_offsets[0]);
    *n_states = long(n);
    *absorber_offset = long(off);
    *absorber_width = long(ipart);
    if (!a_out) return OK;
    const size_t xph_sz = size_t(P.nsp) * size_t(2 * P.L + 1) * size_t(P.npot);
    std::vector<cx<R>> k(static_cast<size_t>(P.nsp)), xp(xph_sz), g0, t;
    for (int s = 0; s < P.nsp; ++s) k[size_t(s)] = ld<R>(wave_numbers + 2 * size_t(s));
    for (size_t i = 0; i < xph_sz; ++i) xp[i] = ld<R>(xphase + 2 * i);
    rc = free_propagator_matrix(P, k.data(), g0, threads);
    if (rc) return rc;
    t_matrix_table(P, xp.data(), t);
    // A = I - G0 T written straight into the caller's buffer (lu_system_matrix's arithmetic, column by column)
#pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : 1)
    for (long cv = 0; cv < long(n); ++cv) {
      const size_t c = size_t(cv);
      const long partner = P.nsp == 2 ? spin_partner_index(P.kets[c], long(c), long(n)) : -1;
      for (size_t r = 0; r < n; ++r) {
        cx<R> v = (-g0[r + n * c]) * t[size_t(P.nsp) * c];
        if (partner >= 0) v -= g0[r + n * size_t(partner)] * t[1 + 2 * c];
        if (r == c) v += cx<R>(R(1), R(0));
        st(a_out + 2 * (r + n * c), v);
      }
    }
    for (size_t c = 0; c < ipart; ++c)
      for (size_t r = 0; r < n; ++r) st(b_out + 2 * (r + n * c), g0[r + n * (off + c)]);
    return OK;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

// Explicit-state entry points used to pin the oracle to the reference's
// known-answer tests, which call the kernels with hand-built G0/T tables.
// g0: n x n col-major, t: (nsp, n) compact table.  Kets given as (atom,l,m,spin) quadruples.
int oracle_lu_scattering_explicit(int mode, int n, const int* kets4, int nsp, int global_lmax, int npot,
                                  const int* pot_lmax, const long* rep_offsets, int pot_start, int pot_end,
                                  const double* g0_in, const double* t_in, double* system_out, double* scat_out) {
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    Plan<R> P;
    P.nsp = nsp;
    P.L = global_lmax;
    P.npot = npot;
    P.pot_lmax.assign(pot_lmax, pot_lmax + npot);
    P.rep_offsets.assign(rep_offsets, rep_offsets + npot);
    P.pot_start = pot_start;
    P.pot_end = pot_end;
    P.kets.resize(size_t(n));
    for (int i = 0; i < n; ++i) P.kets[size_t(i)] = {kets4[4 * i], kets4[4 * i + 1], kets4[4 * i + 2], kets4[4 * i + 3]};
    for (int p = pot_start; p <= pot_end; ++p)
      if (p < 0 || p >= npot || P.rep_offsets[size_t(p)] < 0) return ERR_MISSING_REPRESENTATIVE;
    std::vector<cx<R>> g0(size_t(n) * size_t(n)), t(size_t(nsp) * size_t(n)), A, scat;
    for (size_t i = 0; i < g0.size(); ++i) g0[i] = ld<R>(g0_in + 2 * i);
    for (size_t i = 0; i < t.size(); ++i) t[i] = ld<R>(t_in + 2 * i);
    lu_system_matrix(P, g0, t, A);
    if (system_out)
      for (size_t i = 0; i < A.size(); ++i) st(system_out + 2 * i, A[i]);
    long sp = -1;
    int rc = lu_scattering(P, g0, t, scat, &sp);
    if (rc) return rc;
    for (size_t i = 0; i < scat.size(); ++i) st(scat_out + 2 * i, scat[i]);
    return OK;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

// Iterative forms on explicit G0 / T tables (the reference's solver tests):
// system matrix, scattering table and the last solve's multiple-scattering order.
int oracle_iterative_scattering_explicit(int mode, int minv, int n, const int* kets4, int nsp, int global_lmax, int npot,
                                         const int* pot_lmax, const long* rep_offsets, int pot_start, int pot_end,
                                         const double* g0_in, const double* t_in, double toler1, double toler2,
                                         double* system_out, double* scat_out, int* order_out) {
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    Plan<R> P;
    P.nsp = nsp;
    P.L = global_lmax;
    P.npot = npot;
    P.pot_lmax.assign(pot_lmax, pot_lmax + npot);
    P.rep_offsets.assign(rep_offsets, rep_offsets + npot);
    P.pot_start = pot_start;
    P.pot_end = pot_end;
    P.kets.resize(size_t(n));
    for (int i = 0; i < n; ++i) P.kets[size_t(i)] = {kets4[4 * i], kets4[4 * i + 1], kets4[4 * i + 2], kets4[4 * i + 3]};
    for (int p = pot_start; p <= pot_end; ++p)
      if (p < 0 || p >= npot || P.rep_offsets[size_t(p)] < 0) return ERR_MISSING_REPRESENTATIVE;
    std::vector<cx<R>> g0(size_t(n) * size_t(n)), t(size_t(nsp) * size_t(n)), W, scat;
    for (size_t i = 0; i < g0.size(); ++i) g0[i] = ld<R>(g0_in + 2 * i);
    for (size_t i = 0; i < t.size(); ++i) t[i] = ld<R>(t_in + 2 * i);
    int rc = iterative_scattering(P, g0, t, minv, R(float(toler1)), R(float(toler2)), scat, &W, order_out);
    if (system_out)
      for (size_t i = 0; i < W.size(); ++i) st(system_out + 2 * i, W[i]);
    if (rc) return rc;
    for (size_t i = 0; i < scat.size(); ++i) st(scat_out + 2 * i, scat[i]);
    return OK;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

int oracle_iterative_system_explicit(int mode, int n, const int* kets4, int nsp, const double* g0_in,
                                     const double* t_in, double toler2, double* out) {
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    Plan<R> P;
    P.nsp = nsp;
    P.kets.resize(size_t(n));
    for (int i = 0; i < n; ++i) P.kets[size_t(i)] = {kets4[4 * i], kets4[4 * i + 1], kets4[4 * i + 2], kets4[4 * i + 3]};
    std::vector<cx<R>> g0(size_t(n) * size_t(n)), t(size_t(nsp) * size_t(n)), A;
    for (size_t i = 0; i < g0.size(); ++i) g0[i] = ld<R>(g0_in + 2 * i);
    for (size_t i = 0; i < t.size(); ++i) t[i] = ld<R>(t_in + 2 * i);
    iterative_system_matrix(P, g0, t, R(float(toler2)), A);
    for (size_t i = 0; i < A.size(); ++i) st(out + 2 * i, A[i]);
    return OK;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

// z-axis propagator (FEFF xgllm) for one pair with a given polynomial table
// (crates/refeff-core/src/fms/xgllm.rs:9-57); xclm as clm(l, m) col-major (lx+2, 2lx+3).
int oracle_xgllm(int mode, int lx, int mu, int l1, int l2, const double* clm_in, double* out) {
  if (mu > l1) return ERR_INVALID_LIMIT;
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    const int rows = lx + 2;
    auto X = [&](int l, int m) { return ld<R>(clm_in + 2 * (size_t(l) + size_t(rows) * size_t(m))); };
    if (mu > l2) { st(out, cx<R>()); return OK; }
    R n1 = R(float(legendre_normalization(l1, mu))), n2 = R(float(legendre_normalization(l2, mu)));
    if (!(n1 != R(0)) || !(n2 != R(0))) return ERR_INVALID_LIMIT;
    cx<R> w(R(2 * l1 + 1), R(0));
    R sign = (mu % 2 == 0) ? R(1) : R(-1);
    int numax = std::min(l1, l2 - mu);
    cx<R> sum;
    for (int nu = 0; nu <= numax; ++nu) {
      cx<R> gamtl = w * X(l1, nu) / n1;
      cx<R> gam = X(l2, mu + nu) * (sign * n2);
      sum += gamtl * gam;
    }
    st(out, sum);
    return OK;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

// Spin-orbit / non-spin T element for the KAT (t_matrix.rs:10-143).
// xphase: (nsp_table, 2L+1, npot) column-major with nsp_table = phase spin axis length.
int oracle_t_matrix_element(int mode, int nsp, int ispin, int L, int npot, const double* xphase, const int* first4,
                            const int* second4, int pot, double* out) {
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    Plan<R> P;
    P.nsp = nsp;
    P.ispin = ispin;
    P.L = L;
    P.npot = npot;
    const size_t D = size_t(2 * L + 1);
    P.t3p.assign(size_t(L + 1) * D * 2, R(0));
    P.t3m.assign(size_t(L + 1) * D * 2, R(0));
    for (int l = 0; l <= L; ++l)
      for (int m = -l; m <= l; ++m)
        for (int s = 1; s <= 2; ++s) {
          size_t idx = size_t(l) + size_t(L + 1) * (size_t(m + L) + D * size_t(s - 1));
          P.t3p[idx] = R(float(spin_orbit_coefficient(true, l, m, s)));
          P.t3m[idx] = R(float(spin_orbit_coefficient(false, l, m, s)));
        }
    // The phase table spin axis may be longer than nsp (the KAT uses 2).
    std::vector<cx<R>> xp(2 * D * size_t(npot));
    for (size_t i = 0; i < xp.size(); ++i) xp[i] = ld<R>(xphase + 2 * i);
    Ket a{first4[0], first4[1], first4[2], first4[3]}, b{second4[0], second4[1], second4[2], second4[3]};
    // phase_value indexes with P.nsp as the spin stride: use a 2-spin view.
    Plan<R> Q = P;
    Q.nsp = 2;
    auto val = [&]() {
      // Re-implement the branch selection with the caller's nsp but the 2-spin phase table.
      if (a.atom != b.atom) return cx<R>();
      bool same = a.l == b.l && a.m == b.m && a.spin == b.spin;
      int l1 = a.l;
      if (nsp == 1 && ispin == 0)
        return same ? t_matrix_phase(phase_value(Q, xp.data(), a.spin, l1, pot)) : cx<R>();
      if (same) {
        int cs = nsp == 1 ? (ispin > 0 ? 2 : 1) : a.spin;
        R minus = so_coef(P, false, l1, a.m, cs), plus = so_coef(P, true, l1, a.m, cs);
        return t_matrix_phase(phase_value(Q, xp.data(), a.spin, l1, pot)) * (minus * minus) +
               t_matrix_phase(phase_value(Q, xp.data(), a.spin, -l1, pot)) * (plus * plus);
      }
      if (nsp == 2 && a.l == b.l && a.m + a.spin == b.m + b.spin) {
        R mf = so_coef(P, false, l1, a.m, a.spin), ms = so_coef(P, false, l1, b.m, b.spin);
        R pf = so_coef(P, true, l1, a.m, a.spin), ps = so_coef(P, true, l1, b.m, b.spin);
        cx<R> mph = (t_matrix_phase(phase_value(Q, xp.data(), a.spin, l1, pot)) +
                     t_matrix_phase(phase_value(Q, xp.data(), b.spin, l1, pot))) * R(0.5);
        cx<R> pph = (t_matrix_phase(phase_value(Q, xp.data(), a.spin, -l1, pot)) +
                     t_matrix_phase(phase_value(Q, xp.data(), b.spin, -l1, pot))) * R(0.5);
        return mph * mf * ms + pph * pf * ps;
      }
      return cx<R>();
    };
    st(out, val());
    return OK;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

// One G0 element from explicit tables (pairs.rs:160-236 fms_free_propagator_element):
// clm: polynomial table for the pair (lx+2, 2lx+3); back/fwd rotations (2L+1,2L+1,L+1).
int oracle_free_propagator_element(int mode, int lx, int L, const int* first4, const int* second4, const double* rho,
                                   const double* k, double msd, const double* clm_in, const double* back_in,
                                   const double* fwd_in, double* out) {
  auto run = [&](auto tag) -> int {
    using R = decltype(tag);
    Ket a{first4[0], first4[1], first4[2], first4[3]}, b{second4[0], second4[1], second4[2], second4[3]};
    if (a.atom == b.atom || a.spin != b.spin) { st(out, cx<R>()); return OK; }
    cx<R> r = ld<R>(rho), kk = ld<R>(k);
    if (!is_finite(r)) return ERR_NONFINITE;
    if (is_zero(r)) return ERR_ZERO_RHO;
    if (!is_finite(kk)) return ERR_NONFINITE;
    if (!std::isfinite(msd)) return ERR_NONFINITE;
    const int rows = lx + 2;
    const size_t D = size_t(2 * L + 1);
    auto X = [&](int l, int m) { return ld<R>(clm_in + 2 * (size_t(l) + size_t(rows) * size_t(m))); };
    auto RB = [&](int m2, int m1, int l) { return ld<R>(back_in + 2 * (size_t(m2 + L) + D * (size_t(m1 + L) + D * size_t(l)))); };
    auto RF = [&](int m2, int m1, int l) { return ld<R>(fwd_in + 2 * (size_t(m2 + L) + D * (size_t(m1 + L) + D * size_t(l)))); };
    int l1 = a.l, l2 = b.l;
    cx<R> sum;
    for (int mu = -l1; mu <= l1; ++mu) {
      int amu = mu < 0 ? -mu : mu;
      cx<R> g;
      if (amu <= l2) {
        R n1 = R(float(legendre_normalization(l1, amu))), n2 = R(float(legendre_normalization(l2, amu)));
        cx<R> w(R(2 * l1 + 1), R(0));
        R sign = (amu % 2 == 0) ? R(1) : R(-1);
        int numax = std::min(l1, l2 - amu);
        for (int nu = 0; nu <= numax; ++nu) g += (w * X(l1, nu) / n1) * (X(l2, amu + nu) * (sign * n2));
      }
      sum += RB(mu, a.m, l1) * g * RF(b.m, mu, l2);
    }
    st(out, free_propagator_prefactor(r, kk, R(float(msd))) * sum);
    return OK;
  };
  return mode == 0 ? run(float(0)) : run(double(0));
}

}  // extern "C"
