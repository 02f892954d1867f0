// FF2X XANES mu(E) from the MKGTR trace (host code): the zero-temperature
// xscorr contour correction of the broadened cross section and the xmu.dat
// normalisation, the stage after MKGTR that turns gtr(E) into mu(E).
//
// Reference (crates/refeff-engine/src/ff2x.rs unless noted):
//   chia = s02 * gtr                       ff2x_xanes_fms_trace_for_spectrum  2569-2603
//   total / atomic / fine structure        ff2x_xanes_corrected_components    3186-3262
//   xscorr at zero electronic temperature  ff2x_xscorr                        4437-4641
//   lorenz, astep                          ff2x_xscorr_lorenz / _astep        5052-5076
//   normalisation and mu0, chi, mu         ff2x_xanes_xmu_dat_from_components 3309-3399
//   locat, terp / terpc window, polint     crates/refeff-core/src/interpolation.rs:119-135, 215-236, 338-446
//   vicorr Lorentzian broadening          ff2x_xanes_apply_vicorr_convolution 3265-3306
//   conv1 / conv                           crates/refeff-core/src/convolution/lorentzian.rs:4-100
//   sig_gk Debye factor on chi            ff2x_xanes_xmu_dat_from_components 3388-3397
//                                          (refeff_ff2x_debye_factor, after the mu(E) step)
//   xscorr at a finite temperature         ff2x_thermal_xscorr                4643-5050
//   xsect.dat reader and rdxbin handoff    crates/refeff-io/src/xsect_dat.rs  268-309, 394-760
#include <algorithm>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/refeff_fms.h"

namespace {

using cd = std::complex<double>;
constexpr double kEps4 = 1.0e-4;          // FF2X_EPS4 (ff2x.rs:41)
constexpr double kHartreeEv = 27.211396;  // HARTREE_EV (crates/refeff-core/src/constants.rs:18)
constexpr double kPi = 3.14159265358979323846;

// FEFF locat: how many grid points are <= x (bisection on an increasing grid).
size_t locat(double x, const double* xs, size_t n) {
  size_t lo = 0, hi = n + 1;
  while (hi - lo > 1) {
    const size_t mid = (lo + hi) / 2;
    if (x < xs[mid - 1]) hi = mid;
    else lo = mid;
  }
  return lo;
}

// Neville's recurrence on the points (xs, ys), started from the point nearest
// x and walking the tableau the way FEFF's polint does.
template <typename T>
bool polint(const double* xs, const T* ys, size_t n, double x, T& out) {
  std::vector<T> c(ys, ys + n), d(ys, ys + n);
  size_t ns = 0;
  double best = std::fabs(x - xs[0]);
  for (size_t i = 1; i < n; ++i)
    if (std::fabs(x - xs[i]) < best) {
      best = std::fabs(x - xs[i]);
      ns = i;
    }
  T y = ys[ns];
  for (size_t m = 1; m < n; ++m) {
    for (size_t i = 0; i + m < n; ++i) {
      const double ho = xs[i] - x, hp = xs[i + m] - x, den = ho - hp;
      if (den == 0.0) return false;
      const T w = (c[i + 1] - d[i]) / den;
      d[i] = w * hp;
      c[i] = w * ho;
    }
    T dy;
    if (2 * ns < n - m) {
      dy = c[ns];
    } else {
      dy = d[ns - 1];
      --ns;
    }
    y = y + dy;
  }
  out = y;
  return true;
}

// FEFF terp / terpc: an order-`order` polynomial through the order + 1 grid
// points around x (window from locat, clamped to the table).
template <typename T>
bool terp(const double* xs, const T* ys, size_t n, size_t order, double x, T& out) {
  if (n < order + 1) return false;
  const size_t located = locat(x, xs, n);
  size_t first = located > order / 2 ? located - order / 2 : 0;  // 1-based
  if (first < 1) first = 1;
  if (first > n - order) first = n - order;
  return polint(xs + first - 1, ys + first - 1, order + 1, x, out);
}

double astep(double xloss, double dele) {
  const double v = 0.5 + std::atan(dele / xloss) / kPi;
  return v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
}

cd lorenz(double xloss, double width, double dele) {
  const cd den(xloss * xloss - width * width + dele * dele, -2.0 * width * dele);
  return cd(xloss / kPi, 0.0) / den;
}

bool finite(cd z) { return std::isfinite(z.real()) && std::isfinite(z.imag()); }

// FEFF divides the broadened spectrum by the single-precision pi
// (crates/refeff-core/src/convolution.rs:17).
constexpr double kPiF32 = double(float(3.14159265358979323846));

// FEFF conv1: the Lorentzian (half width `width`) integral at x0 of the
// straight segment from (x1, y1) to (x2, y2), per real and imaginary part, with
// a series for short segments (|t| < 0.1).
cd conv1(double x1, double x2, cd y1, cd y2, double x0, double width) {
  const cd t = cd((x2 - x1) / 2.0, 0.0) / cd((x1 + x2) / 2.0 - x0, -width);
  auto part = [&](double slope, double mid) {
    const cd s(slope, 0.0), m(mid, 0.0);
    const cd v = std::abs(t) >= 0.1 ? s * 2.0 + (m - s / t) * std::log((cd(1.0, 0.0) + t) / (cd(1.0, 0.0) - t))
                                    : m * (2.0 * (t + t * t * t / 3.0)) - s * (2.0 * t * t / 3.0);
    return v.imag();
  };
  return cd(part((y2.real() - y1.real()) / 2.0, (y2.real() + y1.real()) / 2.0),
            part((y2.imag() - y1.imag()) / 2.0, (y2.imag() + y1.imag()) / 2.0));
}

// FEFF conv: the piecewise-linear spectrum over omega, extended past the last
// point by max(last spacing, 50 width) along its last slope, broadened at
// every omega.  False on bad input (fewer than two points, width <= 0, a
// repeated last energy, non-finite values).
bool lorentz_conv(const double* omega, const cd* y, size_t n, double width, std::vector<cd>& out) {
  if (n < 2 || !(width > 0.0) || !std::isfinite(width)) return false;
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(omega[i]) || !finite(y[i])) return false;
  const size_t last = n - 1, prev = n - 2;
  const double fs = omega[last] - omega[prev];
  if (fs == 0.0) return false;
  const double ew = std::max(fs, 50.0 * width);
  const double xlast = omega[last] + ew;
  const cd ylast = y[last] + (y[last] - y[prev]) * (ew / fs);
  out.assign(n, cd(0.0, 0.0));
  for (size_t r = 0; r < n; ++r) {
    cd sum(0.0, 0.0);
    for (size_t i = 0; i + 1 < n; ++i) sum += conv1(omega[i], omega[i + 1], y[i], y[i + 1], omega[r], width);
    sum += conv1(omega[last], xlast, y[last], ylast, omega[r], width);
    out[r] = sum / kPiF32;
  }
  return true;
}

// Zero-temperature xscorr: cchi[row] (row < ne1) = the broadened xmu minus xmu,
// xmu = xsec + chia * xsnorm.  The broadening is the arctangent step times the
// Fermi-level value plus a contour integral of xmu along the vertical contour
// and the horizontal grid beyond the Fermi level (below it for ispec 2).
int xscorr(int ispec, const cd* energy_in, size_t ne, size_t ne1, size_t fermi, const cd* xsec, const double* bg,
           const cd* chia, double vrcorr, std::vector<cd>& cchi, std::string& err) {
  if (ne1 < 2 || ne1 >= ne || fermi >= ne1) {
    err = "xscorr needs at least two horizontal points, a contour after them, and the Fermi row on the horizontal grid";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  std::vector<cd> energy(energy_in, energy_in + ne), xmu(ne);
  for (size_t r = 0; r < ne; ++r) {
    if (!finite(energy[r]) || !finite(xsec[r]) || !std::isfinite(bg[r]) || !finite(chia[r])) {
      err = "xscorr input row " + std::to_string(r) + " is not finite";
      return REFEFF_FMS_ERR_NONFINITE_INPUT;
    }
    xmu[r] = xsec[r] + chia[r] * bg[r];
  }
  const double xloss = energy[0].imag();
  if (!(xloss > 0.0)) {
    err = "xscorr needs a positive broadening (Im of the first energy)";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  double ef = energy[ne - 1].real();
  std::vector<double> omega(ne1);
  for (size_t r = 0; r < ne1; ++r) omega[r] = energy[r].real();
  cd scale(1.0, 0.0);
  const bool shifted = std::fabs(vrcorr) > kEps4;
  if (shifted) {
    // move the contour by vrcorr and rescale it to the horizontal xmu at the shifted Fermi level
    if (std::abs(xmu[fermi]) == 0.0) {
      err = "xscorr cannot rescale the contour from a zero Fermi-level xmu";
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    }
    ef -= vrcorr;
    cd at_ef;
    if (!terp(omega.data(), xmu.data(), ne1, 1, ef, at_ef)) {
      err = "xscorr interpolation at the shifted Fermi level failed";
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    }
    for (size_t r = ne1; r < ne; ++r) energy[r] -= cd(vrcorr, 0.0);
    scale = at_ef / xmu[fermi];
    for (size_t r = ne1; r < ne; ++r) xmu[r] *= scale;
  }
  // contour: the vertical points below the broadening, the Fermi point, then the
  // horizontal points past the Fermi level (ascending; descending for ispec 2)
  std::vector<cd> ze, zv;
  for (size_t r = ne1; r < ne; ++r)
    if (energy[r].imag() < xloss) {
      ze.push_back(energy[r]);
      zv.push_back(xmu[r]);
    }
  if (shifted) {
    ze.push_back(cd(ef, xloss));
    zv.push_back(scale * xmu[fermi]);
  } else {
    ze.push_back(energy[fermi]);
    zv.push_back(xmu[fermi]);
  }
  if (ispec != 2) {
    for (size_t r = 0; r < ne1; ++r)
      if (energy[r].real() - ef > kEps4) {
        ze.push_back(energy[r]);
        zv.push_back(xmu[r]);
      }
  } else {
    for (size_t r = ne1; r-- > 0;)
      if (ef - energy[r].real() > kEps4) {
        ze.push_back(energy[r]);
        zv.push_back(xmu[r]);
      }
  }
  if (ze.size() < 2) {
    err = "xscorr contour has fewer than two points";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  cchi.assign(ne1, cd(0.0, 0.0));
  const cd two_pi_i(0.0, 2.0 * kPi);
  for (size_t r = 0; r < ne1; ++r) {
    const double w = omega[r];
    const cd ref = (w >= ef) == (ispec == 2) ? xmu[fermi] * scale : xmu[r];
    const cd e1(w, xloss), e2(w, -xloss);
    const double dele = w - ef;
    cd conv = ref * astep(xloss, dele);
    if (ispec == 2) conv = ref - conv;
    const double dl = std::fabs(dele) < kEps4 ? 0.0 : dele;
    cd corr = lorenz(xloss, ze[0].imag(), dl) * (zv[0] - ref) * cd(0.0, ze[0].imag());
    for (size_t q = 0; q + 1 < ze.size(); ++q) {
      const cd z1 = ze[q], z2 = ze[q + 1], f1 = zv[q] - ref, f2 = zv[q + 1] - ref, dz = z2 - z1;
      if (std::abs(dz) == 0.0) {
        err = "xscorr contour repeats a point";
        return REFEFF_FMS_ERR_INVALID_ARGUMENT;
      }
      cd seg(0.0, 0.0);
      if (std::abs(z1 - e1) > kEps4 && std::abs(z2 - e1) > kEps4)
        seg = std::log((z2 - e1) / (z1 - e1)) * (f1 * (z2 - e1) + f2 * (e1 - z1));
      seg -= std::log((z2 - e2) / (z1 - e2)) * (f1 * (z2 - e2) + f2 * (e2 - z1));
      corr += seg / dz / two_pi_i;
    }
    if (ispec == 2) corr = -corr;
    cchi[r] = conv + corr - xmu[r];
  }
  return REFEFF_FMS_OK;
}

// ---------------------------------------------------------------------------
// Thermal xscorr (electronic temperature > 0; ff2x_thermal_xscorr,
// crates/refeff-engine/src/ff2x.rs:4643-4800).  The xsect.dat rows then hold
// the ne1 horizontal rows, ne1 loss rows (the horizontal energies at the loss
// width), 10 auxiliary rows, the Matsubara-like poles and a last row at the
// Fermi level.  Per horizontal row (photon energy w, loss-row value xmu0):
//   cchi = xmu0 * [FL(w) or 1 - FL(w)] + contour(w) + residue(w) - xmu[row]
// FL: the Fermi-weighted Lorentzian over the real axis (fermi_lorentz below),
// residue: -2 i T sum over poles z_p of (xmu_p - xmu0) xloss / ((z_p - w)^2 +
// xloss^2) (negated unless ispec == 2), contour: the Fermi-weighted Lorentzian
// integral of xmu - xmu0 along the horizontal grid, refined to 10000 linear
// samples within +-min(10, (E_F - E_0)/T) T of the Fermi level.

double fermi_fn(double e, double t, double ef) {  // ff2x.rs:5029-5042
  if (t > 0.0) {
    const double x = (e - ef) / t;
    return x < 100.0 ? 1.0 / (std::exp(x) + 1.0) : 0.0;
  }
  return e > ef ? 1.0 : 0.0;
}

double cauchy_real(double e, double w, double xloss) { return (xloss / kPi) / ((e - w) * (e - w) + xloss * xloss); }

cd cauchy(cd z, double w, double xloss) {
  const cd d = z - cd(w, 0.0);
  return (xloss / kPi) / (d * d + cd(xloss * xloss, 0.0));
}

// 1-based insertion index of x0 in the ascending grid (len + 1 past the end).
size_t search1(double x0, const std::vector<double>& x) {
  if (x0 >= x.back()) return x.size() + 1;
  if (x0 <= x.front()) return 1;
  return size_t(std::lower_bound(x.begin(), x.end(), x0) - x.begin()) + 1;
}

bool interp1(double x0, const std::vector<double>& x, const cd* y, cd& out) {
  const size_t n = x.size();
  if (x.front() < x0 && x0 < x.back()) {
    const size_t hi = search1(x0, x) - 1, lo = hi - 1;
    if (x[hi] == x[lo]) return false;
    out = (y[hi] - y[lo]) * ((x0 - x[lo]) / (x[hi] - x[lo])) + y[lo];
    return true;
  }
  if (x.front() == x0) {
    out = y[0];
    return true;
  }
  if (std::fabs(x.back() - x0) < 1.0e-10) {
    out = y[n - 1];
    return true;
  }
  return false;
}

// Integral over the real axis of f(E) * Lorentzian(E - w): 20000-point
// rectangles on [-1, 0] and [0, 1] plus the tails mapped by E = 1/u.
double fermi_lorentz(double w, double t, double ef, double xloss) {
  constexpr int kCount = 20000;
  constexpr double kMax = 1.0, dw = kMax / (kCount - 1.0);
  double sum = 0.0;
  for (int i = 0; i < kCount - 1; ++i) {
    const double z = 1.0 / (-kMax + i * dw);
    if ((z - ef) / t < 100.0) sum += fermi_fn(z, t, ef) * cauchy_real(z, w, xloss) * (z * z);
  }
  for (int i = 0; i < kCount - 1; ++i) {
    const double neg = -kMax + i * dw, pos = i * dw;
    sum += fermi_fn(neg, t, ef) * cauchy_real(neg, w, xloss);
    sum += fermi_fn(pos, t, ef) * cauchy_real(pos, w, xloss);
  }
  for (int idx = kCount; idx >= 2; --idx) {
    const double z = 1.0 / (kMax - (kCount - idx) * dw);
    if ((z - ef) / t < 100.0) sum += fermi_fn(z, t, ef) * cauchy_real(z, w, xloss) * (z * z);
  }
  return sum * dw;
}

// The contour part: the horizontal grid with its Fermi window resampled,
// trapezoids inside the window, the exact linear-segment Lorentzian integral
// outside it.
int thermal_contour(const std::vector<cd>& en, const std::vector<cd>& xmu, double ef, double t, cd xmu0, double xloss,
                    double w, int ispec, cd& out, std::string& err) {
  const double first = en.front().real(), last = en.back().real();
  double window = 10.0;
  if (ef > first) window = std::min(std::floor((ef - first) / t), 10.0);
  if (!(std::isfinite(window) && window > 0.0)) {
    err = "thermal xscorr: the Fermi window collapsed";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  constexpr int kSamples = 10000;
  const double de = 2.0 * window * t / kSamples, lo = ef - window * t, hi = ef + window * t;
  if (lo < first || hi > last) {
    err = "thermal xscorr: the Fermi window lies outside the horizontal grid";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  std::vector<double> re(en.size());
  for (size_t i = 0; i < en.size(); ++i) re[i] = en[i].real();
  const size_t s_lo = search1(lo, re), s_hi = search1(hi, re);
  const size_t i_lo = std::max<size_t>(s_lo > 0 ? s_lo - 1 : 0, 1), i_hi = std::min(s_hi, en.size());
  std::vector<cd> ze, zv;
  ze.reserve(i_lo + kSamples + en.size());
  zv.reserve(ze.capacity());
  for (size_t i = 0; i < i_lo; ++i) {
    ze.push_back(en[i]);
    zv.push_back(xmu[i]);
  }
  cd v;
  for (int i = 0; i < kSamples; ++i) {
    const double x = lo + i * de;
    if (!interp1(x, re, xmu.data(), v)) {
      err = "thermal xscorr: interpolation outside the horizontal grid";
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    }
    ze.push_back(cd(x, en[0].imag()));
    zv.push_back(v);
  }
  if (!interp1(hi, re, xmu.data(), v)) {
    err = "thermal xscorr: interpolation outside the horizontal grid";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  ze.push_back(cd(hi, en[0].imag()));
  zv.push_back(v);
  for (size_t i = i_hi; i < en.size(); ++i) {
    ze.push_back(en[i]);
    zv.push_back(xmu[i]);
  }
  const cd e1(w, xloss), e2(w, -xloss), two_pi_i(0.0, 2.0 * kPi);
  cd sum(0.0, 0.0);
  for (size_t q = 0; q + 1 < ze.size(); ++q) {
    const cd z1 = ze[q], z2 = ze[q + 1], k1 = zv[q] - xmu0, k2 = zv[q + 1] - xmu0, dz = z2 - z1;
    double f1 = fermi_fn(z1.real(), t, ef), f2 = fermi_fn(z2.real(), t, ef);
    if (ispec != 2) {
      f1 = 1.0 - f1;
      f2 = 1.0 - f2;
    }
    if (std::abs(dz) == 0.0) {
      err = "thermal xscorr: the resampled contour repeats a point";
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    }
    if (z1.real() > lo && z1.real() < hi) {
      sum += 0.5 * dz * (k1 * f1 * cauchy(z1, w, xloss) + k2 * f2 * cauchy(z2, w, xloss));
    } else {
      cd seg(0.0, 0.0);
      if (std::abs(z1 - e1) > kEps4 && std::abs(z2 - e1) > kEps4)
        seg = -std::log((z2 - e1) / (z1 - e1)) * (k1 * f1 * (z2 - e1) + k2 * f2 * (e1 - z1));
      seg += std::log((z2 - e2) / (z1 - e2)) * (k1 * f1 * (z2 - e2) + k2 * f2 * (e2 - z1));
      sum -= seg / dz / two_pi_i;
    }
  }
  out = sum;
  return finite(out) ? REFEFF_FMS_OK : REFEFF_FMS_ERR_NONFINITE_INPUT;
}

int thermal_xscorr(int ispec, const cd* energy, size_t ne, size_t ne1, const cd* xsec, const double* bg,
                   const cd* chia, double vrcorr, double temp_ev, std::vector<cd>& cchi, std::string& err) {
  constexpr size_t kAux = 10;
  if (ne1 < 2) {
    err = "thermal xscorr needs at least two horizontal points";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  const size_t pole_start = 2 * ne1 + kAux;
  if (ne < pole_start + 1) {
    err = "thermal xscorr needs 2 ne1 + 11 xsect.dat rows";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  if (!(std::isfinite(temp_ev) && temp_ev > 0.0) || !std::isfinite(vrcorr)) {
    err = "thermal xscorr needs a positive finite temperature and a finite real correction";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  std::vector<cd> xmu(ne);
  for (size_t r = 0; r < ne; ++r) {
    if (!finite(energy[r]) || !finite(xsec[r]) || !std::isfinite(bg[r]) || !finite(chia[r])) {
      err = "thermal xscorr input row " + std::to_string(r) + " is not finite";
      return REFEFF_FMS_ERR_NONFINITE_INPUT;
    }
    xmu[r] = xsec[r] + chia[r] * bg[r];
  }
  const double xloss = energy[ne1].imag();
  if (!(xloss > 0.0)) {
    err = "thermal xscorr needs a positive loss width (Im of the first loss row)";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  const bool shifted = std::fabs(vrcorr) > kEps4;
  double ef = energy[ne - 1].real();
  if (shifted) ef -= vrcorr;
  const double t = temp_ev / kHartreeEv;
  const std::vector<cd> hor_e(energy, energy + ne1), hor_x(xmu.begin(), xmu.begin() + ne1);
  cchi.assign(ne1, cd(0.0, 0.0));
  for (size_t r = 0; r < ne1; ++r) {
    const double w = energy[r].real();
    const cd xmu0 = xmu[ne1 + r];
    cd conv = xmu0 * fermi_lorentz(w, t, ef, xloss);
    if (ispec != 2) conv = xmu0 - conv;
    cd res(0.0, 0.0);
    for (size_t p = pole_start; p < ne - 1; ++p) {
      cd z = energy[p];
      if (shifted) z -= cd(vrcorr, 0.0);
      const cd d = z - cd(w, 0.0);
      res += (xmu[p] - xmu0) * xloss / (d * d + cd(xloss * xloss, 0.0));
    }
    res *= cd(0.0, -2.0 * t);
    if (ispec != 2) res = -res;
    cd contour;
    const int rc = thermal_contour(hor_e, hor_x, ef, t, xmu0, xloss, w, ispec, contour, err);
    if (rc) return rc;
    cchi[r] = conv + contour + res - hor_x[r];
    if (!finite(cchi[r])) {
      err = "thermal xscorr row " + std::to_string(r) + " is not finite";
      return REFEFF_FMS_ERR_NONFINITE_INPUT;
    }
  }
  return REFEFF_FMS_OK;
}

// ff2x_xscorr (ff2x.rs:4437-4641): the thermal form above zero temperature.
int xscorr_at(int ispec, const cd* energy, size_t ne, size_t ne1, size_t fermi, const cd* xsec, const double* bg,
              const cd* chia, double vrcorr, double temp_ev, std::vector<cd>& cchi, std::string& err) {
  if (!(std::isfinite(temp_ev) && temp_ev >= 0.0)) {
    err = "xscorr electronic temperature must be finite and non-negative";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  if (temp_ev > 0.0) return thermal_xscorr(ispec, energy, ne, ne1, xsec, bg, chia, vrcorr, temp_ev, cchi, err);
  return xscorr(ispec, energy, ne, ne1, fermi, xsec, bg, chia, vrcorr, cchi, err);
}

}  // namespace

extern "C" int refeff_ff2x_xscorr(int ne, int ne1, int fermi_index, int ispec, const refeff_complex128* energy,
                                  const refeff_complex128* cross_section, const double* background,
                                  const refeff_complex128* path_chi, double real_correction,
                                  double electronic_temperature_ev, refeff_complex128* cchi_out) {
  if (ne <= 0 || ne1 <= 0 || ne1 > ne || fermi_index < 0 || fermi_index >= ne1 || !energy || !cross_section ||
      !background || !path_chi || !cchi_out)
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  const size_t n = size_t(ne);
  std::vector<cd> e(n), xsec(n), chia(n), out;
  for (size_t r = 0; r < n; ++r) {
    e[r] = cd(energy[r].re, energy[r].im);
    xsec[r] = cd(cross_section[r].re, cross_section[r].im);
    chia[r] = cd(path_chi[r].re, path_chi[r].im);
  }
  std::string err;
  const int rc = xscorr_at(ispec, e.data(), n, size_t(ne1), size_t(fermi_index), xsec.data(), background, chia.data(),
                           real_correction, electronic_temperature_ev, out, err);
  if (rc) return rc;
  for (int r = 0; r < ne1; ++r) cchi_out[r] = {out[size_t(r)].real(), out[size_t(r)].imag()};
  return REFEFF_FMS_OK;
}

extern "C" int refeff_ff2x_lorentz_convolve(int n, const double* omega, const refeff_complex128* spectrum, double width,
                                            refeff_complex128* out) {
  if (n < 0 || (n > 0 && (!omega || !spectrum || !out))) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  std::vector<cd> y(static_cast<size_t>(n)), r;
  for (int i = 0; i < n; ++i) y[size_t(i)] = cd(spectrum[i].re, spectrum[i].im);
  if (!lorentz_conv(omega, y.data(), size_t(n), width, r)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < n; ++i) out[i] = {r[size_t(i)].real(), r[size_t(i)].imag()};
  return REFEFF_FMS_OK;
}

extern "C" int refeff_ff2x_xanes_mu_thermal(int ne, int ne1, int fermi_index, int ispec, int absolu,
                                            int include_atomic, const refeff_complex128* energy, const double* omega,
                                            const refeff_complex128* cross_section, const double* background,
                                            const refeff_complex128* trace, double s02, double real_correction,
                                            double imaginary_correction, double fermi_photon_energy,
                                            double electronic_temperature_ev, double* mu, double* mu0, double* chi) {
  const int is = ispec < 0 ? -ispec : ispec;  // ff2x_xmu_effective_ispec (ff2x.rs:1496-1502)
  if (ne <= 0 || ne1 <= 0 || ne1 >= ne || fermi_index < 0 || fermi_index >= ne1 || is < 1 || is > 2 || !energy ||
      !omega || !cross_section || !background || !trace || !std::isfinite(s02))
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  const size_t n = size_t(ne), n1 = size_t(ne1);
  std::vector<cd> e(n), xsec(n), chia(n), zero(n, cd(0.0, 0.0));
  for (size_t r = 0; r < n; ++r) {
    e[r] = cd(energy[r].re, energy[r].im);
    xsec[r] = include_atomic ? cd(cross_section[r].re, cross_section[r].im) : cd(0.0, 0.0);
    chia[r] = cd(trace[r].re, trace[r].im) * s02;
  }
  std::vector<cd> total_corr, atomic_corr;
  std::string err;
  int rc = xscorr_at(is, e.data(), n, n1, size_t(fermi_index), xsec.data(), background, chia.data(),
                     real_correction, electronic_temperature_ev, total_corr, err);
  if (rc) return rc;
  rc = xscorr_at(is, e.data(), n, n1, size_t(fermi_index), xsec.data(), background, zero.data(), real_correction,
                 electronic_temperature_ev, atomic_corr, err);
  if (rc) return rc;
  double norm = 1.0;
  if (absolu != 1) {
    const double at = is == 2 ? fermi_photon_energy : fermi_photon_energy + 50.0 / kHartreeEv;
    if (!terp(omega, background, n1, 1, at, norm) || !std::isfinite(norm) || norm == 0.0)
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  for (size_t r = 0; r < n1; ++r)
    if (!finite(total_corr[r]) || !finite(atomic_corr[r])) return REFEFF_FMS_ERR_NONFINITE_INPUT;
  std::vector<double> total(n1), atomic(n1);
  for (size_t r = 0; r < n1; ++r) {
    total[r] = (xsec[r] + chia[r] * background[r] + total_corr[r]).imag();
    atomic[r] = include_atomic ? (xsec[r] + atomic_corr[r]).imag() : 0.0;
  }
  // vicorr broadening of (total, atomic) over the photon energies (FMS-only spectra, ff2x.rs:3265-3306)
  if (imaginary_correction > kEps4) {
    std::vector<cd> spec(n1), conv;
    for (size_t r = 0; r < n1; ++r) spec[r] = cd(total[r], atomic[r]);
    if (!lorentz_conv(omega, spec.data(), n1, imaginary_correction, conv)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    for (size_t r = 0; r < n1; ++r) {
      total[r] = conv[r].real();
      atomic[r] = conv[r].imag();
    }
  }
  for (size_t r = 0; r < n1; ++r) {
    const double m0 = atomic[r] / norm, c = (total[r] - atomic[r]) / norm;
    if (mu0) mu0[r] = m0;
    if (chi) chi[r] = c;
    if (mu) mu[r] = m0 + c;
  }
  return REFEFF_FMS_OK;
}

extern "C" int refeff_ff2x_xanes_mu(int ne, int ne1, int fermi_index, int ispec, int absolu, int include_atomic,
                                    const refeff_complex128* energy, const double* omega,
                                    const refeff_complex128* cross_section, const double* background,
                                    const refeff_complex128* trace, double s02, double real_correction,
                                    double imaginary_correction, double fermi_photon_energy, double* mu, double* mu0,
                                    double* chi) {
  return refeff_ff2x_xanes_mu_thermal(ne, ne1, fermi_index, ispec, absolu, include_atomic, energy, omega,
                                      cross_section, background, trace, s02, real_correction, imaginary_correction,
                                      fermi_photon_energy, 0.0, mu, mu0, chi);
}

// ff2x.rs:3388-3397: with sig_gk > 1e-4 the fine structure of every output row
// is damped by exp(-(sig_gk k)^2), k the row's wave number in 1/Angstrom, and
// mu = mu0 + chi is formed again (the xmu.dat normalisation branch).
extern "C" int refeff_ff2x_debye_factor(int n, const double* wave_number, double sig_gk, const double* mu0, double* chi,
                                        double* mu) {
  if (n < 0 || (n > 0 && (!wave_number || !chi)) || !std::isfinite(sig_gk)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  for (int r = 0; r < n; ++r) {
    if (sig_gk > kEps4) {
      const double x = sig_gk * wave_number[r];
      chi[r] *= std::exp(-(x * x));
    }
    if (mu && mu0) mu[r] = mu0[r] + chi[r];
  }
  return REFEFF_FMS_OK;
}

// ---------------------------------------------------------------------------
// xsect.dat: XSPH's cross-section table and FEFF's rdxbin handoff to FF2X
// ---------------------------------------------------------------------------
// The text format (crates/refeff-io/src/xsect_dat.rs): title records up to a
// dashed rdhead separator (characters 4-11 all '-'), a method record (s02,
// erelax, wp, edge, emu; edge and emu in Hartree), a gamach record (the core-hole
// width in eV, ne1, ik0), a label naming em, xsnorm and xsec, and one row per
// energy (Re em, Im em in eV, xsnorm, Re xsec, Im xsec).  A leading '#' of any
// record is skipped, blank lines are ignored, and a record may carry trailing
// words after its numbers.
namespace {

std::string g_xsect_error;

int xsect_fail(int code, const std::string& msg) {
  g_xsect_error = msg;
  return code;
}

// Rust str::lines: split on '\n', one trailing '\r' dropped per line
std::vector<std::string> text_lines(const std::string& text) {
  std::vector<std::string> out;
  size_t start = 0;
  while (start < text.size()) {
    size_t end = text.find('\n', start);
    if (end == std::string::npos) end = text.size();
    std::string line = text.substr(start, end - start);
    if (!line.empty() && line.back() == '\r') line.pop_back();
    out.push_back(line);
    start = end + 1;
  }
  return out;
}

bool is_blank(const std::string& s) {
  for (char ch : s)
    if (!std::isspace(static_cast<unsigned char>(ch))) return false;
  return true;
}

// the record without a leading '#' (and the blanks around it)
std::string record_body(const std::string& line) {
  size_t i = 0;
  while (i < line.size() && std::isspace(static_cast<unsigned char>(line[i]))) ++i;
  if (i < line.size() && line[i] == '#') {
    ++i;
    while (i < line.size() && std::isspace(static_cast<unsigned char>(line[i]))) ++i;
  }
  return line.substr(i);
}

std::vector<std::string> record_tokens(const std::string& line) {
  std::vector<std::string> out;
  const std::string body = record_body(line);
  size_t i = 0;
  while (i < body.size()) {
    while (i < body.size() && std::isspace(static_cast<unsigned char>(body[i]))) ++i;
    size_t j = i;
    while (j < body.size() && !std::isspace(static_cast<unsigned char>(body[j]))) ++j;
    if (j > i) out.push_back(body.substr(i, j - i));
    i = j;
  }
  return out;
}

// A decimal float token as Rust's f64 parser takes it: [+-] digits [. digits] [(e|E) [+-] digits], at least
// one digit in the mantissa, or inf / infinity / nan in any case.
bool parse_real_token(const std::string& t, double& v) {
  size_t i = 0, n = t.size();
  if (i < n && (t[i] == '+' || t[i] == '-')) ++i;
  std::string rest = t.substr(i);
  std::string low;
  for (char ch : rest) low.push_back(char(std::tolower(static_cast<unsigned char>(ch))));
  if (low == "inf" || low == "infinity" || low == "nan") {
    v = low == "nan" ? std::nan("") : (t[0] == '-' ? -HUGE_VAL : HUGE_VAL);
    return true;
  }
  size_t digits = 0;
  while (i < n && std::isdigit(static_cast<unsigned char>(t[i]))) ++i, ++digits;
  if (i < n && t[i] == '.') {
    ++i;
    while (i < n && std::isdigit(static_cast<unsigned char>(t[i]))) ++i, ++digits;
  }
  if (digits == 0) return false;
  if (i < n && (t[i] == 'e' || t[i] == 'E')) {
    ++i;
    if (i < n && (t[i] == '+' || t[i] == '-')) ++i;
    size_t ed = 0;
    while (i < n && std::isdigit(static_cast<unsigned char>(t[i]))) ++i, ++ed;
    if (ed == 0) return false;
  }
  if (i != n) return false;
  v = std::strtod(t.c_str(), nullptr);
  return true;
}

// An unsigned integer token as Rust's usize parser takes it: [+] digits.
bool parse_count_token(const std::string& t, long long& v) {
  size_t i = t.size() > 0 && t[0] == '+' ? 1 : 0;
  if (i == t.size()) return false;
  long long x = 0;
  for (; i < t.size(); ++i) {
    if (!std::isdigit(static_cast<unsigned char>(t[i]))) return false;
    if (x > (1LL << 50)) return false;
    x = 10 * x + (t[i] - '0');
  }
  v = x;
  return true;
}

bool is_rdhead_separator(const std::string& line) {
  if (line.size() < 11) return false;
  for (size_t k = 3; k < 11; ++k)
    if (line[k] != '-') return false;
  return true;
}

struct XsectDat {
  int titles = 0;
  double s02 = 0, erelax = 0, wp = 0, edge = 0, emu = 0, gamach_ev = 0;
  long long ne1 = 0, ik0 = 0;
  std::vector<cd> em;
  std::vector<double> xsnorm;
  std::vector<cd> xsec;
};

// parse_xsect_dat, crates/refeff-io/src/xsect_dat.rs:394-429 (the record reader 620-760)
int parse_xsect_dat(const std::string& text, XsectDat& d) {
  const std::vector<std::string> lines = text_lines(text);
  size_t i = 0;
  bool separator = false;
  for (; i < lines.size(); ++i) {
    if (is_rdhead_separator(lines[i])) {
      separator = true;
      ++i;
      break;
    }
    if (!is_blank(lines[i])) ++d.titles;
  }
  if (!separator) return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, "xsect.dat: missing the rdhead separator");
  auto next_record = [&](const char* field, size_t& line_no) -> const std::string* {
    for (; i < lines.size(); ++i)
      if (!is_blank(lines[i])) {
        line_no = i + 1;
        return &lines[i++];
      }
    g_xsect_error = std::string("xsect.dat: missing the ") + field + " record";
    return nullptr;
  };
  auto reals = [&](const std::string& line, size_t line_no, const char* field, int count, double* out) -> int {
    const std::vector<std::string> tok = record_tokens(line);
    if (int(tok.size()) < count)
      return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, "xsect.dat line " + std::to_string(line_no) + ": " + field +
                                                             " record has " + std::to_string(tok.size()) +
                                                             " fields, " + std::to_string(count) + " expected");
    for (int k = 0; k < count; ++k)
      if (!parse_real_token(tok[size_t(k)], out[k]))
        return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, "xsect.dat line " + std::to_string(line_no) + ": " +
                                                               field + " field '" + tok[size_t(k)] + "' is not a number");
    return REFEFF_FMS_OK;
  };
  size_t ln = 0;
  const std::string* method = next_record("method", ln);
  if (!method) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  double mv[5];
  if (int rc = reals(*method, ln, "method", 5, mv)) return rc;
  d.s02 = mv[0], d.erelax = mv[1], d.wp = mv[2], d.edge = mv[3], d.emu = mv[4];
  const std::string* gam = next_record("gamach", ln);
  if (!gam) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  {
    const std::vector<std::string> tok = record_tokens(*gam);
    if (tok.size() < 3)
      return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT,
                        "xsect.dat line " + std::to_string(ln) + ": gamach record has " + std::to_string(tok.size()) +
                            " fields, 3 expected");
    if (!parse_real_token(tok[0], d.gamach_ev) || !parse_count_token(tok[1], d.ne1) ||
        !parse_count_token(tok[2], d.ik0))
      return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT,
                        "xsect.dat line " + std::to_string(ln) + ": gamach record is not 'gamach ne1 ik0'");
  }
  const std::string* label = next_record("label", ln);
  if (!label) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  {
    std::string low = record_body(*label);
    for (char& ch : low) ch = char(std::tolower(static_cast<unsigned char>(ch)));
    if (low.find("em") == std::string::npos || low.find("xsnorm") == std::string::npos ||
        low.find("xsec") == std::string::npos)
      return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, "xsect.dat line " + std::to_string(ln) + ": unexpected label");
  }
  for (; i < lines.size(); ++i) {
    if (is_blank(lines[i])) continue;
    double row[5];
    if (int rc = reals(lines[i], i + 1, "row", 5, row)) return rc;
    d.em.emplace_back(row[0], row[1]);
    d.xsnorm.push_back(row[2]);
    d.xsec.emplace_back(row[3], row[4]);
  }
  // validate_xsect_dat (xsect_dat.rs:443-491): rows, ne1 in 1..=rows, ne1 and ik0 within FEFF's i7 fields,
  // every value finite
  const long long rows = (long long)d.em.size();
  if (rows == 0) return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, "xsect.dat: at least one energy row is required");
  if (d.ne1 < 1 || d.ne1 > rows)
    return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, "xsect.dat: ne1 " + std::to_string(d.ne1) + " must be in 1.." +
                                                           std::to_string(rows));
  if (d.ne1 > 9999999 || d.ik0 > 9999999)
    return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, "xsect.dat: ne1 or ik0 does not fit FEFF's i7 field");
  const double sc[6] = {d.s02, d.erelax, d.wp, d.edge, d.emu, d.gamach_ev};
  for (double v : sc)
    if (!std::isfinite(v)) return xsect_fail(REFEFF_FMS_ERR_NONFINITE_INPUT, "xsect.dat: a scalar is not finite");
  for (long long r = 0; r < rows; ++r)
    if (!std::isfinite(d.em[size_t(r)].real()) || !std::isfinite(d.em[size_t(r)].imag()) ||
        !std::isfinite(d.xsnorm[size_t(r)]) || !std::isfinite(d.xsec[size_t(r)].real()) ||
        !std::isfinite(d.xsec[size_t(r)].imag()))
      return xsect_fail(REFEFF_FMS_ERR_NONFINITE_INPUT, "xsect.dat: row " + std::to_string(r + 1) + " is not finite");
  return REFEFF_FMS_OK;
}

}  // namespace

extern "C" const char* refeff_ff2x_xsect_last_error(void) { return g_xsect_error.c_str(); }

// xsect_dat_ff2x_handoff, crates/refeff-io/src/xsect_dat.rs:268-309
extern "C" int refeff_ff2x_read_xsect_dat(const char* path, double current_s02, int mbconv, int capacity,
                                          int32_t* counts_out, double* scalars_out, refeff_complex128* energy_out,
                                          double* omega_out, double* wave_number_out, double* background_out,
                                          refeff_complex128* cross_section_out) {
  g_xsect_error.clear();
  if (!path || !counts_out || capacity < 0) return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, "null path or counts");
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
  std::string text;
  char buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
  std::fclose(f);
  XsectDat d;
  if (int rc = parse_xsect_dat(text, d)) return rc;
  if (!std::isfinite(current_s02)) return xsect_fail(REFEFF_FMS_ERR_NONFINITE_INPUT, "s02 must be finite");
  if (d.ik0 < 1 || d.ik0 > d.ne1)
    return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, "xsect.dat: Fermi index " + std::to_string(d.ik0) +
                                                           " must be in 1.." + std::to_string(d.ne1));
  const int rows = int(d.em.size());
  counts_out[0] = rows;
  counts_out[1] = int32_t(d.ne1);
  counts_out[2] = int32_t(d.ik0 - 1);
  counts_out[3] = d.titles;
  if (capacity == 0) return REFEFF_FMS_OK;
  if (capacity < rows || !scalars_out || !energy_out || !omega_out || !wave_number_out || !background_out ||
      !cross_section_out)
    return xsect_fail(REFEFF_FMS_ERR_INVALID_ARGUMENT, "capacity below the row count, or a null output");
  // FEFF takes the file's S02 when mbconv > 0 or the current S02 is at most 0.1
  scalars_out[0] = (mbconv > 0 || current_s02 <= 0.1) ? d.s02 : current_s02;
  scalars_out[1] = d.s02;
  scalars_out[2] = d.erelax;
  scalars_out[3] = d.wp;
  scalars_out[4] = d.edge;
  scalars_out[5] = d.emu;
  scalars_out[6] = d.gamach_ev / kHartreeEv;
  for (int r = 0; r < rows; ++r) {
    const cd e = d.em[size_t(r)] / kHartreeEv;
    energy_out[r].re = e.real();
    energy_out[r].im = e.imag();
    omega_out[r] = e.real() - d.edge + d.emu;
    const double x = e.real() - d.edge;  // signed wave number (crates/refeff-core/src/grid/radial.rs:7-10)
    const double mag = std::sqrt(std::fabs(2.0 * x));
    wave_number_out[r] = x < 0.0 ? -mag : mag;
    background_out[r] = d.xsnorm[size_t(r)];
    cross_section_out[r].re = d.xsec[size_t(r)].real();
    cross_section_out[r].im = d.xsec[size_t(r)].imag();
  }
  return REFEFF_FMS_OK;
}
