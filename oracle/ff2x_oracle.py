"""TEST INFRASTRUCTURE ONLY: CPU restatement of the FF2X XANES step that turns the MKGTR trace into mu(E).

Used by tests and by bench.py's mu(E) error figure as the checker of the product's
refeff_ff2x_xanes_mu; never shipped or called by the product.

  lorenz, astep                  crates/refeff-engine/src/ff2x.rs:5052-5076
                                 (crates/refeff-core/src/xscorr.rs:39-73 for the core ports and their known answers)
  xscorr, zero temperature       crates/refeff-engine/src/ff2x.rs:4437-4641
  xscorr, thermal                crates/refeff-engine/src/ff2x.rs:4643-5050 (thermal_xscorr below)
  corrected components           crates/refeff-engine/src/ff2x.rs:3186-3262
  xmu.dat normalisation / rows   crates/refeff-engine/src/ff2x.rs:3309-3399
  locat / terp window / polint   crates/refeff-core/src/interpolation.rs:119-135, 338-446
  vicorr broadening: conv1, conv crates/refeff-engine/src/ff2x.rs:3265-3306,
                                 crates/refeff-core/src/convolution/lorentzian.rs:4-100

Known answers pinned in tests/test_ff2x.py: the three lorenz and three astep values of
crates/refeff-core/src/xscorr.rs:121-157 and the constant-cross-section xscorr case of
crates/refeff-engine/src/ff2x/tests.rs:1127-1149 (fixture 5167-5195), and the thermal xscorr's
constant-cross-section case at 0.5 eV of tests.rs:1152-1178 (fixture 5197-5238).  The contour integral with a
non-constant integrand has no reference known answer here: for it this restatement and the product's
C++ agree with each other (parity of that term unpinned).
"""
from __future__ import annotations

import cmath
import math

import numpy as np

EPS4 = 1.0e-4
HARTREE_EV = 27.211396


def lorenz(xloss: float, width: float, dele: float) -> complex:
    """(xloss / pi) / (xloss^2 - (w - i dele)^2 ... ) in the expanded form of ff2x.rs:5058-5065."""
    den = complex(xloss * xloss - width * width + dele * dele, -2.0 * width * dele)
    if den == 0:
        raise ZeroDivisionError("lorenz denominator is zero")
    return complex(xloss / math.pi, 0.0) / den


def astep(xloss: float, dele: float) -> float:
    return min(1.0, max(0.0, 0.5 + math.atan(dele / xloss) / math.pi))


def _locat(x, xs):
    lo, hi = 0, len(xs) + 1
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if x < xs[mid - 1]:
            hi = mid
        else:
            lo = mid
    return lo


def _polint(xs, ys, x):
    n = len(xs)
    c, d = list(ys), list(ys)
    ns = min(range(n), key=lambda i: (abs(x - xs[i]), i))
    y = ys[ns]
    for m in range(1, n):
        for i in range(n - m):
            ho, hp = xs[i] - x, xs[i + m] - x
            w = (c[i + 1] - d[i]) / (ho - hp)
            d[i], c[i] = w * hp, w * ho
        if 2 * ns < n - m:
            y += c[ns]
        else:
            y += d[ns - 1]
            ns -= 1
    return y


def terp(xs, ys, order, x):
    n = len(xs)
    first = max(_locat(x, xs) - order // 2, 1)
    first = min(first, n - order)
    return _polint(xs[first - 1:first + order], ys[first - 1:first + order], x)


def xscorr(ispec, energy, ne1, fermi, xsec, bg, chia, vrcorr=0.0):
    """cchi[0:ne1] of the zero-temperature xscorr (ff2x.rs:4437-4641)."""
    ne = len(energy)
    energy = [complex(e) for e in energy]
    xmu = [complex(xsec[r]) + complex(chia[r]) * float(bg[r]) for r in range(ne)]
    xloss = energy[0].imag
    ef = energy[-1].real
    omega = [energy[r].real for r in range(ne1)]
    scale = 1.0 + 0.0j
    shifted = abs(vrcorr) > EPS4
    if shifted:
        ef -= vrcorr
        at = terp(omega, xmu[:ne1], 1, ef)
        for r in range(ne1, ne):
            energy[r] -= vrcorr
        scale = at / xmu[fermi]
        for r in range(ne1, ne):
            xmu[r] *= scale
    ze = [energy[r] for r in range(ne1, ne) if energy[r].imag < xloss]
    zv = [xmu[r] for r in range(ne1, ne) if energy[r].imag < xloss]
    if shifted:
        ze.append(complex(ef, xloss))
        zv.append(scale * xmu[fermi])
    else:
        ze.append(energy[fermi])
        zv.append(xmu[fermi])
    rows = range(ne1) if ispec != 2 else range(ne1 - 1, -1, -1)
    for r in rows:
        past = energy[r].real - ef > EPS4 if ispec != 2 else ef - energy[r].real > EPS4
        if past:
            ze.append(energy[r])
            zv.append(xmu[r])
    out = []
    for r in range(ne1):
        w = omega[r]
        if w >= ef:
            x0 = xmu[fermi] * scale if ispec == 2 else xmu[r]
        else:
            x0 = xmu[r] if ispec == 2 else xmu[fermi] * scale
        e1, e2 = complex(w, xloss), complex(w, -xloss)
        dele = w - ef
        conv = x0 * astep(xloss, dele)
        if ispec == 2:
            conv = x0 - conv
        corr = lorenz(xloss, ze[0].imag, 0.0 if abs(dele) < EPS4 else dele) * (zv[0] - x0) * complex(0.0, ze[0].imag)
        for q in range(len(ze) - 1):
            z1, z2 = ze[q], ze[q + 1]
            f1, f2 = zv[q] - x0, zv[q + 1] - x0
            seg = 0j
            if abs(z1 - e1) > EPS4 and abs(z2 - e1) > EPS4:
                seg = cmath.log((z2 - e1) / (z1 - e1)) * (f1 * (z2 - e1) + f2 * (e1 - z1))
            seg -= cmath.log((z2 - e2) / (z1 - e2)) * (f1 * (z2 - e2) + f2 * (e2 - z1))
            corr += seg / (z2 - z1) / complex(0.0, 2.0 * math.pi)
        if ispec == 2:
            corr = -corr
        out.append(conv + corr - xmu[r])
    return out


def _fermi(e, t, ef):
    """Fermi function, zero above (e - ef) / t = 100 (ff2x.rs:5029-5042); e may be an array."""
    x = (np.asarray(e, dtype=np.float64) - ef) / t
    with np.errstate(over="ignore"):
        return np.where(x < 100.0, 1.0 / (np.exp(np.minimum(x, 100.0)) + 1.0), 0.0)


def _cauchy_real(e, w, xloss):
    return (xloss / math.pi) / ((e - w) ** 2 + xloss ** 2)


def _fermi_lorentz(w, t, ef, xloss):
    """Fermi-weighted Lorentzian over the real axis (ff2x.rs:4802-4859): rectangles on [-1, 0] and [0, 1]
    plus the two tails mapped by E = 1/u, 20000 points each."""
    n, top = 20000, 1.0
    dw = top / (n - 1.0)
    i = np.arange(n - 1, dtype=np.float64)
    z = 1.0 / (-top + i * dw)
    keep = (z - ef) / t < 100.0
    total = np.sum(np.where(keep, _fermi(z, t, ef) * _cauchy_real(z, w, xloss) * z * z, 0.0))
    neg, pos = -top + i * dw, i * dw
    total += np.sum(_fermi(neg, t, ef) * _cauchy_real(neg, w, xloss) + _fermi(pos, t, ef) * _cauchy_real(pos, w, xloss))
    idx = np.arange(n, 1, -1, dtype=np.float64)
    z = 1.0 / (top - (n - idx) * dw)
    keep = (z - ef) / t < 100.0
    total += np.sum(np.where(keep, _fermi(z, t, ef) * _cauchy_real(z, w, xloss) * z * z, 0.0))
    return float(total * dw)


def _search1(x0, x):
    """1-based insertion index (len + 1 past the end; ff2x.rs:5015-5027)."""
    if x0 >= x[-1]:
        return len(x) + 1
    if x0 <= x[0]:
        return 1
    return int(np.searchsorted(x, x0, side="left")) + 1


def _interp1(x0, x, y):
    if x[0] < x0 < x[-1]:
        hi = _search1(x0, x) - 1
        lo = hi - 1
        return (y[hi] - y[lo]) * ((x0 - x[lo]) / (x[hi] - x[lo])) + y[lo]
    if x[0] == x0:
        return y[0]
    if abs(x[-1] - x0) < 1e-10:
        return y[-1]
    raise ValueError("interpolation point outside the grid")


def _thermal_contour(en, xmu, ef, t, xmu0, xloss, w, ispec):
    """The Fermi-weighted Lorentzian integral of xmu - xmu0 along the horizontal grid, its Fermi window
    resampled at 10000 points (ff2x.rs:4861-4978)."""
    re = np.array([e.real for e in en])
    window = 10.0
    if ef > re[0]:
        window = min(math.floor((ef - re[0]) / t), 10.0)
    if not window > 0.0:
        raise ValueError("Fermi window collapsed")
    ns = 10000
    de = 2.0 * window * t / ns
    lo, hi = ef - window * t, ef + window * t
    if lo < re[0] or hi > re[-1]:
        raise ValueError("Fermi window outside the horizontal grid")
    i_lo = max(max(_search1(lo, re) - 1, 0), 1)
    i_hi = min(_search1(hi, re), len(en))
    ze = list(en[:i_lo])
    zv = list(xmu[:i_lo])
    for i in range(ns):
        x = lo + i * de
        ze.append(complex(x, en[0].imag))
        zv.append(_interp1(x, re, xmu))
    ze.append(complex(hi, en[0].imag))
    zv.append(_interp1(hi, re, xmu))
    ze += list(en[i_hi:])
    zv += list(xmu[i_hi:])
    ze, zv = np.array(ze), np.array(zv)
    z1, z2 = ze[:-1], ze[1:]
    k1, k2 = zv[:-1] - xmu0, zv[1:] - xmu0
    f1, f2 = _fermi(z1.real, t, ef), _fermi(z2.real, t, ef)
    if ispec != 2:
        f1, f2 = 1.0 - f1, 1.0 - f2
    dz = z2 - z1
    assert np.all(np.abs(dz) > 0.0)
    e1, e2 = complex(w, xloss), complex(w, -xloss)

    def cauchy(z):
        return (xloss / math.pi) / ((z - w) ** 2 + xloss * xloss)

    inside = (z1.real > lo) & (z1.real < hi)
    trap = 0.5 * dz * (k1 * f1 * cauchy(z1) + k2 * f2 * cauchy(z2))
    near = (np.abs(z1 - e1) > EPS4) & (np.abs(z2 - e1) > EPS4)
    with np.errstate(all="ignore"):
        seg = np.where(near, -np.log((z2 - e1) / (z1 - e1)) * (k1 * f1 * (z2 - e1) + k2 * f2 * (e1 - z1)), 0.0)
        seg = seg + np.log((z2 - e2) / (z1 - e2)) * (k1 * f1 * (z2 - e2) + k2 * f2 * (e2 - z1))
    exact = -seg / dz / complex(0.0, 2.0 * math.pi)
    return complex(np.sum(np.where(inside, trap, exact)))


def thermal_xscorr(ispec, energy, ne1, xsec, bg, chia, vrcorr=0.0, temperature_ev=0.5):
    """cchi[0:ne1] of the thermal xscorr (ff2x.rs:4643-4800).  Rows: ne1 horizontal, ne1 at the loss width,
    10 auxiliary, the poles, and the Fermi-level row last."""
    ne = len(energy)
    energy = np.array([complex(e) for e in energy])
    xmu = np.array([complex(xsec[r]) + complex(chia[r]) * float(bg[r]) for r in range(ne)])
    pole_start = 2 * ne1 + 10
    assert ne >= pole_start + 1 and temperature_ev > 0.0
    xloss = energy[ne1].imag
    ef = energy[-1].real
    shifted = abs(vrcorr) > EPS4
    if shifted:
        ef -= vrcorr
    t = temperature_ev / HARTREE_EV
    poles = energy[pole_start:ne - 1] - (vrcorr if shifted else 0.0)
    out = []
    for r in range(ne1):
        w = energy[r].real
        xmu0 = xmu[ne1 + r]
        conv = xmu0 * _fermi_lorentz(w, t, ef, xloss)
        if ispec != 2:
            conv = xmu0 - conv
        res = complex(np.sum((xmu[pole_start:ne - 1] - xmu0) * xloss / ((poles - w) ** 2 + xloss * xloss)))
        res *= complex(0.0, -2.0 * t)
        if ispec != 2:
            res = -res
        contour = _thermal_contour(energy[:ne1], xmu[:ne1], ef, t, xmu0, xloss, w, ispec)
        out.append(conv + contour + res - xmu[r])
    return out


PI_F32 = float(__import__("numpy").float32(math.pi))  # FEFF divides by the single-precision pi (convolution.rs:17)


def conv1(x1, x2, y1, y2, x0, width):
    """Lorentzian integral at x0 of the segment (x1, y1)-(x2, y2), per part (lorentzian.rs:4-30)."""
    t = complex((x2 - x1) / 2.0, 0.0) / complex((x1 + x2) / 2.0 - x0, -width)

    def part(slope, mid):
        if abs(t) >= 0.1:
            v = slope * 2.0 + (mid - slope / t) * cmath.log((1.0 + t) / (1.0 - t))
        else:
            v = mid * (2.0 * (t + t * t * t / 3.0)) - slope * (2.0 * t * t / 3.0)
        return complex(v).imag
    y1, y2 = complex(y1), complex(y2)
    return complex(part((y2.real - y1.real) / 2.0, (y2.real + y1.real) / 2.0),
                   part((y2.imag - y1.imag) / 2.0, (y2.imag + y1.imag) / 2.0))


def conv(omega, spectrum, width):
    """FEFF conv (lorentzian.rs:32-100): the spectrum extended past its last point, broadened at every omega."""
    n = len(omega)
    fs = omega[-1] - omega[-2]
    ew = max(fs, 50.0 * width)
    xlast = omega[-1] + ew
    ylast = complex(spectrum[-1]) + (complex(spectrum[-1]) - complex(spectrum[-2])) * (ew / fs)
    out = []
    for x0 in omega:
        s = 0j
        for i in range(n - 1):
            s += conv1(omega[i], omega[i + 1], spectrum[i], spectrum[i + 1], x0, width)
        s += conv1(omega[-1], xlast, spectrum[-1], ylast, x0, width)
        out.append(s / PI_F32)
    return out


def xanes_mu(*, energy, ne1, fermi, omega, cross_section, background, trace, s02=1.0, ispec=1, absolu=0,
             include_atomic=True, vrcorr=0.0, vicorr=0.0, fermi_photon_energy=0.0):
    """(mu, mu0, chi) over the ne1 main rows (ff2x.rs:3186-3306 and 3309-3399, sig_gk = 0)."""
    ispec = abs(ispec)
    ne = len(energy)
    xsec = [complex(v) if include_atomic else 0j for v in cross_section]
    chia = [complex(t) * s02 for t in trace]
    tot = xscorr(ispec, energy, ne1, fermi, xsec, background, chia, vrcorr)
    atm = xscorr(ispec, energy, ne1, fermi, xsec, background, [0j] * ne, vrcorr)
    norm = 1.0
    if absolu != 1:
        at = fermi_photon_energy if ispec == 2 else fermi_photon_energy + 50.0 / HARTREE_EV
        norm = terp(list(omega[:ne1]), [float(b) for b in background[:ne1]], 1, at)
    total = [(xsec[r] + chia[r] * float(background[r]) + tot[r]).imag for r in range(ne1)]
    atomic = [(xsec[r] + atm[r]).imag if include_atomic else 0.0 for r in range(ne1)]
    if vicorr > EPS4:
        c = conv(list(omega[:ne1]), [complex(a, b) for a, b in zip(total, atomic)], vicorr)
        total, atomic = [v.real for v in c], [v.imag for v in c]
    mu, mu0, chi = [], [], []
    for r in range(ne1):
        mu0.append(atomic[r] / norm)
        chi.append((total[r] - atomic[r]) / norm)
        mu.append(mu0[-1] + chi[-1])
    return mu, mu0, chi


def debye_factor(wave_number, sig_gk, mu0, chi):
    """ff2x.rs:3388-3397: chi *= exp(-(sig_gk k)^2) when sig_gk > 1e-4 (k in 1/Angstrom); mu = mu0 + chi."""
    chi = np.array(chi, float)
    if sig_gk > 1e-4:
        chi = chi * np.exp(-(sig_gk * np.asarray(wave_number, float)) ** 2)
    return np.asarray(mu0, float) + chi, chi
