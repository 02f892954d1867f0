"""CPU check of the arithmetic of the tensor-core refinement residual (refeff_gb300/csrc/tc_residual.cu).

The kernel makes r = b - A x exact on the bf16 tensor path by cutting every scaled entry of A and x into six
signed digits (weights 2^-7 .. 2^-47) and summing the digit products of each level s = i + j (2 .. 8) in FP32,
then combining the level sums in double-float.  This test restates that arithmetic in numpy float32 (each
operation rounded once, as the kernel's intrinsics are) and pins the facts the kernel relies on:

* every digit is an integer with |t| <= 128 (so a product of two digits is below 2^14 and exact in bf16);
* six digits reconstruct a value to within 2^-48;
* a level sum of one 32-column segment stays an integer below 2^24, so FP32 accumulation is exact;
* the whole residual, levels 2 .. 8 combined in double-float, against exact rational arithmetic on rows
  whose entries span six orders of magnitude and columns of x spanning four: within 2^-47 of
  ||a_row||_1 ||x_col||_inf, the normwise scale of the refinement's stopping rule (each digit cut is exact
  to 2^-48 of its power-of-two scale, shared by a row segment of A or a column of x).  Componentwise the
  error can reach about 2^-43 of sum |a||x| where a row's large entries meet a column's small ones; the
  double-float (Dot2) residual holds about 2^-47 componentwise.
"""
from fractions import Fraction

import numpy as np

F32 = np.float32
MAGIC = F32(12582912.0)  # 1.5 x 2^23
DIGITS = 6


def fma32(a, b, c):
    # a*b + c rounded once: exact in float64 here (a digit times a power of two, plus a float32)
    return (np.float64(a) * np.float64(b) + np.float64(c)).astype(F32)


def cut_digits(h, l):
    """The kernel's cut_digits on float32 arrays h, l (|h + l| < 1): list of six digit arrays."""
    rh = h.astype(F32)
    l = l.astype(F32)
    out = []
    for k in range(DIGITS):
        w = F32(2.0 ** (7 + 8 * k))
        wi = F32(2.0 ** (-7 - 8 * k))
        s = (rh + l).astype(F32)
        d = ((s * w + MAGIC).astype(F32) - MAGIC).astype(F32)
        rh = fma32(-d, wi, rh)
        out.append(d)
    return out


def split(v):
    h = v.astype(F32)
    return h, (v - h.astype(np.float64)).astype(F32)


def two_sum(a, b):
    s = F32(a + b)
    bb = F32(s - a)
    return s, F32(F32(a - F32(s - bb)) + F32(b - bb))


def test_digits_bounded_and_exact():
    rng = np.random.default_rng(5)
    v = rng.uniform(-1, 1, 200000) * 10.0 ** rng.uniform(-9, 0, 200000)
    v[::7] = np.sign(v[::7]) * (1 - 2.0 ** -rng.integers(20, 52, v[::7].size))  # just below 1
    h, l = split(v)
    keep = np.abs(h.astype(np.float64) + l.astype(np.float64)) < 1
    h, l = h[keep], l[keep]
    t = cut_digits(h, l)
    tmax = max(float(np.abs(d).max()) for d in t)
    assert tmax <= 128.0
    for d in t:
        assert np.all(d == np.round(d))  # integers
        assert np.all(d.astype(np.float32).view(np.uint32) & 0xFFFF == 0)  # exact in bf16
    rec = sum(d.astype(np.float64) * 2.0 ** (-7 - 8 * k) for k, d in enumerate(t))
    err = np.abs(h.astype(np.float64) + l.astype(np.float64) - rec)
    assert err.max() <= 2.0 ** -48 * (1 + 2.0 ** -16)  # the last digit's half unit, plus the rounding of rh + l


def test_level_sums_fit_fp32():
    # 6 digit pairs at most per level, re and im products, 32 columns, |product| <= 2^14
    assert 6 * 2 * 32 * 128 * 128 < 2 ** 24


def _scale_inv(mx):
    e = int((np.array(mx, dtype=F32).view(np.uint32) >> 23) & 0xFF)
    e = min(max(e, 1), 252)
    return F32(2.0 ** (-(e - 127) - 1))


def test_residual_against_exact_arithmetic():
    rng = np.random.default_rng(11)
    rows, n, m, seg = 3, 96, 3, 32
    A = (rng.normal(size=(rows, n)) + 1j * rng.normal(size=(rows, n))) * 10.0 ** rng.uniform(-6, 0, (rows, n))
    A[np.arange(rows), np.arange(rows)] = 1.0
    X = (rng.normal(size=(n, m)) + 1j * rng.normal(size=(n, m))) * 10.0 ** rng.uniform(-3, 1, (n, m))
    ah, al = split(A.real)
    aih, ail = split(A.imag)
    # x: a power of two per column above its largest |re|, |im|; digits of the scaled FP64 values
    xd_r, xd_i, tau = [], [], []
    for c in range(m):
        mx = max(np.abs(X[:, c].real).max(), np.abs(X[:, c].imag).max())
        ex = int(np.frexp(mx)[1])
        tau.append(2.0 ** ex)
        xd_r.append(np.stack(cut_digits(*split(X[:, c].real / 2.0 ** ex)), 1).astype(np.int64))
        xd_i.append(np.stack(cut_digits(*split(X[:, c].imag / 2.0 ** ex)), 1).astype(np.int64))
    pairs = [(i, j) for i in range(1, 7) for j in range(1, 7) if i + j <= 8]
    worst = worst_cw = 0.0
    for r in range(rows):
        for c in range(m):
            acc = {0: (F32(0), F32(0)), 1: (F32(0), F32(0))}
            for s0 in range(0, n, seg):
                ks = slice(s0, s0 + seg)
                mx = max(np.abs(ah[r, ks]).max(), np.abs(aih[r, ks]).max())
                si = _scale_inv(mx)
                sig = F32(1.0 / float(si))
                dr = np.stack(cut_digits((ah[r, ks] * si).astype(F32), (al[r, ks] * si).astype(F32)), 1).astype(np.int64)
                di = np.stack(cut_digits((aih[r, ks] * si).astype(F32), (ail[r, ks] * si).astype(F32)), 1).astype(np.int64)
                xr, xi = xd_r[c][ks], xd_i[c][ks]
                for part in (0, 1):
                    L = {s: 0 for s in range(2, 9)}
                    for i, j in pairs:
                        if part == 0:
                            L[i + j] += int(np.sum(dr[:, i - 1] * xr[:, j - 1] - di[:, i - 1] * xi[:, j - 1]))
                        else:
                            L[i + j] += int(np.sum(dr[:, i - 1] * xi[:, j - 1] + di[:, i - 1] * xr[:, j - 1]))
                    assert max(abs(v) for v in L.values()) < 2 ** 24
                    lv = {s: F32(L[s]) for s in L}
                    t = fma32(lv[7], F32(2.0 ** -40), F32(lv[8] * F32(2.0 ** -48)))
                    hh, ll = two_sum(F32(lv[6] * F32(2.0 ** -32)), t)
                    for s in (5, 4, 3, 2):
                        hh, e = two_sum(F32(lv[s] * F32(2.0 ** (-8 * (s - 2)))), hh)
                        ll = F32(ll + e)
                    sc = F32(float(sig) * 2.0 ** -14)
                    hh, ll = F32(hh * sc), F32(ll * sc)
                    a_hi, a_lo = acc[part]
                    s1, e1 = two_sum(a_hi, hh)
                    e1 = F32(F32(e1 + a_lo) + ll)
                    hi = F32(s1 + e1)
                    acc[part] = (hi, F32(e1 - F32(hi - s1)))
            got = [(float(acc[p][0]) + float(acc[p][1])) * tau[c] for p in (0, 1)]
            er = ei = den = Fraction(0)
            arow = Fraction(0)
            for k in range(n):
                a_r = Fraction(float(ah[r, k])) + Fraction(float(al[r, k]))
                a_i = Fraction(float(aih[r, k])) + Fraction(float(ail[r, k]))
                x_r, x_i = Fraction(X[k, c].real), Fraction(X[k, c].imag)
                er += a_r * x_r - a_i * x_i
                ei += a_r * x_i + a_i * x_r
                den += (abs(a_r) + abs(a_i)) * (abs(x_r) + abs(x_i))
                arow += abs(a_r) + abs(a_i)
            err = max(abs(Fraction(got[0]) - er), abs(Fraction(got[1]) - ei))
            xmax = max(abs(Fraction(X[k, c].real)) + abs(Fraction(X[k, c].imag)) for k in range(n))
            worst = max(worst, float(err / (arow * xmax)))
            worst_cw = max(worst_cw, float(err / den))
    assert worst < 2.0 ** -47, worst          # measured 2^-48.8
    assert worst_cw < 2.0 ** -42, worst_cw    # measured 2^-43.1
