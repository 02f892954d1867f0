// Complex arithmetic for the FMS kernels, templated on the real type.
// Plain (naive) formulas, matching the num-complex semantics the reference
// uses (no Annex-G special cases); the kernels never rely on inf/NaN rules.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace rfx {

template <typename R> struct cplx_t;
template <> struct cplx_t<double> { using type = double2; };
template <> struct cplx_t<float> { using type = float2; };
template <typename R> using cplx = typename cplx_t<R>::type;

template <typename R> __host__ __device__ __forceinline__ cplx<R> mk(R re, R im) { cplx<R> z; z.x = re; z.y = im; return z; }
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __host__ __device__ __forceinline__ C cneg(C a) { a.x = -a.x; a.y = -a.y; return a; }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename C, typename R> __host__ __device__ __forceinline__ C cscale(C a, R s) { a.x *= s; a.y *= s; return a; }
// acc += a*b with fused multiply-adds (the device path is allowed to contract).
template <typename C> __device__ __forceinline__ void cfma(C& acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
}
// acc -= a*b
template <typename C> __device__ __forceinline__ void cfms(C& acc, C a, C b) {
  acc.x = fma(-a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(-a.x, b.y, acc.y); acc.y = fma(-a.y, b.x, acc.y);
}
template <typename C> __host__ __device__ __forceinline__ C cdiv(C a, C b) {
  auto n = b.x * b.x + b.y * b.y;
  C r; r.x = (a.x * b.x + a.y * b.y) / n; r.y = (a.y * b.x - a.x * b.y) / n; return r;
}
template <typename C> __host__ __device__ __forceinline__ auto cabs1(C a) -> decltype(a.x) {
  return fabs(a.x) + fabs(a.y);
}
template <typename C> __host__ __device__ __forceinline__ bool cfinite(C a) { return isfinite(a.x) && isfinite(a.y); }

__device__ __forceinline__ double2 cexp(double2 a) {
  double s, c; sincos(a.y, &s, &c); double r = exp(a.x); return make_double2(r * c, r * s);
}
__device__ __forceinline__ float2 cexp(float2 a) {
  float s, c; sincosf(a.y, &s, &c); float r = expf(a.x); return make_float2(r * c, r * s);
}

template <typename Dst, typename Src> __device__ __forceinline__ Dst ccast(Src s) { Dst d; d.x = s.x; d.y = s.y; return d; }

// Complex double -> (hi.re, hi.im, lo.re, lo.im) with hi = fl32(v), lo = fl32(v - hi):
// hi + lo carries v to about 2^-48 relative.
__device__ __forceinline__ float4 split_hi_lo(double2 v) {
  const float hr = float(v.x), hi = float(v.y);
  return make_float4(hr, hi, float(v.x - double(hr)), float(v.y - double(hi)));
}
__device__ __forceinline__ double2 join_hi_lo(float4 s) {
  return make_double2(double(s.x) + double(s.z), double(s.y) + double(s.w));
}

// ---- double-float (FP32 pair) arithmetic on the FP32 pipes ----
// Error-free transforms after Dekker / Knuth: two_prod via FMA, two_sum.
struct df { float hi, lo; };
__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// acc += (ah + al) * (xh + xl), dropping al*xl (below 2^-48 relative); the
// result is renormalised (|lo| <= ulp(hi)/2) so that every step adds an error
// of about 2^-48 |acc| only.
__device__ __forceinline__ void df_mac(df& acc, float ah, float al, float xh, float xl) {
  const float p = __fmul_rn(ah, xh);  // rounded product: must not be fused into the sums below
  float e = fmaf(ah, xh, -p);
  e = fmaf(ah, xl, e);
  e = fmaf(al, xh, e);
  float s, t;
  df_two_sum(acc.hi, p, s, t);
  t += acc.lo + e;
  acc.hi = s + t;
  acc.lo = t - (acc.hi - s);
}
// Compensated dot product step (Ogita, Rump and Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26 (2005), Dot2): s carries the rounded sum
// of the products ah*xh, c the sum of their exact rounding errors (two_prod
// and two_sum) plus the cross terms ah*xl + al*xh, in plain FP32.  s + c is as
// accurate as the sum computed in twice the working precision; 12 FP32
// operations per product against 15 for a renormalised double-float step.
__device__ __forceinline__ void dot2_mac(df& acc, float ah, float al, float xh, float xl) {
  const float p = __fmul_rn(ah, xh);  // rounded product: must not be fused into the sums below
  float e = fmaf(ah, xh, -p);
  e = fmaf(ah, xl, e);
  e = fmaf(al, xh, e);
  float s, q;
  df_two_sum(acc.hi, p, s, q);
  acc.hi = s;
  acc.lo += q + e;
}
__device__ __forceinline__ void df_renorm(df& a) {
  const float s = a.hi + a.lo;
  a.lo = a.lo - (s - a.hi);
  a.hi = s;
}

}  // namespace rfx
