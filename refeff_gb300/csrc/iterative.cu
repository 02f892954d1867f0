// Iterative FMS forms (FEFF minv != 0) on the GPU.
//
//   system W = I - T G0 (G0 entries with |G0| <= toler2 dropped), or T G0 for
//   Graves-Morris                    crates/refeff-core/src/fms/solvers.rs:10-78
//   ggbi one-step BiCGSTAB           crates/refeff-core/src/fms/internals/iterative.rs:181-254
//   ggrm two-sided Lanczos recursion iterative.rs:256-375
//   gggm Graves-Morris               iterative.rs:377-497
//   ggtf transpose-free QMR          iterative.rs:499-612
//   gg[row, col] = sum_s G0[abs + row, s] x_col[s]   iterative.rs:38-179
//
// One CTA solves one (energy, absorber column) system: the solver's scalar
// recurrences are uniform across the CTA, its vectors live in a global
// scratch slab, and the matrix-vector products stream W through the CTA with
// the input vector staged in shared memory.  R = double gives the FP64 form,
// R = float the reference-precision (Complex32) form.  Every loop is bounded
// by the reference's own restart and iteration limits.
#include <cuda_runtime.h>

#include <cstdint>

#include "cplx.cuh"
#include "fms_plan.cuh"
#include "iterative.cuh"

namespace rfx {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRowsPerThread = 4;

template <typename C> __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }
template <typename C> __device__ __forceinline__ bool czero(C a) { return a.x == 0 && a.y == 0; }

// ---------------------------------------------------------------------------
// system assembly
// ---------------------------------------------------------------------------

// The block whose columns hold global column c (the blocks' columns partition [0, m)).
__device__ __forceinline__ const SolvedBlock& block_of(const SolvedBlock* blocks, int nblocks, int c) {
  int q = 0;
  while (q + 1 < nblocks && c >= blocks[q + 1].col) ++q;
  return blocks[q];
}

// The solved blocks' rows of G0 (row r of grow is state bl.row + r - bl.col of
// its block bl), kept for gg = G0 x before W overwrites G0.
template <typename R>
__global__ void block_rows_kernel(BatchLayout lay, const double2* __restrict__ G0, const SolvedBlock* blocks,
                                  int nblocks, cplx<R>* __restrict__ grow) {
  const int e = blockIdx.y, n = lay.n, m = lay.m;
  const double2* g = G0 + size_t(e) * lay.stride;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < m * n; idx += gridDim.x * blockDim.x) {
    const int r = idx % m, s = idx / m;
    const SolvedBlock& bl = block_of(blocks, nblocks, r);
    grow[size_t(e) * m * n + idx] = ccast<cplx<R>>(g[size_t(bl.row + r - bl.col) + size_t(lay.lda) * s]);
  }
}

// W[r, c] = diag d(r, c) + f t0[r] G0[r, c] [|G0[r, c]| > tol2] + f t1[p] G0[p, c] [|G0[p, c]| > tol2],
// p the spin partner of r.  One thread writes a partner pair (r, p) of one column together, so W may
// overwrite G0 in place.
template <typename R>
__global__ void iterative_system_kernel(BatchLayout lay, const double2* __restrict__ G0, cplx<R>* __restrict__ W,
                                        const double2* __restrict__ t, const int* __restrict__ partner, double tol2,
                                        double factor, double diag) {
  const int e = blockIdx.z, n = lay.n;
  const int c = blockIdx.y;
  const double2* g = G0 + size_t(e) * lay.stride + size_t(lay.lda) * c;
  cplx<R>* w = W + size_t(e) * lay.stride + size_t(lay.lda) * c;
  const double2* te = t + size_t(e) * n * 2;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const int p = partner[r];
    if (p >= 0 && p < r) continue;  // written by the partner's thread
    const double2 gr = g[r];
    const bool kr = hypot(gr.x, gr.y) > tol2;
    double2 wr = make_double2(0.0, 0.0);
    if (kr) wr = cmul(cscale(te[2 * size_t(r)], factor), gr);
    if (p >= 0) {
      const double2 gp = g[p];
      const bool kp = hypot(gp.x, gp.y) > tol2;
      double2 wp = make_double2(0.0, 0.0);
      if (kp) {
        wr = cadd(wr, cmul(cscale(te[2 * size_t(p) + 1], factor), gp));
        wp = cmul(cscale(te[2 * size_t(p)], factor), gp);
      }
      if (kr) wp = cadd(wp, cmul(cscale(te[2 * size_t(r) + 1], factor), gr));
      if (p == c) wp.x += diag;
      w[p] = ccast<cplx<R>>(wp);
    }
    if (r == c) wr.x += diag;
    w[r] = ccast<cplx<R>>(wr);
  }
}

// ---------------------------------------------------------------------------
// CTA-wide vector primitives
// ---------------------------------------------------------------------------
template <typename R>
struct Cta {
  using C = cplx<R>;
  int n;
  C* red;  // kWarps + 1 entries
  C* vs;   // n entries (staged input vector)

  __device__ C dot(const C* a, const C* b) const {  // sum conj(a) b
    C s = mk<R>(R(0), R(0));
    for (int i = threadIdx.x; i < n; i += kThreads) cfma(s, cconj(a[i]), b[i]);
    return reduce(s);
  }
  __device__ C reduce(C s) const {
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      C t = red[0];
      for (int w = 1; w < kWarps; ++w) t = cadd(t, red[w]);
      red[kWarps] = t;
    }
    __syncthreads();
    const C out = red[kWarps];
    __syncthreads();
    return out;
  }
  // y = W v (W column-major with leading dimension lda)
  __device__ void matvec(const C* W, size_t lda, const C* v, C* y) const {
    for (int i = threadIdx.x; i < n; i += kThreads) vs[i] = v[i];
    __syncthreads();
    for (int r0 = 0; r0 < n; r0 += kThreads * kRowsPerThread) {
      C acc[kRowsPerThread];
#pragma unroll
      for (int k = 0; k < kRowsPerThread; ++k) acc[k] = mk<R>(R(0), R(0));
      for (int c = 0; c < n; ++c) {
        const C x = vs[c];
        const C* col = W + lda * size_t(c);
#pragma unroll
        for (int k = 0; k < kRowsPerThread; ++k) {
          const int r = r0 + k * kThreads + threadIdx.x;
          if (r < n) cfma(acc[k], col[r], x);
        }
      }
#pragma unroll
      for (int k = 0; k < kRowsPerThread; ++k) {
        const int r = r0 + k * kThreads + threadIdx.x;
        if (r < n) y[r] = acc[k];
      }
    }
    __syncthreads();
  }
  // y = W^H v: one warp per output entry, lanes down the column
  __device__ void adj_matvec(const C* W, size_t lda, const C* v, C* y) const {
    for (int i = threadIdx.x; i < n; i += kThreads) vs[i] = v[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < n; c += kWarps) {
      const C* col = W + lda * size_t(c);
      C s = mk<R>(R(0), R(0));
      for (int r = lane; r < n; r += 32) cfma(s, cconj(col[r]), vs[r]);
      for (int o = 16; o > 0; o >>= 1) {
        s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
        s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
      }
      if (lane == 0) y[c] = s;
    }
    __syncthreads();
  }
  // every entry with |re| <= tol and |im| <= tol
  __device__ bool within(const C* v, R tol) const {
    int ok = 1;
    for (int i = threadIdx.x; i < n; i += kThreads)
      if (!(fabs(v[i].x) <= tol && fabs(v[i].y) <= tol)) ok = 0;
    return __syncthreads_and(ok) != 0;
  }
  template <typename F> __device__ void each(F f) const {
    for (int i = threadIdx.x; i < n; i += kThreads) f(i);
    __syncthreads();
  }
};

// num-complex sqrt (axes special-cased, else the polar form)
template <typename R> __device__ cplx<R> csqrt_nc(cplx<R> z) {
  if (z.y == R(0)) {
    if (!signbit(z.x)) return mk<R>(sqrt(z.x), z.y);
    const R r = sqrt(-z.x);
    return mk<R>(R(0), signbit(z.y) ? -r : r);
  }
  if (z.x == R(0)) {
    const R x = sqrt(fabs(z.y) / R(2));
    return mk<R>(x, signbit(z.y) ? -x : x);
  }
  const R r = hypot(z.x, z.y), h = atan2(z.y, z.x) / R(2), sr = sqrt(r);
  return mk<R>(sr * cos(h), sr * sin(h));
}

enum : int { kOk = 0, kBreak = 1, kNoConv = 2 };

// ---------------------------------------------------------------------------
// the four solvers; each returns kOk / kBreak / kNoConv, x in V[0]
// ---------------------------------------------------------------------------
template <typename R>
__device__ int ggbi(const Cta<R>& K, const cplx<R>* W, size_t lda, int src, R tol, cplx<R>* V, int n) {
  using C = cplx<R>;
  C *x = V, *r = V + n, *a = V + 2 * n, *y = V + 3 * n, *s = V + 4 * n, *as = V + 5 * n;
  const C zero = mk<R>(R(0), R(0)), one = mk<R>(R(1), R(0));
  K.each([&](int i) { x[i] = zero; r[i] = i == src ? one : zero; });
  if (K.within(r, tol)) return kOk;
  K.matvec(W, lda, r, a);  // p = r
  C aa = K.dot(a, a), wa = K.dot(r, a), ww = K.dot(r, r);
  const C aw = cconj(wa);
  if (czero(aa) || czero(ww)) return kBreak;
  const C dd = csub(cmul(aa, ww), cmul(aw, wa));
  const C sdd = cdiv(cdiv(dd, aa), ww);
  if (hypot(sdd.x, sdd.y) < R(1.0e-8)) {
    K.each([&](int i) { y[i] = cdiv(r[i], ww); });
  } else {
    if (czero(dd)) return kBreak;
    ww = cdiv(csub(ww, aw), dd);
    aa = cdiv(csub(wa, aa), dd);
    K.each([&](int i) { y[i] = cadd(cmul(r[i], aa), cmul(a[i], ww)); });
  }
  const C del = K.dot(y, r), delp = K.dot(y, a);
  if (czero(delp)) return kBreak;
  const C omega = cdiv(del, delp);
  K.each([&](int i) { s[i] = csub(r[i], cmul(omega, a[i])); });
  if (K.within(s, tol)) {
    K.each([&](int i) { x[i] = cadd(x[i], cmul(omega, r[i])); });
    return kOk;
  }
  K.matvec(W, lda, s, as);
  const C a2 = K.dot(as, as), w2 = K.dot(as, s);
  if (czero(a2)) return kBreak;
  const C chi = cdiv(w2, a2);
  K.each([&](int i) { x[i] = cadd(x[i], cadd(cmul(omega, r[i]), cmul(chi, s[i]))); });
  return kOk;
}

template <typename R>
__device__ int ggrm(const Cta<R>& K, const cplx<R>* W, size_t lda, int src, R tol, cplx<R>* V, int n) {
  using C = cplx<R>;
  C *x = V, *r = V + n, *xket = V + 2 * n, *xbra = V + 3 * n, *tket = V + 4 * n, *tbra = V + 5 * n,
    *xketp = V + 6 * n, *xbrap = V + 7 * n, *z = V + 8 * n, *sv = V + 9 * n;
  const C zero = mk<R>(R(0), R(0)), one = mk<R>(R(1), R(0));
  K.each([&](int i) { x[i] = zero; });
  for (int restart = 0; restart < 128; ++restart) {
    if (restart > 0) K.matvec(W, lda, x, r);
    else K.each([&](int i) { r[i] = zero; });
    K.each([&](int i) {
      if (i == src) r[i] = csub(r[i], one);
      xket[i] = cneg(r[i]);
    });
    const C rn = K.dot(xket, xket);
    if (czero(rn)) return kOk;
    if (!(isfinite(rn.x) && rn.x > R(0))) return kBreak;
    const R xf = R(1) / rn.x;
    K.each([&](int i) { xbra[i] = cscale(xket[i], xf); });
    K.matvec(W, lda, xket, tket);
    C aa = K.dot(xbra, tket), aac = cconj(aa), bb = zero, bbc = zero, betac = aa;
    if (czero(betac)) return kBreak;
    C yy = one;
    K.each([&](int i) {
      xketp[i] = zero;
      xbrap[i] = zero;
      z[i] = xket[i];
      sv[i] = tket[i];
      x[i] = cadd(x[i], cdiv(z[i], betac));
      r[i] = cadd(r[i], cdiv(sv[i], betac));
    });
    for (int it = 0; it < 100; ++it) {
      K.each([&](int i) { tket[i] = csub(tket[i], cadd(cmul(aa, xket[i]), cmul(bb, xketp[i]))); });
      K.adj_matvec(W, lda, xbra, tbra);
      K.each([&](int i) { tbra[i] = csub(tbra[i], cadd(cmul(aac, xbra[i]), cmul(bbc, xbrap[i]))); });
      const C rnorm = K.dot(tbra, tket);
      if (czero(rnorm)) return kOk;
      bb = csqrt_nc<R>(rnorm);
      bbc = cconj(bb);
      if (czero(bb)) return kBreak;
      K.each([&](int i) {
        xketp[i] = xket[i];
        xbrap[i] = xbra[i];
        xket[i] = cdiv(tket[i], bb);
        xbra[i] = cdiv(tbra[i], bbc);
      });
      K.matvec(W, lda, xket, tket);
      aa = K.dot(xbra, tket);
      aac = cconj(aa);
      if (czero(betac)) return kBreak;
      const C alphac = cdiv(bb, betac);
      K.each([&](int i) {
        z[i] = csub(xket[i], cmul(alphac, z[i]));
        sv[i] = csub(tket[i], cmul(alphac, sv[i]));
      });
      betac = csub(aa, cmul(alphac, bb));
      if (czero(betac)) return kBreak;
      yy = cmul(cneg(alphac), yy);
      const C gamma = cdiv(yy, betac);
      K.each([&](int i) {
        x[i] = cadd(x[i], cmul(gamma, z[i]));
        r[i] = cadd(r[i], cmul(gamma, sv[i]));
      });
      if (K.within(r, tol)) return kOk;
    }
  }
  return kNoConv;
}

template <typename R>
__device__ int gggm(const Cta<R>& K, const cplx<R>* W, size_t lda, int src, R tol, cplx<R>* V, int n) {
  using C = cplx<R>;
  C *x = V, *b = V + n, *x0 = V + 2 * n, *r0 = V + 3 * n, *x1 = V + 4 * n, *r1 = V + 5 * n, *wv = V + 6 * n,
    *t0 = V + 7 * n, *tv = V + 8 * n;
  const C zero = mk<R>(R(0), R(0)), one = mk<R>(R(1), R(0));
  C q0 = one;
  K.each([&](int i) { x[i] = zero; x0[i] = zero; b[i] = i == src ? one : zero; });
  for (int restart = 0; restart < 128; ++restart) {
    if (restart > 0) {
      if (czero(q0)) return kBreak;
      K.each([&](int i) { x[i] = cadd(x[i], cdiv(x0[i], q0)); });
      K.matvec(W, lda, x, tv);
      K.each([&](int i) {
        b[i] = csub(tv[i], x[i]);
        if (i == src) b[i] = cadd(b[i], one);
      });
    }
    K.each([&](int i) { r0[i] = b[i]; x0[i] = zero; x1[i] = b[i]; });
    K.matvec(W, lda, b, r1);
    C ww = K.dot(r0, r0), aa = K.dot(r1, r1);
    const C wa = K.dot(r0, r1), aw = cconj(wa);
    if (czero(aa) || czero(ww)) return kBreak;
    const C dd = csub(cmul(aa, ww), cmul(aw, wa));
    const C sdd = cdiv(cdiv(dd, aa), ww);
    if (hypot(sdd.x, sdd.y) < R(1.0e-8)) {
      K.each([&](int i) { wv[i] = cdiv(r0[i], ww); });
    } else {
      if (czero(dd)) return kBreak;
      ww = cdiv(csub(ww, aw), dd);
      aa = cdiv(csub(wa, aa), dd);
      K.each([&](int i) { wv[i] = cadd(cmul(r0[i], aa), cmul(r1[i], ww)); });
    }
    C e0 = K.dot(wv, r0), e1 = K.dot(wv, r1);
    q0 = one;
    C q1 = one;
    for (int it = 0; it < 10; ++it) {
      const R t1l = tol * (hypot(q1.x, q1.y) / R(10));
      if (!(isfinite(t1l) && t1l >= R(0))) return kBreak;
      if (K.within(r1, t1l)) {
        if (czero(q1)) return kBreak;
        K.each([&](int i) { x[i] = cadd(x[i], cdiv(x1[i], q1)); });
        return kOk;
      }
      if (czero(e0)) return kBreak;
      const C alpha = cdiv(e1, e0);
      K.each([&](int i) { t0[i] = csub(r1[i], cmul(alpha, r0[i])); });
      K.matvec(W, lda, t0, tv);
      const C wa2 = K.dot(t0, tv), ww2 = K.dot(t0, t0), aa2 = K.dot(tv, tv);
      const C den = csub(ww2, cconj(wa2));
      if (czero(den)) return kBreak;
      const C theta = cdiv(csub(wa2, aa2), den);
      const C d1 = csub(one, theta);
      K.each([&](int i) {
        r0[i] = csub(tv[i], cmul(theta, t0[i]));
        x0[i] = cadd(t0[i], cmul(d1, csub(x1[i], cmul(alpha, x0[i]))));
      });
      q0 = cmul(d1, csub(q1, cmul(alpha, q0)));
      const R t0l = tol * hypot(q0.x, q0.y);
      if (!(isfinite(t0l) && t0l >= R(0))) return kBreak;
      if (K.within(r0, t0l)) {
        if (czero(q0)) return kBreak;
        K.each([&](int i) { x[i] = cadd(x[i], cdiv(x0[i], q0)); });
        return kOk;
      }
      e0 = K.dot(wv, r0);
      if (czero(e1)) return kBreak;
      const C beta = cdiv(e0, e1);
      K.each([&](int i) { t0[i] = csub(r0[i], cmul(beta, r1[i])); });
      K.matvec(W, lda, t0, tv);
      const C d2 = cmul(beta, theta);
      K.each([&](int i) { r1[i] = cadd(tv[i], cmul(d2, r1[i])); });
      e1 = K.dot(wv, r1);
      const C d3 = cmul(beta, d1);
      K.each([&](int i) { x1[i] = cadd(csub(x0[i], cmul(d3, x1[i])), t0[i]); });
      q1 = csub(q0, cmul(cmul(d1, beta), q1));
    }
  }
  return kNoConv;
}

template <typename R>
__device__ int ggtf(const Cta<R>& K, const cplx<R>* W, size_t lda, int src, R tol, cplx<R>* V, int n) {
  using C = cplx<R>;
  C *x = V, *a = V + n, *u = V + 2 * n, *w = V + 3 * n, *v = V + 4 * n, *d = V + 5 * n, *rv = V + 6 * n;
  const C zero = mk<R>(R(0), R(0)), one = mk<R>(R(1), R(0));
  K.each([&](int i) { x[i] = zero; a[i] = zero; });
  for (int restart = 0; restart < 128; ++restart) {
    if (restart > 0) K.matvec(W, lda, x, a);
    K.each([&](int i) {
      u[i] = cneg(a[i]);
      if (i == src) u[i] = cadd(u[i], one);
    });
    K.matvec(W, lda, u, a);
    K.each([&](int i) { w[i] = u[i]; v[i] = a[i]; d[i] = zero; });
    const C aa0 = K.dot(u, u);
    if (czero(aa0)) return kBreak;
    if (!(isfinite(aa0.x) && aa0.x > R(0))) return kBreak;
    R tau = sqrt(aa0.x), nu = R(0);
    C eta = zero, alpha = zero, rho = one;
    K.each([&](int i) { rv[i] = cdiv(u[i], aa0); });
    for (int nit = 0; nit <= 20; ++nit) {
      if (nit % 2 == 0) {
        const C rvv = K.dot(rv, v);
        if (czero(rvv)) return kBreak;
        alpha = cdiv(rho, rvv);
      } else {
        K.matvec(W, lda, u, a);
      }
      if (czero(alpha)) return kBreak;
      const C f = cdiv(cscale(eta, nu * nu), alpha);
      K.each([&](int i) {
        w[i] = csub(w[i], cmul(alpha, a[i]));
        d[i] = cadd(u[i], cmul(f, d[i]));
      });
      const C wn = K.dot(w, w);
      if (!(isfinite(wn.x) && wn.x >= R(0))) return kBreak;
      nu = sqrt(wn.x) / tau;
      const R cm = R(1) / sqrt(R(1) + nu * nu);
      tau *= nu * cm;
      eta = cscale(alpha, cm * cm);
      K.each([&](int i) { x[i] = cadd(x[i], cmul(eta, d[i])); });
      const R err = tau * sqrt((R(1) + R(nit)) / R(n)) * R(10);
      if (fabs(err) < tol) return kOk;
      if (nit % 2 != 0) {
        const C prho = rho;
        rho = K.dot(rv, w);
        if (czero(prho)) return kBreak;
        const C beta = cdiv(rho, prho);
        K.each([&](int i) {
          u[i] = cadd(w[i], cmul(beta, u[i]));
          v[i] = cmul(beta, cadd(a[i], cmul(beta, v[i])));
        });
        K.matvec(W, lda, u, a);
        K.each([&](int i) { v[i] = cadd(v[i], a[i]); });
      } else {
        K.each([&](int i) { u[i] = csub(u[i], cmul(alpha, v[i])); });
      }
    }
  }
  return kNoConv;
}

template <typename R, int kMethod>
__global__ void __launch_bounds__(kThreads) iterative_solve_kernel(IterArgs a) {
  using C = cplx<R>;
  extern __shared__ unsigned char smem_raw[];
  C* vs = reinterpret_cast<C*>(smem_raw);
  C* red = vs + a.n;
  const int col = blockIdx.x, e = blockIdx.y, n = a.n, m = a.m;
  if (a.skip && a.skip[e]) return;
  Cta<R> K{n, red, vs};
  const C* W = reinterpret_cast<const C*>(a.W) + size_t(e) * a.stride;
  C* V = reinterpret_cast<C*>(a.scratch) + (size_t(e) * m + col) * kIterVectors * size_t(n);
  // the source state of this column: column col - bl.col of its potential's block
  // (iterative.rs:98-150: solve A' x = e_src for every representative state)
  const SolvedBlock& bl = block_of(a.blocks, a.nblocks, col);
  const int lc = col - bl.col;
  const int src = bl.row + lc;
  const R tol = R(a.tol1);
  int rc;
  if (kMethod == 1) rc = ggbi<R>(K, W, a.lda, src, tol, V, n);
  else if (kMethod == 2) rc = ggrm<R>(K, W, a.lda, src, tol, V, n);
  else if (kMethod == 3) rc = gggm<R>(K, W, a.lda, src, tol, V, n);
  else rc = ggtf<R>(K, W, a.lda, src, tol, V, n);
  if (rc != kOk) {
    if (threadIdx.x == 0) atomicMax(a.status + e, rc == kBreak ? int(kDevBreakdown) : int(kDevNotConverged));
    return;
  }
  // block entry (row, lc) = sum_s G0[bl.row + row, s] x[s]
  const C* grow = reinterpret_cast<const C*>(a.grow) + size_t(e) * m * n;
  const C* x = V;
  for (int row = 0; row < bl.size; ++row) {
    C s = mk<R>(R(0), R(0));
    for (int i = threadIdx.x; i < n; i += kThreads) cfma(s, grow[size_t(bl.col + row) + size_t(m) * i], x[i]);
    s = K.reduce(s);
    if (threadIdx.x == 0)
      a.gg[size_t(e) * a.gg_per + size_t(bl.pack) + size_t(row) + size_t(bl.size) * lc] = ccast<double2>(s);
  }
}

template <typename R, int kMethod>
cudaError_t launch_solve(const IterArgs& a, int batch, cudaStream_t s) {
  const size_t smem = (size_t(a.n) + kWarps + 1) * sizeof(cplx<R>);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = ensure_smem_limit(reinterpret_cast<const void*>(iterative_solve_kernel<R, kMethod>), smem);
    if (e != cudaSuccess) return e;
  }
  count_launch();
  iterative_solve_kernel<R, kMethod><<<dim3(unsigned(a.m), unsigned(batch)), kThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_iterative_t(int minv, const BatchLayout& lay, int batch, const double2* G0, void* W,
                               const double2* t, const int* partner, double tol1, double tol2, void* grow,
                               void* scratch, const SolvedBlock* blocks, int nblocks, int gg_per, double2* gg,
                               int* status, cudaStream_t s) {
  {
    const unsigned gx = unsigned(std::min(256, (lay.m * lay.n + 255) / 256));
    count_launch();
    block_rows_kernel<R><<<dim3(gx, unsigned(batch)), 256, 0, s>>>(lay, G0, blocks, nblocks,
                                                                  reinterpret_cast<cplx<R>*>(grow));
  }
  {
    const bool gms = minv == 3;
    dim3 grid(unsigned((lay.n + 255) / 256), unsigned(lay.n), unsigned(batch));
    count_launch();
    iterative_system_kernel<R><<<grid, 256, 0, s>>>(lay, G0, reinterpret_cast<cplx<R>*>(W), t, partner, tol2,
                                                   gms ? 1.0 : -1.0, gms ? 0.0 : 1.0);
  }
  IterArgs a;
  a.n = lay.n;
  a.m = lay.m;
  a.lda = size_t(lay.lda);
  a.stride = lay.stride;
  a.W = W;
  a.grow = grow;
  a.scratch = scratch;
  a.blocks = blocks;
  a.nblocks = nblocks;
  a.gg_per = gg_per;
  a.gg = gg;
  a.status = status;
  a.skip = nullptr;
  a.tol1 = tol1;
  switch (minv) {
    case 1: return launch_solve<R, 1>(a, batch, s);
    case 2: return launch_solve<R, 2>(a, batch, s);
    case 3: return launch_solve<R, 3>(a, batch, s);
    default: return launch_solve<R, 4>(a, batch, s);
  }
}

}  // namespace

cudaError_t launch_iterative(bool fp64, int minv, const BatchLayout& lay, int batch, double2* G0, float2* W32,
                             const double2* t, const int* partner, double tol1, double tol2, void* grow, void* scratch,
                             const SolvedBlock* blocks, int nblocks, int gg_per, double2* gg, int* status,
                             cudaStream_t s) {
  if (fp64)
    return launch_iterative_t<double>(minv, lay, batch, G0, G0, t, partner, tol1, tol2, grow, scratch, blocks, nblocks,
                                      gg_per, gg, status, s);
  return launch_iterative_t<float>(minv, lay, batch, G0, W32, t, partner, tol1, tol2, grow, scratch, blocks, nblocks,
                                   gg_per, gg, status, s);
}

}  // namespace rfx
