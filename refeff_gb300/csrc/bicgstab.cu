// Batched right-preconditioned BiCGSTAB for the dense FMS systems.
//
// The reference's iterative form solves each absorber column on its own
// (fms_bicgstab_solve, crates/refeff-core/src/fms/internals/iterative.rs:181-254),
// so every column streams the whole matrix once per matrix-vector product.
// Here the m absorber columns of every energy in a batch advance together:
// one product kernel reads each FP32 system matrix once per product for all m
// columns, and the per-column scalars (rho, alpha, omega) live in FP64 with
// FP64 dot-product accumulation.  Right preconditioning by a diagonal D or a
// block diagonal (one channel block per atom; the learned form) solves
// A P y = b and returns x = P y.
//
// Iteration (van der Vorst), per column:
//   beta = (rho_new / rho)(alpha / omega);  p = r + beta (p - omega v);  p^ = D p
//   v = A p^;  alpha = rho_new / (r~, v);   s = r - alpha v;  s^ = D s
//   t = A s^;  omega = (t, s) / (t, t);     x += alpha p^ + omega s^;  r = s - omega t
//   rho_new = (r~, r);  stop when |r| <= tol |b|.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "bicgstab.cuh"
#include "cplx.cuh"

namespace rfx {
namespace {

// scalar slots per (matrix, column)
// complex values take two slots (re, im)
enum : int { kRho = 0, kAlpha = 2, kOmega = 4, kB2 = 6, kAcc1 = 7, kAcc2 = 9, kAcc3 = 11, kAcc4 = 12 };
static_assert(kAcc4 < kBicgScalars, "scalar slots");
enum : int { kX = 0, kR = 1, kRh = 2, kP = 3, kV = 4, kPh = 5, kSh = 6, kT = 7 };

constexpr int kVecThreads = 256, kVecRowsPerThread = 4, kVecRows = kVecThreads * kVecRowsPerThread;

struct View {
  int n, m, lda, batch;
  float2* vec;
  double* sc;
  int* state;
  int* done;
  float2* part;    // partial products of slices 1..nsplit-1 of the last split product
  int nsplit = 1;  // column slices of that product (1: not split)
  const int* act = nullptr;  // running matrices, compacted (-1 past the count); NULL: blockIdx.y is the matrix
  __device__ __forceinline__ int matrix() const { return act ? act[blockIdx.y] : int(blockIdx.y); }
  __device__ float2* v(int k, int b, int c) const {
    return vec + (size_t(k) * batch + b) * size_t(lda) * m + size_t(lda) * c;
  }
  __device__ float2* pv(int slice, int b, int c) const {  // slice >= 1
    return part + ((size_t(slice - 1) * batch + b) * m + c) * size_t(lda);
  }
  __device__ double* s(int b, int c) const { return sc + (size_t(b) * m + c) * kBicgScalars; }
  // y[i] += the other slices' partial products, written back (slice 0 wrote y)
  __device__ __forceinline__ float2 gather(float2* y, int b, int c, int i) const {
    float2 a = y[i];
    if (nsplit > 1) {
      for (int sl = 1; sl < nsplit; ++sl) a = cadd(a, pv(sl, b, c)[i]);
      y[i] = a;
    }
    return a;
  }
};

__device__ __forceinline__ double2 cdot_acc(double2 acc, float2 a, float2 b) {  // acc += conj(a) b
  acc.x += double(a.x) * b.x + double(a.y) * b.y;
  acc.y += double(a.x) * b.y - double(a.y) * b.x;
  return acc;
}

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kVecThreads / 32; ++i) t += red[i];
  return t;  // valid on thread 0
}

// Adds the block's partial sums of up to three values to sc slots (one atomic each).
__device__ __forceinline__ void block_accumulate(double* slot0, double a, double* slot1, double b, double* slot2,
                                                 double c) {
  __shared__ double red[kVecThreads / 32];
  const double ta = block_sum(a, red);
  const double tb = slot1 ? block_sum(b, red) : 0.0;
  const double tc = slot2 ? block_sum(c, red) : 0.0;
  if (threadIdx.x == 0) {
    atomicAdd(slot0, ta);
    if (slot1) atomicAdd(slot1, tb);
    if (slot2) atomicAdd(slot2, tc);
  }
}

__device__ __forceinline__ bool column_idle(const View& w, int b, int c, const int* skip) {
  return (skip && skip[b]) || w.done[b] || w.state[size_t(b) * w.m + c] != 0;
}

// x = 0, r = r~ = b, p = v = 0; |b|^2 and rho = (r~, r) accumulated.
__global__ void bicg_init_kernel(View w, const float2* __restrict__ M32, size_t stride, const int* skip) {
  const int b = blockIdx.y, c = blockIdx.z;
  if (skip && skip[b]) return;
  const float2* rhs = M32 + size_t(b) * stride + size_t(w.lda) * (w.n + c);
  float2 *x = w.v(kX, b, c), *r = w.v(kR, b, c), *rh = w.v(kRh, b, c), *p = w.v(kP, b, c), *v = w.v(kV, b, c);
  double b2 = 0.0;
  for (int k = 0; k < kVecRowsPerThread; ++k) {
    const int i = blockIdx.x * kVecRows + k * kVecThreads + threadIdx.x;
    if (i >= w.n) break;
    const float2 bi = rhs[i];
    x[i] = make_float2(0.f, 0.f);
    r[i] = bi;
    rh[i] = bi;
    p[i] = make_float2(0.f, 0.f);
    v[i] = make_float2(0.f, 0.f);
    b2 += double(bi.x) * bi.x + double(bi.y) * bi.y;
  }
  double* sc = w.s(b, c);
  // rho_new = (r~, r) = |b|^2 at the start
  block_accumulate(sc + kB2, b2, sc + kAcc1, b2, nullptr, 0.0);
}

// p = r + beta (p - omega v);  p^ = D p
__global__ void bicg_p_kernel(View w, const float2* __restrict__ D, const int* skip) {
  const int b = w.matrix(), c = blockIdx.z;
  if (b < 0) return;
  if (column_idle(w, b, c, skip)) return;
  const double* sc = w.s(b, c);
  const double2 rho_new = make_double2(sc[kAcc1], sc[kAcc1 + 1]);
  const double2 rho = make_double2(sc[kRho], sc[kRho + 1]);
  const double2 alpha = make_double2(sc[kAlpha], sc[kAlpha + 1]);
  const double2 omega = make_double2(sc[kOmega], sc[kOmega + 1]);
  const double2 beta = cmul(cdiv(rho_new, rho), cdiv(alpha, omega));
  const float2 bf = make_float2(float(beta.x), float(beta.y)), of = make_float2(float(omega.x), float(omega.y));
  const float2 *r = w.v(kR, b, c), *v = w.v(kV, b, c);
  float2 *p = w.v(kP, b, c), *ph = w.v(kPh, b, c);
  const float2* Db = D ? D + size_t(b) * w.lda : nullptr;
  for (int k = 0; k < kVecRowsPerThread; ++k) {
    const int i = blockIdx.x * kVecRows + k * kVecThreads + threadIdx.x;
    if (i >= w.n) break;
    float2 pi = csub(p[i], cmul(of, v[i]));
    pi = cadd(r[i], cmul(bf, pi));
    p[i] = pi;
    ph[i] = Db ? cmul(Db[i], pi) : pi;
  }
}

// Y = A X for the FP32 system matrices: 128 rows x 16 columns per CTA, each
// thread 4 rows (rg + 32 i) x 4 adjacent columns (read as two 16-byte
// shared loads), A streamed through shared memory in 16-column slabs by a
// three-stage cp.async pipeline (each A entry is read from HBM once per
// product; rows past n and columns past the slice are zero-filled by the
// copies; 55 KB per CTA, four CTAs per SM).  The columns of A are split into
// w.nsplit slices of kchunk (blockIdx.z = column group + groups * slice), so
// that even one running matrix spreads over the SMs: slice 0 writes Y, slice
// s > 0 its partial product, and the next dot kernel sums them in slice order.
constexpr int kMvRows = 128, kMvCols = 16, kMvK = 16, kMvThreads = 128, kMvStages = 3, kMvSliceCols = 512;
constexpr size_t kMvSmem = size_t(kMvStages) * kMvK * (kMvRows + kMvCols) * sizeof(float2);

__device__ __forceinline__ void cp_async16(void* dst, const void* src, int bytes) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src, int bytes) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__global__ void __launch_bounds__(kMvThreads) bicg_matvec_kernel(View w, const float2* __restrict__ M32, size_t stride,
                                                                  int src, int dst, int groups, int kchunk,
                                                                  const int* skip) {
  const int b = w.matrix();
  if (b < 0 || (skip && skip[b]) || w.done[b]) return;
  extern __shared__ __align__(16) float2 mv_smem[];
  float2* As = mv_smem;                                       // [stage][kMvK][kMvRows]
  float2* Xs = mv_smem + size_t(kMvStages) * kMvK * kMvRows;  // [stage][kMvK][kMvCols]
  const int slice = blockIdx.z / groups;
  const int n = w.n, r0 = blockIdx.x * kMvRows, c0 = (blockIdx.z % groups) * kMvCols;
  const int kbeg = slice * kchunk, kend = min(n, kbeg + kchunk);
  const int slabs = (kend - kbeg + kMvK - 1) / kMvK;
  const float2* A = M32 + size_t(b) * stride;
  const int tid = threadIdx.x, rg = tid & 31, cq = tid >> 5;
  // one slab: kMvK columns of A (128 rows as 16-byte row pairs) and of X; a
  // slab past the slice's end commits an empty group (uniform group counts)
  auto load = [&](int slab) {
    if (slab < slabs) {
      const int k0 = kbeg + slab * kMvK, stage = slab % kMvStages;
      float2* as = As + size_t(stage) * kMvK * kMvRows;
      float2* xs = Xs + size_t(stage) * kMvK * kMvCols;
      for (int idx = tid; idx < kMvK * (kMvRows / 2); idx += kMvThreads) {
        const int rr = (idx % (kMvRows / 2)) * 2, kk = idx / (kMvRows / 2), row = r0 + rr;
        const bool in = k0 + kk < kend && row < n;
        const int bytes = in ? (row + 1 < n ? 16 : 8) : 0;
        cp_async16(as + size_t(kk) * kMvRows + rr, in ? A + size_t(row) + size_t(w.lda) * (k0 + kk) : A, bytes);
      }
      for (int idx = tid; idx < kMvK * kMvCols; idx += kMvThreads) {
        const int kk = idx % kMvK, cc = idx / kMvK;
        const bool in = k0 + kk < kend && c0 + cc < w.m;
        const float2* xsrc = in ? w.v(src, b, c0 + cc) + (k0 + kk) : A;
        cp_async8(xs + size_t(kk) * kMvCols + cc, xsrc, in ? 8 : 0);
      }
    }
    cp_async_commit();
  };
  float2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);
#pragma unroll
  for (int sl = 0; sl < kMvStages - 1; ++sl) load(sl);
  for (int sl = 0; sl < slabs; ++sl) {
    cp_async_wait<kMvStages - 2>();  // slab sl has landed (this thread's copies)
    __syncthreads();                 // ... everyone's; and slab sl - 1's stage is free again
    load(sl + kMvStages - 1);
    const int stage = sl % kMvStages;
    const float2* as = As + size_t(stage) * kMvK * kMvRows;
    const float4* xs = reinterpret_cast<const float4*>(Xs + size_t(stage) * kMvK * kMvCols);
#pragma unroll
    for (int kk = 0; kk < kMvK; ++kk) {
      float2 a[4], x[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = as[kk * kMvRows + rg + 32 * i];
      const float4 x01 = xs[(kk * kMvCols + 4 * cq) / 2], x23 = xs[(kk * kMvCols + 4 * cq) / 2 + 1];
      x[0] = make_float2(x01.x, x01.y);
      x[1] = make_float2(x01.z, x01.w);
      x[2] = make_float2(x23.x, x23.y);
      x[3] = make_float2(x23.z, x23.w);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(acc[i][j], a[i], x[j]);
    }
  }
  cp_async_wait<0>();  // no copy outlives the CTA (the trailing groups are empty)
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = c0 + 4 * cq + j;
    if (c >= w.m) continue;
    float2* y = slice == 0 ? w.v(dst, b, c) : w.pv(slice, b, c);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = r0 + rg + 32 * i;
      if (r < n) y[r] = acc[i][j];
    }
  }
}

// acc2 += (r~, v)
__global__ void bicg_dot_rv_kernel(View w, const int* skip) {
  const int b = w.matrix(), c = blockIdx.z;
  if (b < 0) return;
  if (column_idle(w, b, c, skip)) return;
  const float2* rh = w.v(kRh, b, c);
  float2* v = w.v(kV, b, c);
  double2 acc = make_double2(0.0, 0.0);
  for (int k = 0; k < kVecRowsPerThread; ++k) {
    const int i = blockIdx.x * kVecRows + k * kVecThreads + threadIdx.x;
    if (i >= w.n) break;
    acc = cdot_acc(acc, rh[i], w.gather(v, b, c, i));
  }
  double* sc = w.s(b, c);
  block_accumulate(sc + kAcc2, acc.x, sc + kAcc2 + 1, acc.y, nullptr, 0.0);
}

__device__ __forceinline__ bool czero(double2 z) { return z.x == 0.0 && z.y == 0.0; }

// alpha = rho_new / (r~, v); rho = rho_new.  One thread per (matrix, column).
__global__ void bicg_alpha_kernel(View w, const int* skip) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= w.batch * w.m) return;
  const int b = idx / w.m, c = idx % w.m;
  if (column_idle(w, b, c, skip)) return;
  double* sc = w.s(b, c);
  if (sc[kB2] == 0.0) {  // b = 0: x = 0 is exact
    w.state[idx] = 1;
    return;
  }
  const double2 rho_new = make_double2(sc[kAcc1], sc[kAcc1 + 1]);
  const double2 rv = make_double2(sc[kAcc2], sc[kAcc2 + 1]);
  sc[kAcc1] = sc[kAcc1 + 1] = sc[kAcc2] = sc[kAcc2 + 1] = 0.0;
  if (czero(rho_new) || czero(rv) || !isfinite(rv.x) || !isfinite(rv.y)) {
    w.state[idx] = 2;
    return;
  }
  const double2 alpha = cdiv(rho_new, rv);
  sc[kAlpha] = alpha.x;
  sc[kAlpha + 1] = alpha.y;
  sc[kRho] = rho_new.x;
  sc[kRho + 1] = rho_new.y;
}

// dst = Bblk src for every running column: the block-diagonal preconditioner,
// one C x C block per atom (Bblk[(b N + atom) C^2 + q C + q']), one thread
// per row.
__global__ void bicg_block_apply_kernel(View w, int src, int dst, const float2* __restrict__ Bblk,
                                        const int* __restrict__ state_atom, const int* __restrict__ atom_off, int N,
                                        int C, const int* skip) {
  const int b = w.matrix(), c = blockIdx.z;
  if (b < 0) return;
  if (column_idle(w, b, c, skip)) return;
  const float2* in = w.v(src, b, c);
  float2* out = w.v(dst, b, c);
  for (int k = 0; k < kVecRowsPerThread; ++k) {
    const int i = blockIdx.x * kVecRows + k * kVecThreads + threadIdx.x;
    if (i >= w.n) break;
    const int a = state_atom[i], s0 = atom_off[a], cnt = atom_off[a + 1] - s0, q = i - s0;
    const float2* row = Bblk + ((size_t(b) * N + a) * C + q) * C;
    float2 acc = make_float2(0.f, 0.f);
    for (int q2 = 0; q2 < cnt; ++q2) cfma(acc, row[q2], in[s0 + q2]);
    out[i] = acc;
  }
}

// s = r - alpha v (in r);  s^ = D s
__global__ void bicg_s_kernel(View w, const float2* __restrict__ D, const int* skip) {
  const int b = w.matrix(), c = blockIdx.z;
  if (b < 0) return;
  if (column_idle(w, b, c, skip)) return;
  const double* sc = w.s(b, c);
  const float2 af = make_float2(float(sc[kAlpha]), float(sc[kAlpha + 1]));
  float2 *r = w.v(kR, b, c), *sh = w.v(kSh, b, c);
  const float2* v = w.v(kV, b, c);
  const float2* Db = D ? D + size_t(b) * w.lda : nullptr;
  for (int k = 0; k < kVecRowsPerThread; ++k) {
    const int i = blockIdx.x * kVecRows + k * kVecThreads + threadIdx.x;
    if (i >= w.n) break;
    const float2 si = csub(r[i], cmul(af, v[i]));
    r[i] = si;
    sh[i] = Db ? cmul(Db[i], si) : si;
  }
}

// acc2 += (t, s), acc3 += |t|^2
__global__ void bicg_dot_ts_kernel(View w, const int* skip) {
  const int b = w.matrix(), c = blockIdx.z;
  if (b < 0) return;
  if (column_idle(w, b, c, skip)) return;
  float2* t = w.v(kT, b, c);
  const float2* sv = w.v(kR, b, c);
  double2 ts = make_double2(0.0, 0.0);
  double tt = 0.0;
  for (int k = 0; k < kVecRowsPerThread; ++k) {
    const int i = blockIdx.x * kVecRows + k * kVecThreads + threadIdx.x;
    if (i >= w.n) break;
    const float2 ti = w.gather(t, b, c, i);
    ts = cdot_acc(ts, ti, sv[i]);
    tt += double(ti.x) * ti.x + double(ti.y) * ti.y;
  }
  double* sc = w.s(b, c);
  block_accumulate(sc + kAcc2, ts.x, sc + kAcc2 + 1, ts.y, sc + kAcc3, tt);
}

// omega = (t, s) / (t, t)
__global__ void bicg_omega_kernel(View w, const int* skip) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= w.batch * w.m) return;
  const int b = idx / w.m, c = idx % w.m;
  if (column_idle(w, b, c, skip)) return;
  double* sc = w.s(b, c);
  const double2 ts = make_double2(sc[kAcc2], sc[kAcc2 + 1]);
  const double tt = sc[kAcc3];
  sc[kAcc2] = sc[kAcc2 + 1] = sc[kAcc3] = 0.0;
  if (!(tt > 0.0) || czero(ts) || !isfinite(ts.x) || !isfinite(ts.y)) {
    w.state[idx] = 2;
    return;
  }
  sc[kOmega] = ts.x / tt;
  sc[kOmega + 1] = ts.y / tt;
}

// x += alpha p^ + omega s^;  r = s - omega t;  acc4 += |r|^2, acc1 += (r~, r)
__global__ void bicg_xr_kernel(View w, const int* skip) {
  const int b = w.matrix(), c = blockIdx.z;
  if (b < 0) return;
  if (column_idle(w, b, c, skip)) return;
  const double* sc = w.s(b, c);
  const float2 af = make_float2(float(sc[kAlpha]), float(sc[kAlpha + 1]));
  const float2 of = make_float2(float(sc[kOmega]), float(sc[kOmega + 1]));
  float2 *x = w.v(kX, b, c), *r = w.v(kR, b, c);
  const float2 *ph = w.v(kPh, b, c), *sh = w.v(kSh, b, c), *t = w.v(kT, b, c), *rh = w.v(kRh, b, c);
  double rr = 0.0;
  double2 rho = make_double2(0.0, 0.0);
  for (int k = 0; k < kVecRowsPerThread; ++k) {
    const int i = blockIdx.x * kVecRows + k * kVecThreads + threadIdx.x;
    if (i >= w.n) break;
    x[i] = cadd(x[i], cadd(cmul(af, ph[i]), cmul(of, sh[i])));
    const float2 ri = csub(r[i], cmul(of, t[i]));
    r[i] = ri;
    rr += double(ri.x) * ri.x + double(ri.y) * ri.y;
    rho = cdot_acc(rho, rh[i], ri);
  }
  double* s2 = w.s(b, c);
  block_accumulate(s2 + kAcc4, rr, s2 + kAcc1, rho.x, s2 + kAcc1 + 1, rho.y);
}

// Convergence per column; per matrix done flag and iteration count; the
// number of running matrices for the host poll.
__global__ void bicg_check_kernel(View w, double tol2, int iter, int* iters, int* active, const int* skip) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= w.batch) return;
  if ((skip && skip[b]) || w.done[b]) return;
  bool all = true;
  for (int c = 0; c < w.m; ++c) {
    int& st = w.state[size_t(b) * w.m + c];
    double* sc = w.s(b, c);
    if (st == 0) {
      const double rr = sc[kAcc4];
      if (!isfinite(rr)) st = 2;
      else if (rr <= tol2 * sc[kB2]) st = 1;
    }
    sc[kAcc4] = 0.0;
    all = all && st != 0;
  }
  iters[b] = iter;
  if (all) w.done[b] = 1;
  else atomicAdd(active, 1);
}

// The compacted list of running matrices (one block, batch <= kCompactMax):
// act[0..count) the running ones in order, -1 after.
constexpr int kCompactMax = 1024;
__device__ __forceinline__ void compact_running(bool alive, int b, int batch, int* act) {
  __shared__ int warp_total[kCompactMax / 32];
  const unsigned bal = __ballot_sync(0xffffffffu, alive);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) warp_total[wid] = __popc(bal);
  __syncthreads();
  int base = 0, total = 0;
  for (int i = 0; i < int(blockDim.x >> 5); ++i) {
    if (i < wid) base += warp_total[i];
    total += warp_total[i];
  }
  if (alive) act[base + __popc(bal & ((1u << lane) - 1u))] = b;
  if (b >= total && b < batch) act[b] = -1;  // disjoint from the positions below total
}

__global__ void bicg_act_init_kernel(int batch, const int* skip, int* act) {
  const int b = threadIdx.x;
  compact_running(b < batch && !(skip && skip[b]), b, batch, act);
}

// bicg_check_kernel for one block over the whole batch, which also rebuilds
// the compacted list of running matrices for the next iteration's launches.
__global__ void bicg_check_compact_kernel(View w, double tol2, int iter, int* iters, int* active, const int* skip,
                                          int* act) {
  const int b = threadIdx.x;
  bool alive = false;
  if (b < w.batch && !(skip && skip[b]) && !w.done[b]) {
    bool all = true;
    for (int c = 0; c < w.m; ++c) {
      int& st = w.state[size_t(b) * w.m + c];
      double* sc = w.s(b, c);
      if (st == 0) {
        const double rr = sc[kAcc4];
        if (!isfinite(rr)) st = 2;
        else if (rr <= tol2 * sc[kB2]) st = 1;
      }
      sc[kAcc4] = 0.0;
      all = all && st != 0;
    }
    iters[b] = iter;
    if (all) {
      w.done[b] = 1;
    } else {
      alive = true;
      atomicAdd(active, 1);
    }
  }
  compact_running(alive, b, w.batch, act);
}

// Solution X -> RHS columns of M32; failed[b] = 2 when a column did not converge.
__global__ void bicg_finish_kernel(View w, float2* __restrict__ M32, size_t stride, int* failed, const int* skip) {
  const int b = blockIdx.y, c = blockIdx.z;
  if (skip && skip[b]) return;
  const float2* x = w.v(kX, b, c);
  float2* out = M32 + size_t(b) * stride + size_t(w.lda) * (w.n + c);
  for (int k = 0; k < kVecRowsPerThread; ++k) {
    const int i = blockIdx.x * kVecRows + k * kVecThreads + threadIdx.x;
    if (i >= w.n) break;
    out[i] = x[i];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && w.state[size_t(b) * w.m + c] != 1) failed[b] = 2;
}

}  // namespace

cudaError_t bicgstab_solve(const BatchLayout& lay, int batch, float2* M32, const float2* D, const BlockPrecond* blk,
                           const BicgWork& w, double tol, int max_iter, int poll, const int* skip, int* failed,
                           cudaStream_t s) {
  View v{lay.n, lay.m, lay.lda, batch, w.vec, w.sc, w.state, w.done, w.part, 1};
  const dim3 vgrid(unsigned((lay.n + kVecRows - 1) / kVecRows), unsigned(batch), unsigned(lay.m));
  const int row_blocks = (lay.n + kMvRows - 1) / kMvRows, groups = (lay.m + kMvCols - 1) / kMvCols;
  {
    const cudaError_t e = cudaFuncSetAttribute(bicg_matvec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               int(kMvSmem));
    if (e != cudaSuccess) return e;
  }
  // Slices of A's columns: kMvSliceCols columns each (more for large n, at
  // most kBicgMaxSplit slices), so that the last running matrices still fill the
  // GPU with product CTAs.  The slicing depends on n alone: a matrix's
  // arithmetic does not depend on which others share its batch.
  int chunk = lay.n, nsplit = 1;
  if (w.part) {
    chunk = std::max(kMvSliceCols, ((lay.n + kBicgMaxSplit - 1) / kBicgMaxSplit + kMvK - 1) / kMvK * kMvK);
    nsplit = (lay.n + chunk - 1) / chunk;
  }
  const int sthreads = 128, sblocks = (batch * lay.m + sthreads - 1) / sthreads;
  const int bblocks = (batch + sthreads - 1) / sthreads;
  cudaMemsetAsync(w.sc, 0, size_t(batch) * lay.m * kBicgScalars * sizeof(double), s);
  cudaMemsetAsync(w.state, 0, size_t(batch) * lay.m * sizeof(int), s);
  cudaMemsetAsync(w.done, 0, size_t(batch) * sizeof(int), s);
  cudaMemsetAsync(w.iters, 0, size_t(batch) * sizeof(int), s);
  // rho = alpha = omega = 1 (the first p = r)
  {
    std::vector<double> init(size_t(batch) * lay.m * kBicgScalars, 0.0);
    for (size_t i = 0; i < size_t(batch) * lay.m; ++i) {
      init[i * kBicgScalars + kRho] = 1.0;
      init[i * kBicgScalars + kAlpha] = 1.0;
      init[i * kBicgScalars + kOmega] = 1.0;
    }
    cudaMemcpyAsync(w.sc, init.data(), init.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    count_launch();
    bicg_init_kernel<<<vgrid, kVecThreads, 0, s>>>(v, M32, lay.stride, skip);
    // the host vector must outlive the copy
    cudaStreamSynchronize(s);
  }
  // The iteration's launches cover only the running matrices: the check
  // kernel keeps a compacted list of them, and the grids are sized by the
  // count of the last host poll (an upper bound: matrices only finish).
  const bool compact = w.act && batch <= kCompactMax;
  const unsigned cthreads = unsigned((batch + 31) / 32 * 32);
  if (compact) {
    count_launch();
    bicg_act_init_kernel<<<1, cthreads, 0, s>>>(batch, skip, w.act);
  }
  View vr = v;  // the view of the iteration's launches
  vr.act = compact ? w.act : nullptr;
  int running = batch;
  for (int it = 1; it <= max_iter && running > 0; ++it) {
    vr.nsplit = nsplit;  // the dot kernels sum the slices
    const unsigned rows_y = unsigned(compact ? running : batch);
    const dim3 rgrid(vgrid.x, rows_y, vgrid.z);
    const dim3 mgrid(unsigned(row_blocks), rows_y, unsigned(groups * vr.nsplit));
    count_launch();
    bicg_p_kernel<<<rgrid, kVecThreads, 0, s>>>(vr, blk ? nullptr : D, skip);
    if (blk) {
      count_launch();
      bicg_block_apply_kernel<<<rgrid, kVecThreads, 0, s>>>(vr, kP, kPh, blk->B, blk->state_atom, blk->atom_off,
                                                            blk->N, blk->C, skip);
    }
    count_launch();
    bicg_matvec_kernel<<<mgrid, kMvThreads, kMvSmem, s>>>(vr, M32, lay.stride, kPh, kV, groups, chunk, skip);
    count_launch();
    bicg_dot_rv_kernel<<<rgrid, kVecThreads, 0, s>>>(vr, skip);
    count_launch();
    bicg_alpha_kernel<<<sblocks, sthreads, 0, s>>>(v, skip);
    count_launch();
    bicg_s_kernel<<<rgrid, kVecThreads, 0, s>>>(vr, blk ? nullptr : D, skip);
    if (blk) {
      count_launch();
      bicg_block_apply_kernel<<<rgrid, kVecThreads, 0, s>>>(vr, kR, kSh, blk->B, blk->state_atom, blk->atom_off,
                                                            blk->N, blk->C, skip);
    }
    count_launch();
    bicg_matvec_kernel<<<mgrid, kMvThreads, kMvSmem, s>>>(vr, M32, lay.stride, kSh, kT, groups, chunk, skip);
    count_launch();
    bicg_dot_ts_kernel<<<rgrid, kVecThreads, 0, s>>>(vr, skip);
    count_launch();
    bicg_omega_kernel<<<sblocks, sthreads, 0, s>>>(v, skip);
    count_launch();
    bicg_xr_kernel<<<rgrid, kVecThreads, 0, s>>>(vr, skip);
    const bool poll_now = (it % std::max(poll, 1)) == 0 || it == max_iter;
    if (poll_now) cudaMemsetAsync(w.active, 0, sizeof(int), s);
    count_launch();
    if (compact)
      bicg_check_compact_kernel<<<1, cthreads, 0, s>>>(v, tol * tol, it, w.iters, w.active, skip, w.act);
    else
      bicg_check_kernel<<<bblocks, sthreads, 0, s>>>(v, tol * tol, it, w.iters, w.active, skip);
    if (poll_now) {
      cudaError_t e = cudaMemcpyAsync(&running, w.active, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return e;
    }
  }
  count_launch();
  bicg_finish_kernel<<<vgrid, kVecThreads, 0, s>>>(v, M32, lay.stride, failed, skip);
  return cudaGetLastError();
}

}  // namespace rfx
