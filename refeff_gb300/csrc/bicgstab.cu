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
#include <type_traits>
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

// ---------------------------------------------------------------------------
// Tensor-core product (tcgen05, split TF32): the same Y = A X, slices and
// partial products as bicg_matvec_kernel, with the complex products on the
// 5th-generation tensor cores.  Each of the four operand warps owns one row of
// the CTA's 128-row tile: it loads the row's 16 A entries of a slab with
// coalesced global loads (two slabs ahead in registers), splits them into TF32
// hi / lo parts and stores the four real planes (re hi, re lo, im hi, im lo)
// in the K-major 64-byte-swizzled UMMA layout; the X slab becomes six slots
// (-im hi, re hi, im hi, -im lo, re lo, im lo) in an order where each adjacent
// pair is one 2N-row B operand.  One thread issues 6 MMAs of 2N columns per K
// step of 8 into the adjacent TMEM accumulators [Yr | Yi] (N = 16 or 32):
//     Yr += Ar Xr + Ai (-Xi)        Yi += Ar Xi + Ai Xr,
// each real product hi*hi + hi*lo + lo*hi, one A plane against [Xr | Xi] or
// [-Xi | Xr] at a time (half the MMA instructions of N-column products, as
// many multiply-adds).  Two plane stages let the operand
// warps fill one while the MMAs read the other.  Every wait is bounded; a
// timeout sets *err (the solve then hands its matrices to the LU) and the
// CTA drains its MMAs and frees its tensor memory before it returns.
constexpr int kTcRows = 128, kTcK = 16, kTcThreads = 160, kTcStages = 2;
constexpr long long kTcBicgPolls = 1LL << 26;  // poll budget of each wait (about 1 s is the other bound)
constexpr int kTcAPlane = kTcRows * 64;  // 8 KB: 128 rows of 16 TF32 values

// k3M: the three-product form P1 = Ar Xr, P2 = Ai Xi, P3 = (Ar + Ai)(Xr + Xi),
// Yr = P1 - P2, Yi = P3 - P1 - P2 (9 MMAs per K step; six A planes, three
// accumulators); otherwise the four products above (12 MMAs, two accumulators).
template <int N, bool k3M = false> struct TcMv {
  static constexpr int kAPlanes = k3M ? 6 : 4;
  static constexpr int kA = kAPlanes * kTcAPlane;
  static constexpr int kBPlane = N * 64;
  static constexpr int kB = 6 * kBPlane;
  static constexpr int kStage = kA + kB;
  static constexpr int kBars = 128;        // barriers, TMEM slot, abort flag
  static constexpr int kSmem = kTcStages * kStage + kBars + 1024;
  // TMEM columns (a power of two >= 32): Yr, Yi, or P1, P2, P3
  static constexpr uint32_t kCols = k3M ? (3 * N <= 64 ? 64u : 128u) : 2u * N;
  // kind::tf32, D = F32, A = B = TF32, both K-major, M = 128; N columns per MMA for the three-product
  // form, 2N (one A plane against two adjacent B slots) for the four-product form
  static constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t((k3M ? N : 2 * N) >> 3) << 17) |
                                     (uint32_t(kTcRows >> 4) << 24);
};

__device__ __forceinline__ uint32_t tc_smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint32_t tc_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
// hi / lo TF32 parts of the real and imaginary parts
__device__ __forceinline__ void tc_split(float2 v, uint32_t out[4]) {
  const uint32_t rh = tc_tf32(v.x), ih = tc_tf32(v.y);
  out[0] = rh;
  out[1] = tc_tf32(v.x - __uint_as_float(rh));
  out[2] = ih;
  out[3] = tc_tf32(v.y - __uint_as_float(ih));
}
// Byte offset of (row, k), k < 16, in a K-major tile of 64-byte rows with the
// 64-byte swizzle: the 16-byte chunk index XOR (row / 2) % 4.
__device__ __forceinline__ int tc_sw64(int row, int k) {
  return row * 64 + ((((k >> 2) ^ ((row >> 1) & 3))) << 4) + ((k & 3) << 2);
}
// start >> 4, LBO 1 (unused when swizzled), SBO = 8 rows x 64 B, version 1, 64-byte swizzle (layout 4)
__device__ __forceinline__ uint64_t tc_desc64(uint32_t saddr) {
  return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t(1) << 16) | (uint64_t(512 >> 4) << 32) | (uint64_t(1) << 46) |
         (uint64_t(4) << 61);
}
template <uint32_t kIdesc>
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}
__device__ __forceinline__ void tc_bar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void tc_bar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ uint64_t tc_now() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool tc_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait (poll budget, or 1 s); a timeout raises the CTA's abort flag and *err.
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* err,
                                        long long polls) {
  const uint64_t t0 = tc_now();
  for (long long it = 0; it < polls; ++it) {
    if (tc_try(bar, parity)) return true;
    if ((it & 255) == 255) {
      if (*abort_flag) return false;
      if (tc_now() - t0 > 1000000000ull) break;
    }
  }
  *abort_flag = 1;
  atomicExch(err, 1);
  return false;
}

template <int N, bool k3M>
__global__ void __launch_bounds__(kTcThreads) bicg_tc_matvec_kernel(View w, const float2* __restrict__ M32,
                                                                     size_t stride, int src, int dst, int kchunk,
                                                                     const int* skip, int* err, long long polls) {
  using L = TcMv<N, k3M>;
  const int b = w.matrix();
  // decided once for the whole CTA (another CTA may raise the error flag meanwhile), before any tensor
  // memory is taken; a raised error skips the product
  __shared__ int go;
  if (threadIdx.x == 0) go = !(b < 0 || (skip && skip[b]) || w.done[b] || *reinterpret_cast<volatile int*>(err));
  __syncthreads();
  if (!go) return;
  extern __shared__ uint8_t tsm[];
  const uint32_t raw = tc_smem_u32(tsm);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t* const gbase = tsm + (sbase - raw);
  uint8_t* const meta = gbase + kTcStages * L::kStage;
  // barriers: full[2] (128 operand threads), empty[2] (commit), acc (commit), drain (commit)
  auto bar = [&](int i) { return tc_smem_u32(meta + 8 * i); };
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(meta + 64);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(meta + 68);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int slice = blockIdx.z;
  const int n = w.n, r0 = blockIdx.x * kTcRows;
  const int kbeg = slice * kchunk, kend = min(n, kbeg + kchunk);
  const int slabs = (kend - kbeg + kTcK - 1) / kTcK;  // >= 1: slices start below n
  const float2* A = M32 + size_t(b) * stride;

  if (warp == 4) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem_u32(tmem_slot)),
                 "r"(L::kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kTcStages; ++i) {
      tc_bar_init(bar(i), 128);            // full: every operand thread
      tc_bar_init(bar(kTcStages + i), 1);  // empty: one commit
    }
    tc_bar_init(bar(2 * kTcStages), 1);      // accumulators complete
    tc_bar_init(bar(2 * kTcStages + 1), 1);  // drain
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp < 4) {
    // ---- operand warps: row r0 + tid of A, and the X slab ----
    const int row = r0 + tid;
    const bool row_ok = row < n;
    auto load = [&](int sl, float2 (&v)[kTcK]) {
      const int k0 = kbeg + sl * kTcK;
#pragma unroll
      for (int kk = 0; kk < kTcK; ++kk)
        v[kk] = (row_ok && sl < slabs && k0 + kk < kend) ? __ldcs(A + size_t(row) + size_t(w.lda) * (k0 + kk))
                                                          : make_float2(0.f, 0.f);
    };
    float2 v0[kTcK], v1[kTcK], v2[kTcK];
    load(0, v0);
    load(1, v1);
    bool ok = true;
    for (int sl = 0; sl < slabs && ok; ++sl) {
      load(sl + 2, v2);
      const int st = sl & 1;
      const uint32_t ph = uint32_t((sl >> 1) & 1);
      ok = tc_wait(bar(kTcStages + st), ph ^ 1u, abort_flag, err, polls);  // the MMAs of slab sl - 2 are done
      if (!ok) break;
      uint8_t* const sA = gbase + st * L::kStage;
      uint8_t* const sB = sA + L::kA;
#pragma unroll
      for (int k4 = 0; k4 < kTcK / 4; ++k4) {
        uint32_t q[L::kAPlanes][4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float2 a = v0[4 * k4 + i];
          uint32_t sv[4];
          tc_split(a, sv);
#pragma unroll
          for (int pl = 0; pl < 4; ++pl) q[pl][i] = sv[pl];
          if constexpr (k3M) {  // Ar + Ai, hi and lo
            const float sum = a.x + a.y;
            const uint32_t hi = tc_tf32(sum);
            q[4][i] = hi;
            q[5][i] = tc_tf32(sum - __uint_as_float(hi));
          }
        }
        const int off = tc_sw64(tid, 4 * k4);
#pragma unroll
        for (int pl = 0; pl < L::kAPlanes; ++pl)
          *reinterpret_cast<uint4*>(sA + pl * kTcAPlane + off) = make_uint4(q[pl][0], q[pl][1], q[pl][2], q[pl][3]);
      }
      const int k0 = kbeg + sl * kTcK;
#pragma unroll
      for (int j = 0; j < N * kTcK / 128; ++j) {
        const int e = tid + 128 * j, kk = e % kTcK, c = e / kTcK;
        const float2 x = (c < w.m && k0 + kk < kend) ? w.v(src, b, c)[k0 + kk] : make_float2(0.f, 0.f);
        uint32_t sv[4];
        tc_split(x, sv);
        const int off = tc_sw64(c, kk);
        auto put = [&](int slot, uint32_t v) { *reinterpret_cast<uint32_t*>(sB + slot * L::kBPlane + off) = v; };
        if constexpr (k3M) {  // Xr hi, Xr lo, Xi hi, Xi lo, (Xr + Xi) hi, lo
#pragma unroll
          for (int pl = 0; pl < 4; ++pl) put(pl, sv[pl]);
          const float sum = x.x + x.y;
          const uint32_t hi = tc_tf32(sum);
          put(4, hi);
          put(5, tc_tf32(sum - __uint_as_float(hi)));
        } else {
          // slots -Xi hi, Xr hi, Xi hi, -Xi lo, Xr lo, Xi lo: each adjacent pair is one 2N-row B operand
          put(0, sv[2] ^ 0x80000000u);
          put(1, sv[0]);
          put(2, sv[2]);
          put(3, sv[3] ^ 0x80000000u);
          put(4, sv[1]);
          put(5, sv[3]);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the planes are read by the tensor cores
      tc_bar_arrive(bar(st));
#pragma unroll
      for (int kk = 0; kk < kTcK; ++kk) {
        v0[kk] = v1[kk];
        v1[kk] = v2[kk];
      }
    }
    // ---- epilogue: the tile's rows of Y (or of this slice's partial product) ----
    const bool ready = ok && tc_wait(bar(2 * kTcStages), 0u, abort_flag, err, polls);
    if (__all_sync(0xffffffffu, ready)) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tr = tmem + (uint32_t(warp * 32) << 16), ti = tr + uint32_t(N);
      auto ld8 = [](uint32_t addr, uint32_t (&o)[8]) {
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                     : "=r"(o[0]), "=r"(o[1]), "=r"(o[2]), "=r"(o[3]), "=r"(o[4]), "=r"(o[5]), "=r"(o[6]), "=r"(o[7])
                     : "r"(addr));
      };
#pragma unroll
      for (int cb = 0; cb < N / 8; ++cb) {
        uint32_t yr[8], yi[8], y3[8];
        ld8(tr + uint32_t(cb * 8), yr);
        ld8(ti + uint32_t(cb * 8), yi);
        if constexpr (k3M) ld8(ti + uint32_t(N + cb * 8), y3);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row_ok) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int c = cb * 8 + j;
            if (c < w.m) {
              float2* y = slice == 0 ? w.v(dst, b, c) : w.pv(slice, b, c);
              float2 out;
              if constexpr (k3M) {  // Yr = P1 - P2, Yi = P3 - P1 - P2
                const float p1 = __uint_as_float(yr[j]), p2 = __uint_as_float(yi[j]), p3 = __uint_as_float(y3[j]);
                out = make_float2(p1 - p2, p3 - p1 - p2);
              } else {
                out = make_float2(__uint_as_float(yr[j]), __uint_as_float(yi[j]));
              }
              y[row] = out;
            }
          }
        }
      }
    }
  } else if (lane == 0) {
    // ---- MMA issuer ----
    bool issued = false, ok = true;
    for (int sl = 0; sl < slabs; ++sl) {
      const int st = sl & 1;
      ok = tc_wait(bar(st), uint32_t((sl >> 1) & 1), abort_flag, err, polls);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sA = sbase + uint32_t(st * L::kStage), sB = sA + uint32_t(L::kA);
#pragma unroll
      for (int ks = 0; ks < kTcK / 8; ++ks) {
        const uint32_t koff = uint32_t(ks * 32);
        auto ad = [&](int pl) { return tc_desc64(sA + uint32_t(pl * kTcAPlane) + koff); };
        auto bd = [&](int pl) { return tc_desc64(sB + uint32_t(pl * L::kBPlane) + koff); };
        const uint32_t a0 = (sl == 0 && ks == 0) ? 0u : 1u;
        const uint32_t tr = tmem, ti = tmem + uint32_t(N);
        if constexpr (k3M) {
          const uint32_t t3 = tmem + uint32_t(2 * N);
          // P1 = Ar Xr, P2 = Ai Xi, P3 = (Ar + Ai)(Xr + Xi), each hi*hi + hi*lo + lo*hi
          tc_mma<L::kIdesc>(tr, ad(0), bd(0), a0);
          tc_mma<L::kIdesc>(tr, ad(0), bd(1), 1u);
          tc_mma<L::kIdesc>(tr, ad(1), bd(0), 1u);
          tc_mma<L::kIdesc>(ti, ad(2), bd(2), a0);
          tc_mma<L::kIdesc>(ti, ad(2), bd(3), 1u);
          tc_mma<L::kIdesc>(ti, ad(3), bd(2), 1u);
          tc_mma<L::kIdesc>(t3, ad(4), bd(4), a0);
          tc_mma<L::kIdesc>(t3, ad(4), bd(5), 1u);
          tc_mma<L::kIdesc>(t3, ad(5), bd(4), 1u);
        } else {
          // [Yr | Yi] (2N columns) += A-plane x [left | right] B slots:
          //   Ar hi [Xr hi | Xi hi], Ar hi [Xr lo | Xi lo], Ar lo [Xr hi | Xi hi],
          //   Ai hi [-Xi hi | Xr hi], Ai hi [-Xi lo | Xr lo], Ai lo [-Xi hi | Xr hi]
          // i.e. Yr += Ar Xr + Ai (-Xi), Yi += Ar Xi + Ai Xr, each hi*hi + hi*lo + lo*hi, six MMAs
          (void)ti;
          tc_mma<L::kIdesc>(tr, ad(0), bd(1), a0);
          tc_mma<L::kIdesc>(tr, ad(0), bd(4), 1u);
          tc_mma<L::kIdesc>(tr, ad(1), bd(1), 1u);
          tc_mma<L::kIdesc>(tr, ad(2), bd(0), 1u);
          tc_mma<L::kIdesc>(tr, ad(2), bd(3), 1u);
          tc_mma<L::kIdesc>(tr, ad(3), bd(0), 1u);
        }
      }
      issued = true;
      tc_commit(bar(kTcStages + st));  // the stage is free once these MMAs have read it
    }
    if (ok) tc_commit(bar(2 * kTcStages));  // Y complete
    if (issued) {
      // every MMA of this CTA has completed before the tensor memory is freed
      tc_commit(bar(2 * kTcStages + 1));
      const uint64_t t0 = tc_now();
      for (long long it = 0; it < polls; ++it)
        if (tc_try(bar(2 * kTcStages + 1), 0u) || ((it & 1023) == 1023 && tc_now() - t0 > 1000000000ull)) break;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 4) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L::kCols));
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
__global__ void bicg_finish_kernel(View w, float2* __restrict__ M32, size_t stride, int* failed, const int* skip,
                                   const int* tc_err) {
  const int b = blockIdx.y, c = blockIdx.z;
  if (skip && skip[b]) return;
  const float2* x = w.v(kX, b, c);
  float2* out = M32 + size_t(b) * stride + size_t(w.lda) * (w.n + c);
  for (int k = 0; k < kVecRowsPerThread; ++k) {
    const int i = blockIdx.x * kVecRows + k * kVecThreads + threadIdx.x;
    if (i >= w.n) break;
    out[i] = x[i];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (w.state[size_t(b) * w.m + c] != 1 || (tc_err && *tc_err))) failed[b] = 2;
}

}  // namespace

int bicg_slices(int n, bool tensor, int* chunk) {
  int c = tensor ? kBicgTcSliceCols
                 : std::max(kMvSliceCols, ((n + kBicgMaxSplit - 1) / kBicgMaxSplit + kMvK - 1) / kMvK * kMvK);
  c = std::min(c, std::max(n, 1));
  if (chunk) *chunk = c;
  return (n + c - 1) / c;
}

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
  // the tensor-core product for up to 32 right-hand sides (N = 16 or 32 accumulator columns)
  const bool tensor = w.tensor && w.tc_err && lay.m <= 32;
  const bool n16 = lay.m <= 16, three = w.tensor == 2;
  // the four instantiations: N = 16 / 32 accumulator columns, four or three products
  auto tc_launch = [&](auto kN, auto k3, const dim3& grid, const View& view, int src, int dst, int chunk) {
    constexpr int N = decltype(kN)::value;
    constexpr bool M3 = decltype(k3)::value;
    bicg_tc_matvec_kernel<N, M3><<<grid, kTcThreads, TcMv<N, M3>::kSmem, s>>>(view, M32, lay.stride, src, dst, chunk,
                                                                              skip, w.tc_err, kTcBicgPolls);
  };
  auto tc_attr = [&](auto kN, auto k3) {
    constexpr int N = decltype(kN)::value;
    constexpr bool M3 = decltype(k3)::value;
    return cudaFuncSetAttribute(bicg_tc_matvec_kernel<N, M3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                TcMv<N, M3>::kSmem);
  };
  using I16 = std::integral_constant<int, 16>;
  using I32 = std::integral_constant<int, 32>;
  using T3 = std::true_type;
  using T4 = std::false_type;
  if (tensor) {
    const cudaError_t e = n16 ? (three ? tc_attr(I16{}, T3{}) : tc_attr(I16{}, T4{}))
                              : (three ? tc_attr(I32{}, T3{}) : tc_attr(I32{}, T4{}));
    if (e != cudaSuccess) return e;
    cudaMemsetAsync(w.tc_err, 0, sizeof(int), s);
  }
  const unsigned tc_row_blocks = unsigned((lay.n + kTcRows - 1) / kTcRows);
  // Slices of A's columns (bicg_slices): the last running matrices still fill
  // the GPU with product CTAs.  The slicing depends on n (and the product's
  // kind) alone: a matrix's arithmetic does not depend on which others share
  // its batch.
  int chunk = lay.n, nsplit = 1;
  if (w.part) nsplit = bicg_slices(lay.n, tensor, &chunk);
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
  // dst = A src over the running matrices: V = A P^ or T = A S^
  auto product = [&](unsigned rows_y, int src, int dst) {
    count_launch();
    if (tensor) {
      const dim3 tgrid(tc_row_blocks, rows_y, unsigned(nsplit));
      if (n16) {
        if (three) tc_launch(I16{}, T3{}, tgrid, vr, src, dst, chunk);
        else tc_launch(I16{}, T4{}, tgrid, vr, src, dst, chunk);
      } else {
        if (three) tc_launch(I32{}, T3{}, tgrid, vr, src, dst, chunk);
        else tc_launch(I32{}, T4{}, tgrid, vr, src, dst, chunk);
      }
    } else {
      const dim3 mgrid(unsigned(row_blocks), rows_y, unsigned(groups * nsplit));
      bicg_matvec_kernel<<<mgrid, kMvThreads, kMvSmem, s>>>(vr, M32, lay.stride, src, dst, groups, chunk, skip);
    }
  };
  int running = batch;
  for (int it = 1; it <= max_iter && running > 0; ++it) {
    vr.nsplit = nsplit;  // the dot kernels sum the slices
    const unsigned rows_y = unsigned(compact ? running : batch);
    const dim3 rgrid(vgrid.x, rows_y, vgrid.z);
    count_launch();
    bicg_p_kernel<<<rgrid, kVecThreads, 0, s>>>(vr, blk ? nullptr : D, skip);
    if (blk) {
      count_launch();
      bicg_block_apply_kernel<<<rgrid, kVecThreads, 0, s>>>(vr, kP, kPh, blk->B, blk->state_atom, blk->atom_off,
                                                            blk->N, blk->C, skip);
    }
    product(rows_y, kPh, kV);
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
    product(rows_y, kSh, kT);
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
  bicg_finish_kernel<<<vgrid, kVecThreads, 0, s>>>(v, M32, lay.stride, failed, skip, tensor ? w.tc_err : nullptr);
  return cudaGetLastError();
}

}  // namespace rfx
