// Refinement residual R = B - A X on the 5th-generation tensor cores.
//
// The refinement of the FP32 LU form needs r = b - A x to well below its
// stopping tolerance times |A| |x| (A and B are stored as hi/lo FP32 pairs
// exact to 2^-48, X in FP64).  This residual reaches about 2^-48 of
// ||a_row||_1 ||x||_inf (each digit cut is exact to 2^-48 of its power-of-two
// scale); componentwise, where a row's large entries meet small entries of x,
// about 2^-43 of sum |a| |x|.  The products are made exact on the bf16 tensor
// path by an error-free splitting after Ozaki, Ogita, Oishi and Rump,
// "Error-free transformations of matrix multiplication by using fast routines
// of matrix multiplication and its applications", Numer. Algorithms 59 (2012):
//
//   * every entry of A is scaled by a power of two shared by its row over a
//     32-column segment, and every column of X by a power of two shared by the
//     column, so that all scaled values lie in (-1, 1);
//   * each scaled value is cut into six signed digits t_1 .. t_6 of weights
//     2^-7, 2^-15, ..., 2^-47 (integers, |t| <= 128, exact in bf16);
//   * a digit product is an integer below 2^14, so a tcgen05.mma kind::f16
//     with FP32 accumulation sums the products of one level s = i + j (digit i
//     of A times digit j of X) without rounding as long as every partial sum
//     stays below 2^24: at most 6 pairs x 2 real products x 32 columns x 2^14
//     = 2^22.6 per level and segment.
//
// Levels 2 .. 8 are kept (26 digit pairs; a dropped pair weighs at most 2^-54
// of the scales).  After each segment the seven exact level sums are combined
// in double-float on the FP32 pipes, scaled by the row's power of two and added
// to a double-float accumulator per output; the column's power of two is
// applied at the end.
//
// One pass per 16 right-hand sides; per pass one CTA per (128 rows, system), 10 warps:
//   warps 0-7  load their rows of A (two threads per row, 16 columns each), cut
//              the digits into 12 bf16 planes (re / im x 6 digits; 128 rows x
//              16 columns, K-major, 32-byte swizzle) of a three-stage ring,
//              and after the MMAs of a segment read its level sums from TMEM;
//   warp 8     bulk-copies the digit slots of X (cut once per residual by
//              residual_x_image_kernel) into the stage;
//   warp 9     issues per stage one MMA per A plane: digit i of A against the
//              adjacent X slots of digits 1 .. min(6, 8 - i) (N = 32 per slot:
//              [re | im] of 16 columns) into the adjacent level accumulators.
// Complex products: Cr = Ar Xr - Ai Xi, Ci = Ar Xi + Ai Xr through the slots
// P = [Xr | Xi] (against Ar) and Q = [-Xi | Xr] (against Ai).  Every wait is
// bounded; a timeout sets the error flag (the caller then re-solves with the
// FP64 LU) and the CTA drains its copies and MMAs and frees TMEM.
#include <cuda_runtime.h>

#include <cstdint>

#include "batched_lu.cuh"
#include "cplx.cuh"

namespace rfx {
namespace {

constexpr int kRtRows = 128;    // rows per CTA (TMEM lanes, MMA M)
constexpr int kRtK = 16;        // A columns per stage (one bf16 MMA K step)
constexpr int kRtSeg = 32;      // columns per row scale and per exact accumulation (two stages)
constexpr int kRtDigits = 6;
constexpr int kRtStages = 3;
constexpr int kRtWorkerWarps = 8;
constexpr int kRtThreads = 32 * (kRtWorkerWarps + 2);
constexpr int kRtCols = 16;                               // right-hand sides per pass
constexpr int kRtAPlane = kRtRows * kRtK * 2;             // 4 KB: 128 rows of 16 bf16
constexpr int kRtA = 2 * kRtDigits * kRtAPlane;           // 48 KB
constexpr int kRtSlot = 2 * kRtCols * kRtK * 2;           // 1 KB: 32 rows of 16 bf16
constexpr int kRtImage = 2 * kRtDigits * kRtSlot;         // 12 KB: Q_1 .. Q_6, P_1 .. P_6
constexpr int kRtStage = kRtA + kRtImage + kRtSlot;       // + a zero slot after P_6
constexpr int kRtLevels = 7;                              // s = 2 .. 8
constexpr uint32_t kRtBufCols = 256, kRtTmemCols = 512;   // two accumulator sets of 7 x 32 columns
constexpr int kRtSigBufs = 3;
constexpr int kRtMetaOff = kRtStages * kRtStage;          // row scales, then barriers
constexpr int kRtBarOff = kRtMetaOff + kRtSigBufs * kRtRows * 4;
constexpr int kRtSmem = kRtBarOff + 256 + 1024;           // + alignment of the base to 1 KB
static_assert(kRtStage % 1024 == 0, "stages stay 1 KB aligned");
constexpr float kRtMagic = 12582912.0f;  // 1.5 x 2^23: (x + kRtMagic) - kRtMagic rounds |x| < 2^22 to an integer

// barriers: full[3] (8 worker warps), xfull[3] (the X copy), empty[3] (MMA
// commit), accfull[2] (MMA commit), accempty[2] (8 worker warps), drain
enum : int { kBarFull = 0, kBarXFull = 3, kBarEmpty = 6, kBarAccFull = 9, kBarAccEmpty = 11, kBarDrain = 13 };

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// Byte offset of the 16-byte chunk `chunk` (0, 1) of row `row` in a K-major
// tile of 32-byte rows with the 32-byte swizzle: chunk XOR (row / 4) % 2.
__device__ __forceinline__ int sw32(int row, int chunk) { return row * 32 + ((chunk ^ ((row >> 2) & 1)) << 4); }
// start >> 4, LBO 1 (unused when swizzled), SBO = 8 rows x 32 B, version 1, 32-byte swizzle (layout 6)
__device__ __forceinline__ uint64_t desc_sw32(uint32_t saddr) {
  return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t(1) << 16) | (uint64_t(256 >> 4) << 32) | (uint64_t(1) << 46) |
         (uint64_t(6) << 61);
}
// kind::f16, D = F32, A = B = BF16, both K-major, M = 128, N columns
__device__ __forceinline__ uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(kRtRows >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded role wait (poll budget, or 1 s); gives up early once the CTA's abort
// flag is up, and a timeout raises that flag and the error flag.
__device__ __forceinline__ bool role_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* err,
                                          long long polls) {
  const uint64_t t0 = global_ns();
  for (long long it = 0; it < polls; ++it) {
    if (mbar_try(bar, parity)) return true;
    if ((it & 255) == 255) {
      if (*abort_flag) return false;
      if (global_ns() - t0 > 1000000000ull) break;
    }
  }
  *abort_flag = 1;
  atomicExch(err, 1);
  return false;
}
// Drain wait for work this thread issued itself (full default budget, no abort exit).
__device__ __forceinline__ void drain_wait(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = global_ns();
  for (long long it = 0; it < kTcWaitPolls; ++it)
    if (mbar_try(bar, parity) || ((it & 1023) == 1023 && global_ns() - t0 > 1000000000ull)) return;
}
// OR of v over the 256 worker threads (named barrier 1 with reduction)
__device__ __forceinline__ bool workers_any(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, 1, %2, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
      : "=r"(r)
      : "r"(uint32_t(v)), "n"(32 * kRtWorkerWarps)
      : "memory");
  return r != 0;
}

// Six digits of h + l (|h + l| < 1, l the FP32 remainder of h): integers t_k,
// |t_k| <= 128, with h + l = sum_k t_k 2^(-7 - 8k) to within 2^-48.  Each digit
// rounds the running remainder (rh + l, rh exact) to the digit's grid; rh -=
// t_k 2^(-7 - 8k) is exact because t_k 2^(-7 - 8k) lies within a digit of rh + l.
__device__ __forceinline__ void cut_digits(float h, float l, float (&t)[kRtDigits]) {
  float rh = h;
#pragma unroll
  for (int k = 0; k < kRtDigits; ++k) {
    const float w = __uint_as_float(uint32_t(127 + 7 + 8 * k) << 23);
    const float wi = __uint_as_float(uint32_t(127 - 7 - 8 * k) << 23);
    const float s = __fadd_rn(rh, l);
    const float d = __fsub_rn(__fmaf_rn(s, w, kRtMagic), kRtMagic);
    rh = __fmaf_rn(-d, wi, rh);
    t[k] = d;
  }
}
// two small integers (exact in bf16: the high half of their FP32 patterns) as one bf16x2, a first
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  return __byte_perm(__float_as_uint(a), __float_as_uint(b), 0x7632);
}
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Digit slots of X for the residual, once per residual: per system, per
// 16-row stage g of X, 12 slots of 32 rows x 16 bf16 (the K-major, 32-byte
// swizzled layout of the MMA's B operand): Q_j = [-Xi | Xr] then P_j = [Xr | Xi]
// for digits j = 1 .. 6, row c (c < 16) of the left half holding column c.
// The column scales tau_c (powers of two, max |x| < tau_c) follow the slots.
__global__ void __launch_bounds__(512) residual_x_image_kernel(BatchLayout lay, const double2* __restrict__ X64,
                                                                uint8_t* __restrict__ ximg, float* __restrict__ tau,
                                                                int nseg, int c0, const int* skip, int* err) {
  const int b = blockIdx.x;
  if (skip && skip[b]) return;
  __shared__ unsigned long long cmax[kRtCols];
  __shared__ double tinv[kRtCols];
  // columns c0 .. c0 + mc - 1 of X in this pass
  const int n = lay.n, mc = min(kRtCols, lay.m - c0), tid = threadIdx.x;
  const double2* X = X64 + size_t(b) * lay.lda * lay.m + size_t(lay.lda) * c0;
  if (tid < kRtCols) cmax[tid] = 0ull;
  __syncthreads();
  for (int idx = tid; idx < n * mc; idx += blockDim.x) {
    const int r = idx % n, c = idx / n;
    const double2 v = X[size_t(r) + size_t(lay.lda) * c];
    const double a = fmax(fabs(v.x), fabs(v.y));
    // non-negative doubles order as their bit patterns; a NaN (above +inf) is caught below
    atomicMax(&cmax[c], static_cast<unsigned long long>(__double_as_longlong(a)));
  }
  __syncthreads();
  if (tid < kRtCols) {
    const double mx = __longlong_as_double(static_cast<long long>(cmax[tid]));
    int ex = 0;
    if (mx > 0.0) frexp(mx, &ex);  // mx in [2^(ex - 1), 2^ex)
    if (!(mx <= 1.0e30) || ex < -100) {  // non-finite or out of the float scale range: leave it to the FP64 LU
      atomicExch(err, 1);
      ex = 0;
    }
    tinv[tid] = ldexp(1.0, -ex);
    tau[size_t(b) * kRtCols + tid] = ldexpf(1.0f, ex);
  }
  __syncthreads();
  uint8_t* const out = ximg + size_t(b) * size_t(2 * nseg) * kRtImage;
  for (int it = tid; it < 2 * nseg * kRtCols * 2; it += blockDim.x) {
    const int ch = it & 1, c = (it >> 1) % kRtCols, g = it / (2 * kRtCols);
    uint32_t pr[kRtDigits][4], pi[kRtDigits][4], ni[kRtDigits][4];
#pragma unroll
    for (int u = 0; u < 8; u += 2) {
      float dr[2][kRtDigits], di[2][kRtDigits];
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        const int k = g * kRtK + ch * 8 + u + v;
        double2 x = (c < mc && k < n) ? X[size_t(k) + size_t(lay.lda) * c] : make_double2(0.0, 0.0);
        x.x *= tinv[c];
        x.y *= tinv[c];
        const float rh = float(x.x), ih = float(x.y);
        cut_digits(rh, float(x.x - double(rh)), dr[v]);
        cut_digits(ih, float(x.y - double(ih)), di[v]);
      }
#pragma unroll
      for (int i = 0; i < kRtDigits; ++i) {
        pr[i][u / 2] = pack_bf16(dr[0][i], dr[1][i]);
        pi[i][u / 2] = pack_bf16(di[0][i], di[1][i]);
        ni[i][u / 2] = pack_bf16(-di[0][i], -di[1][i]);
      }
    }
    uint8_t* const st = out + size_t(g) * kRtImage;
#pragma unroll
    for (int i = 0; i < kRtDigits; ++i) {
      uint8_t* const q = st + i * kRtSlot;
      uint8_t* const p = st + (kRtDigits + i) * kRtSlot;
      *reinterpret_cast<uint4*>(q + sw32(c, ch)) = make_uint4(ni[i][0], ni[i][1], ni[i][2], ni[i][3]);
      *reinterpret_cast<uint4*>(q + sw32(kRtCols + c, ch)) = make_uint4(pr[i][0], pr[i][1], pr[i][2], pr[i][3]);
      *reinterpret_cast<uint4*>(p + sw32(c, ch)) = make_uint4(pr[i][0], pr[i][1], pr[i][2], pr[i][3]);
      *reinterpret_cast<uint4*>(p + sw32(kRtCols + c, ch)) = make_uint4(pi[i][0], pi[i][1], pi[i][2], pi[i][3]);
    }
  }
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* p, double v) {
  atomicMax(p, static_cast<unsigned long long>(__double_as_longlong(v)));
}

__global__ void __launch_bounds__(kRtThreads, 1)
    residual_tc_kernel(BatchLayout lay, const float4* __restrict__ Ms, const uint8_t* __restrict__ ximg,
                       const float* __restrict__ tau, int nseg, int c0, double2* __restrict__ R, unsigned long long* rnorm,
                       unsigned long long* bnorm, const int* skip, int* err, long long polls) {
  const int b = blockIdx.y;
  // decided once for the whole CTA (another CTA may raise the error flag meanwhile), before any tensor
  // memory is taken
  __shared__ int go;
  if (threadIdx.x == 0) go = !((skip && skip[b]) || *reinterpret_cast<volatile int*>(err));
  __syncthreads();
  if (!go) return;
  extern __shared__ uint8_t rt_sm[];
  const uint32_t raw = smem_u32(rt_sm);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t* const gbase = rt_sm + (sbase - raw);
  float* const sig = reinterpret_cast<float*>(gbase + kRtMetaOff);
  uint8_t* const meta = gbase + kRtBarOff;
  auto bar = [&](int i) { return smem_u32(meta + 8 * i); };
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(meta + 128);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(meta + 132);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // right-hand sides c0 .. c0 + mc - 1 in this pass
  const int n = lay.n, mc = min(kRtCols, lay.m - c0), r0 = blockIdx.x * kRtRows;
  const float4* A = Ms + size_t(b) * lay.stride;

  if (warp == kRtWorkerWarps + 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kRtTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kRtStages; ++i) {
      mbar_init(bar(kBarFull + i), kRtWorkerWarps);
      mbar_init(bar(kBarXFull + i), 1);
      mbar_init(bar(kBarEmpty + i), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(bar(kBarAccFull + i), 1);
      mbar_init(bar(kBarAccEmpty + i), kRtWorkerWarps);
    }
    mbar_init(bar(kBarDrain), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the zero slot after P_6 of every stage (digit 1 of A reaches level 8 through it)
  for (int i = tid; i < kRtStages * kRtSlot / 16; i += kRtThreads) {
    const int st = i / (kRtSlot / 16), off = (i % (kRtSlot / 16)) * 16;
    *reinterpret_cast<uint4*>(gbase + st * kRtStage + kRtA + kRtImage + off) = make_uint4(0u, 0u, 0u, 0u);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp < kRtWorkerWarps) {
    const int quad = warp & 3, hw = warp >> 2;
    // cutting: row 32 quad + 16 hw + lane / 2 of the tile, columns 16 h .. 16 h + 15 of each segment
    const int srow = 32 * quad + 16 * hw + (lane >> 1), h = lane & 1;
    const int grow = r0 + srow;
    const bool srow_ok = grow < n;
    // level sums: row 32 quad + lane (this warp's TMEM lanes), complex columns 8 hw .. 8 hw + 7
    const int erow = 32 * quad + lane;
    float4 a[kRtK];
    auto load = [&](int seg) {
      const int k0 = seg * kRtSeg + h * kRtK;
#pragma unroll
      for (int kk = 0; kk < kRtK; ++kk)
        a[kk] = (srow_ok && k0 + kk < n) ? __ldcs(A + size_t(grow) + size_t(lay.lda) * (k0 + kk))
                                         : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    df acc_r[8], acc_i[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) acc_r[u] = acc_i[u] = {0.f, 0.f};
    auto ld8 = [](uint32_t addr, uint32_t (&o)[8]) {
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                   : "=r"(o[0]), "=r"(o[1]), "=r"(o[2]), "=r"(o[3]), "=r"(o[4]), "=r"(o[5]), "=r"(o[6]), "=r"(o[7])
                   : "r"(addr));
    };
    // add segment q's level sums into the accumulators (warp-uniform result)
    auto extract = [&](int q) -> bool {
      const int buf = q & 1;
      const bool ready = role_wait(bar(kBarAccFull + buf), uint32_t((q >> 1) & 1), abort_flag, err, polls);
      if (!__all_sync(0xffffffffu, ready)) return false;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // one unit of level 2 is sigma_row tau_c 2^-14; tau_c is applied at the end
      const float sc = sig[(q % kRtSigBufs) * kRtRows + erow] * 0x1p-14f;
      const uint32_t base = tmem + (uint32_t(32 * quad) << 16) + uint32_t(buf) * kRtBufCols + uint32_t(8 * hw);
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        uint32_t L[kRtLevels][8];
#pragma unroll
        for (int s = 0; s < kRtLevels; ++s) ld8(base + uint32_t(32 * s + 16 * part), L[s]);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          auto lv = [&](int s) { return __uint_as_float(L[s][u]); };
          // levels 8 and 7 in FP32 (far below the others), then levels 6 .. 2 in double-float
          const float t = __fmaf_rn(lv(5), 0x1p-40f, __fmul_rn(lv(6), 0x1p-48f));
          float hh, ll;
          two_sum(__fmul_rn(lv(4), 0x1p-32f), t, hh, ll);
#pragma unroll
          for (int s = 3; s >= 0; --s) {
            float e;
            two_sum(__fmul_rn(lv(s), __uint_as_float(uint32_t(127 - 8 * s) << 23)), hh, hh, e);
            ll = __fadd_rn(ll, e);
          }
          hh = __fmul_rn(hh, sc);
          ll = __fmul_rn(ll, sc);
          df& acc = part ? acc_i[u] : acc_r[u];
          float s1, e1;
          two_sum(acc.hi, hh, s1, e1);
          e1 = __fadd_rn(__fadd_rn(e1, acc.lo), ll);
          acc.hi = __fadd_rn(s1, e1);
          acc.lo = __fsub_rn(e1, __fsub_rn(acc.hi, s1));
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(bar(kBarAccEmpty + buf));
      return true;
    };

    load(0);
    bool failed = false;
    for (int seg = 0; seg < nseg; ++seg) {
      const int g0 = 2 * seg;
      bool ok = role_wait(bar(kBarEmpty + g0 % kRtStages), uint32_t(((g0 / kRtStages) & 1) ^ 1), abort_flag, err,
                          polls) &&
                role_wait(bar(kBarEmpty + (g0 + 1) % kRtStages), uint32_t((((g0 + 1) / kRtStages) & 1) ^ 1),
                          abort_flag, err, polls);
      ok = __all_sync(0xffffffffu, ok);
      if (ok) {
        // the row's power of two over this segment (both threads of the row), from the hi parts
        float mx = 0.f;
#pragma unroll
        for (int kk = 0; kk < kRtK; ++kk) mx = fmaxf(mx, fmaxf(fabsf(a[kk].x), fabsf(a[kk].y)));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
        const uint32_t e = min(max((__float_as_uint(mx) >> 23) & 0xFFu, 1u), 252u);
        const float sinv = __uint_as_float((253u - e) << 23);  // 2^-(E + 1), mx < 2^(E + 1)
        if (h == 0) sig[(seg % kRtSigBufs) * kRtRows + srow] = __uint_as_float((e + 1u) << 23);
        uint8_t* const sA = gbase + ((g0 + h) % kRtStages) * kRtStage;
#pragma unroll
        for (int ch = 0; ch < 2; ++ch) {
          uint32_t q[2 * kRtDigits][4];
#pragma unroll
          for (int u = 0; u < 8; u += 2) {
            const float4 v0 = a[8 * ch + u], v1 = a[8 * ch + u + 1];
            float r0d[kRtDigits], i0d[kRtDigits], r1d[kRtDigits], i1d[kRtDigits];
            cut_digits(v0.x * sinv, v0.z * sinv, r0d);
            cut_digits(v0.y * sinv, v0.w * sinv, i0d);
            cut_digits(v1.x * sinv, v1.z * sinv, r1d);
            cut_digits(v1.y * sinv, v1.w * sinv, i1d);
#pragma unroll
            for (int i = 0; i < kRtDigits; ++i) {
              q[2 * i][u / 2] = pack_bf16(r0d[i], r1d[i]);
              q[2 * i + 1][u / 2] = pack_bf16(i0d[i], i1d[i]);
            }
          }
          const int off = sw32(srow, ch);
#pragma unroll
          for (int p = 0; p < 2 * kRtDigits; ++p)
            *reinterpret_cast<uint4*>(sA + p * kRtAPlane + off) = make_uint4(q[p][0], q[p][1], q[p][2], q[p][3]);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the planes are read by the tensor cores
      __syncwarp();
      if (ok && lane == 0) {
        mbar_arrive(bar(kBarFull + g0 % kRtStages));
        mbar_arrive(bar(kBarFull + (g0 + 1) % kRtStages));
      }
      if (seg + 1 < nseg) load(seg + 1);
      // the worker threads agree whether to go on; the row scales of this segment are now visible to all
      if (workers_any(!ok || *abort_flag != 0)) {
        failed = true;
        break;
      }
      if (seg >= 1 && !extract(seg - 1)) {
        *abort_flag = 1;
        atomicExch(err, 1);
      }
    }
    if (!failed) failed = !extract(nseg - 1);
    if (!failed) {
      const int row = r0 + erow;
      double rmax = 0.0, bmax = 0.0;
      if (row < n) {
        double2* Rb = R + size_t(b) * lay.lda * lay.m + size_t(lay.lda) * c0;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int c = 8 * hw + u;
          if (c >= mc) continue;
          const double t = double(tau[size_t(b) * kRtCols + c]);
          const double ax = (double(acc_r[u].hi) + double(acc_r[u].lo)) * t;
          const double ay = (double(acc_i[u].hi) + double(acc_i[u].lo)) * t;
          const double2 bv = join_hi_lo(A[size_t(row) + size_t(lay.lda) * (n + c0 + c)]);
          const double2 rv = make_double2(bv.x - ax, bv.y - ay);
          Rb[size_t(row) + size_t(lay.lda) * c] = rv;
          rmax = fmax(rmax, cabs1(rv));
          bmax = fmax(bmax, cabs1(bv));
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        rmax = fmax(rmax, __shfl_down_sync(0xffffffffu, rmax, off));
        bmax = fmax(bmax, __shfl_down_sync(0xffffffffu, bmax, off));
      }
      if (lane == 0) {
        atomic_max_nonneg(rnorm + b, rmax);
        atomic_max_nonneg(bnorm + b, bmax);
      }
    }
  } else if (warp == kRtWorkerWarps && lane == 0) {
    // ---- X digit slots: one bulk copy per stage ----
    const uint8_t* xb = ximg + size_t(b) * size_t(2 * nseg) * kRtImage;
    int issued = 0;
    bool ok = true;
    for (int g = 0; g < 2 * nseg; ++g) {
      const int st = g % kRtStages;
      ok = role_wait(bar(kBarEmpty + st), uint32_t(((g / kRtStages) & 1) ^ 1), abort_flag, err, polls);
      if (!ok) break;
      mbar_expect_tx(bar(kBarXFull + st), kRtImage);
      bulk_copy(sbase + uint32_t(st * kRtStage + kRtA), xb + size_t(g) * kRtImage, kRtImage, bar(kBarXFull + st));
      issued = g + 1;
    }
    // copies still in flight (the MMA role may have given up on them) land before the CTA exits
    for (int g = max(0, issued - kRtStages); g < issued; ++g)
      drain_wait(bar(kBarXFull + g % kRtStages), uint32_t((g / kRtStages) & 1));
  } else if (warp == kRtWorkerWarps + 1 && lane == 0) {
    // ---- MMA issuer ----
    bool issued = false, ok = true;
    for (int seg = 0; seg < nseg && ok; ++seg) {
      const int buf = seg & 1;
      ok = role_wait(bar(kBarAccEmpty + buf), uint32_t(((seg >> 1) & 1) ^ 1), abort_flag, err, polls);
      for (int hs = 0; hs < 2 && ok; ++hs) {
        const int g = 2 * seg + hs, st = g % kRtStages;
        const uint32_t ph = uint32_t((g / kRtStages) & 1);
        ok = role_wait(bar(kBarFull + st), ph, abort_flag, err, polls) &&
             role_wait(bar(kBarXFull + st), ph, abort_flag, err, polls);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t sA = sbase + uint32_t(st * kRtStage), sQ = sA + uint32_t(kRtA),
                       sP = sQ + uint32_t(kRtDigits * kRtSlot);
        const uint32_t d0 = tmem + uint32_t(buf) * kRtBufCols;
#pragma unroll
        for (int i = 0; i < kRtDigits; ++i) {
          // digit i + 1 of A against X digits 1 .. jn: levels i + 2 .. i + 1 + jn at TMEM columns 32 i ..
          const int jn = min(kRtDigits, kRtDigits + 1 - i);
          const uint32_t d = d0 + uint32_t(32 * i);
          // digit 1 of Ar also takes the zero slot, so that the segment's first MMA (which overwrites)
          // covers every level 2 .. 8
          const int nre = i == 0 ? jn + 1 : jn;
          mma_bf16(d, desc_sw32(sA + uint32_t(2 * i * kRtAPlane)), desc_sw32(sP), idesc_bf16(32 * nre),
                   (hs == 0 && i == 0) ? 0u : 1u);
          mma_bf16(d, desc_sw32(sA + uint32_t((2 * i + 1) * kRtAPlane)), desc_sw32(sQ), idesc_bf16(32 * jn), 1u);
        }
        issued = true;
        mma_commit(bar(kBarEmpty + st));  // the stage is free once these MMAs have read it
      }
      if (ok) mma_commit(bar(kBarAccFull + buf));
    }
    if (issued) {  // every MMA of this CTA has completed before the tensor memory is freed
      mma_commit(bar(kBarDrain));
      drain_wait(bar(kBarDrain), 0u);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kRtWorkerWarps + 1) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kRtTmemCols));
  }
}

}  // namespace

size_t residual_tc_image_bytes(int n, int batch) {
  const int nseg = (n + kRtSeg - 1) / kRtSeg;
  return size_t(batch) * size_t(2 * nseg) * kRtImage + size_t(batch) * kRtCols * sizeof(float);
}

bool launch_residual_tc(const BatchLayout& lay, int batch, const float4* Ms, const double2* X64, const ResidualTc& tc,
                        double2* R, unsigned long long* rnorm_bits, unsigned long long* bnorm_bits, const int* skip,
                        cudaStream_t s) {
  if (lay.m < 1 || !tc.images || !tc.err || residual_tc_image_bytes(lay.n, batch) > tc.bytes) return false;
  if (ensure_smem_limit(reinterpret_cast<const void*>(residual_tc_kernel), size_t(kRtSmem)) != cudaSuccess)
    return false;
  const int nseg = (lay.n + kRtSeg - 1) / kRtSeg;
  float* tau = reinterpret_cast<float*>(tc.images + size_t(batch) * size_t(2 * nseg) * kRtImage);
  dim3 grid(unsigned((lay.n + kRtRows - 1) / kRtRows), unsigned(batch));
  // one pass per 16 right-hand sides (the passes reuse the scratch, one after the other on the stream);
  // each pass reads A again, which costs far less than the double-float products it replaces
  for (int c0 = 0; c0 < lay.m; c0 += kRtCols) {
    count_launch();
    residual_x_image_kernel<<<unsigned(batch), 512, 0, s>>>(lay, X64, tc.images, tau, nseg, c0, skip, tc.err);
    count_launch();
    residual_tc_kernel<<<grid, kRtThreads, kRtSmem, s>>>(lay, Ms, tc.images, tau, nseg, c0, R, rnorm_bits,
                                                          bnorm_bits, skip, tc.err, tc.polls);
  }
  return true;
}

}  // namespace rfx
