// Tensor-core (tcgen05, sm_103a) trailing update of the FP32 LU:
//     C[r, c] -= sum_k A[r, k] B[k, c]      (complex, K <= 128)
// with A = L21 (rows below the block) and B = U12 (block rows, trailing
// columns); K is one 64-column block, or two when the elimination pairs them.
//
// Each complex product is formed from real TF32 MMAs with FP32 accumulation in
// tensor memory, using a two-term split x = hi + lo (hi = tf32(x), lo =
// tf32(x - hi)) and the three products hi*hi + hi*lo + lo*hi, which keeps the
// update at about FP32 accuracy:
//     Cr += Ar Br + Ai (-Bi)        Ci += Ar Bi + Ai Br
// The operands are first written by tc_split_* into tile images that are
// already in the UMMA shared-memory layout (K-major, 128-byte rows, 128-byte
// swizzle), so the update kernel moves them with plain cp.async.bulk copies
// completed on mbarriers.  The update runs as one persistent, warp-specialised
// CTA per SM over 128 x 64 complex tiles (tc_update_persistent_kernel below).
// Every wait on an mbarrier is bounded; on timeout the kernel records an error
// flag, ends every role, waits for its copies and MMAs in flight, frees its
// tensor memory and returns.
#include <cuda_runtime.h>
#include <cstdint>
#include "cplx.cuh"
#include "batched_lu.cuh"

namespace rfx {

namespace {

constexpr int BM = kTcBM;         // 128 rows per tile (MMA M)
constexpr int BN = kTcBN;         // 64 columns per tile (MMA N)
// Operand rows of kRowBytes bytes with the matching swizzle (128 or 64): with
// 64-byte rows a K chunk holds KC = 16 TF32 values per row (56 KB of planes),
// and four chunks are in flight; 128-byte rows (112 KB chunks, two in flight)
// measured 2% slower with the paired-N MMAs (and faster before them).
constexpr int kRowBytes = 64;
constexpr int KC = kRowBytes / 4;          // K elements per chunk
constexpr int A_PLANE = BM * kRowBytes;    // bytes per A plane per chunk (16 KB)
constexpr int B_PLANE = BN * kRowBytes;    // bytes per B plane per chunk (8 KB)
constexpr int A_PLANES = 4;       // re_hi, re_lo, im_hi, im_lo
// B slots -im_hi, re_hi, im_hi, -im_lo, re_lo, im_lo: each adjacent pair is one 2 BN-row B operand
constexpr int B_PLANES = 6;
constexpr int SMEM_OPS = A_PLANES * A_PLANE + B_PLANES * B_PLANE;  // 112 KB
constexpr long long kWaitLimit = kTcWaitPolls;  // drains of copies and MMAs in flight
constexpr int kChunks = kTcKMax / KC;  // K chunks per tile image (K up to 128)

__device__ __forceinline__ uint32_t tf32_bits(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// Byte offset of element (row, k) (k < KC, 4 bytes) in a K-major tile of
// kRowBytes-byte rows with the matching swizzle: the 16-byte chunk index is
// XORed with address bits [7, 10) shifted down (row % 8 for 128-byte rows,
// (row / 2) % 4 for 64-byte rows), the canonical UMMA layouts.
__device__ __forceinline__ int sw_offset(int row, int k) {
  if constexpr (kRowBytes == 128) return row * 128 + ((((k >> 2) ^ (row & 7))) << 4) + ((k & 3) << 2);
  return row * 64 + ((((k >> 2) ^ ((row >> 1) & 3))) << 4) + ((k & 3) << 2);
}

__device__ __forceinline__ void split4(float2 v, uint32_t out[4]) {
  const uint32_t rh = tf32_bits(v.x), ih = tf32_bits(v.y);
  out[0] = rh;
  out[1] = tf32_bits(v.x - __uint_as_float(rh));
  out[2] = ih;
  out[3] = tf32_bits(v.y - __uint_as_float(ih));
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t umma_desc_sw(uint32_t saddr) {
  // start address >> 4 (14 bits), LBO = 1 (unused for swizzled K-major), SBO = 8 rows (the 8-row groups),
  // descriptor version 1, base offset 0, layout type 2 = 128-byte swizzle / 4 = 64-byte swizzle.
  constexpr uint64_t kLayout = kRowBytes == 128 ? 2 : 4;
  return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t(1) << 16) | (uint64_t((8 * kRowBytes) >> 4) << 32) |
         (uint64_t(1) << 46) | (kLayout << 61);
}

// kind::tf32, D = F32, A = B = TF32, both K-major, M = BM, N = 2 BN: one A plane against two adjacent B
// slots, into the adjacent accumulators [Cr | Ci].
constexpr uint32_t kIdesc =
    (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t((2 * BN) >> 3) << 17) | (uint32_t(BM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

}  // namespace

// ---------------------------------------------------------------------------
// operand images: A[b][bm][chunk][plane] (8 KB), B[b][bn][chunk][plane] (4 KB), chunks of KC = 16
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) tc_split_a_kernel(BatchLayout lay, int k, int kb, const float2* __restrict__ M,
                                                         uint8_t* __restrict__ img, int nbm) {
  // The tile is read down the columns (coalesced in the column-major matrix),
  // turned around in shared memory, and written as 16-byte chunks of the
  // swizzled K-major rows, so that every warp stores 512 contiguous bytes.
  constexpr int TS = BM + 1;  // padded row of the transposed tile
  __shared__ float2 T[KC * TS];
  const int nch = (kb + KC - 1) / KC;  // the grid holds nch chunks per row tile
  const int bm = blockIdx.x / nch, chunk = blockIdx.x % nch, b = blockIdx.y;
  const int n = lay.n;
  const int r0 = k + kb + bm * BM;
  const float2* Mb = M + size_t(b) * lay.stride;
  for (int e = threadIdx.x; e < BM * KC; e += blockDim.x) {
    const int r = e % BM, kk = e / BM;
    const int kcol = chunk * KC + kk;
    T[kk * TS + r] = (r0 + r < n && kcol < kb) ? Mb[size_t(r0 + r) + size_t(lay.lda) * (k + kcol)] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  uint8_t* base = img + ((size_t(b) * nbm + bm) * kChunks + chunk) * size_t(A_PLANES) * A_PLANE;
  for (int e = threadIdx.x; e < BM * (KC / 4); e += blockDim.x) {
    const int k4 = e % (KC / 4), r = e / (KC / 4);
    uint32_t q[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      uint32_t sv[4];
      split4(T[(4 * k4 + i) * TS + r], sv);
#pragma unroll
      for (int p = 0; p < 4; ++p) q[p][i] = sv[p];
    }
    const int off = sw_offset(r, 4 * k4);
#pragma unroll
    for (int p = 0; p < 4; ++p)
      *reinterpret_cast<uint4*>(base + size_t(p) * A_PLANE + off) = make_uint4(q[p][0], q[p][1], q[p][2], q[p][3]);
  }
}

__global__ void __launch_bounds__(256) tc_split_b_kernel(BatchLayout lay, int k, int kb, int col_end,
                                                         const float2* __restrict__ M, uint8_t* __restrict__ img,
                                                         int nbn) {
  const int nch = (kb + KC - 1) / KC;  // the grid holds nch chunks per column tile
  const int bn = blockIdx.x / nch, chunk = blockIdx.x % nch, b = blockIdx.y;
  const int c0 = k + kb + bn * BN;
  const float2* Mb = M + size_t(b) * lay.stride;
  uint8_t* base = img + ((size_t(b) * nbn + bn) * kChunks + chunk) * size_t(B_PLANES) * B_PLANE;
  for (int e = threadIdx.x; e < BN * KC; e += blockDim.x) {
    const int kk = e % KC, c = e / KC;
    const int krow = chunk * KC + kk;
    float2 v = make_float2(0.f, 0.f);
    if (c0 + c < col_end && krow < kb) v = Mb[size_t(k + krow) + size_t(lay.lda) * (c0 + c)];
    uint32_t s[4];
    split4(v, s);
    const int off = sw_offset(c, kk);
    auto put = [&](int slot, uint32_t x) { *reinterpret_cast<uint32_t*>(base + size_t(slot) * B_PLANE + off) = x; };
    put(0, s[2] ^ 0x80000000u);  // -im_hi
    put(1, s[0]);                // re_hi
    put(2, s[2]);                // im_hi
    put(3, s[3] ^ 0x80000000u);  // -im_lo
    put(4, s[1]);                // re_lo
    put(5, s[3]);                // im_lo
  }
}

// ---------------------------------------------------------------------------
// the update, persistent and warp-specialised
// ---------------------------------------------------------------------------
// One CTA per SM walks the tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...
// (t -> matrix b, row tile bm, column tile bn, bn fastest).  Roles:
//   warp 0   producer: bulk-copies each K-chunk (56 KB of planes) into a
//            four-stage ring, waiting for the stage to be released;
//   warp 1   MMA: 12 tcgen05.mma (N = 128: [Cr | Ci]) per chunk into one of four TMEM accumulators
//            (128 columns each), releasing the stage with tcgen05.commit and
//            signalling the tile's accumulator the same way;
//   warps 2-17   four epilogue groups of four warps, group g taking the tiles
//            i = g mod 4 of the CTA: C of the tile is loaded into registers
//            16 columns ahead, then tcgen05.ld, subtract, store, release.
// The copies of tile i + 1, its MMAs and the epilogues of the previous tiles
// overlap; four epilogues are in flight per SM, which keeps enough C loads
// outstanding to approach the bandwidth of moving C.  Every wait is bounded; a timeout sets
// the error flag and a shared abort flag that ends every role's loop, then
// the producer waits (bounded) for its copies still in flight and the MMA
// thread for its MMAs before the tensor memory is freed.
constexpr int kPStages = 4;                    // operand ring depth (4 x 56 KB)
constexpr int kPGroups = 4;                     // epilogue groups of 4 warps, one accumulator each
constexpr int kPThreads = 64 + kPGroups * 128;  // producer warp, MMA warp, epilogue groups
constexpr uint32_t kPTmemCols = 512;  // kPGroups * 128 columns, rounded up to a power of two
// barriers: full[kPStages], empty[kPStages], acc_full[kPGroups], acc_empty[kPGroups], drain
constexpr int kBarFull = 0, kBarEmpty = kPStages, kBarAccFull = 2 * kPStages, kBarAccEmpty = 2 * kPStages + kPGroups,
              kBarDrain = 2 * kPStages + 2 * kPGroups;
static_assert((kBarDrain + 1) * 8 <= 256, "barrier area");
constexpr int kPSmem = kPStages * SMEM_OPS + 1024 + 512;
static_assert(kPSmem <= 227 * 1024, "dynamic shared memory per CTA");

__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                                   int* err_flag, long long polls) {
  const uint64_t t0 = global_ns();
  for (long long it = 0; it < polls; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 255) == 255) {
      if (*abort_flag) return false;
      if (global_ns() - t0 > 1000000000ull) break;
    }
  }
  *abort_flag = 1;
  atomicExch(err_flag, 1);
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__global__ void __launch_bounds__(kPThreads, 1) tc_update_persistent_kernel(
    BatchLayout lay, int k, int kb, int col_end, float2* __restrict__ M, const uint8_t* __restrict__ aimg,
    const uint8_t* __restrict__ bimg, int nbm_all, int nbn_all, int nbm, int nbn, int batch, int* __restrict__ err_flag,
    const int* skip, long long polls) {
  extern __shared__ uint8_t smraw[];
  const uint32_t raw = smem_u32(smraw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t* const gbase = smraw + (sbase - raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(gbase + kPStages * SMEM_OPS);
  // bars at kBarFull / kBarEmpty / kBarAccFull / kBarAccEmpty / kBarDrain; then the TMEM slot and flags
  auto bar = [&](int i) { return smem_u32(&bars[i]); };
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + kPStages * SMEM_OPS + 256);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(gbase + kPStages * SMEM_OPS + 260);
  int* consumed = reinterpret_cast<int*>(gbase + kPStages * SMEM_OPS + 264);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n = lay.n;
  const int per_matrix = nbm * nbn;
  const int total = per_matrix * batch;  // the host keeps this below 2^31
  const int nchunks = (kb + KC - 1) / KC;  // 1 .. kChunks

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kPTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 32) {
    for (int i = 0; i < kPStages; ++i) {
      mbar_init(bar(kBarFull + i), 1);   // full: the producer's expect_tx
      mbar_init(bar(kBarEmpty + i), 1);  // empty: one commit
    }
    for (int a = 0; a < kPGroups; ++a) {
      mbar_init(bar(kBarAccFull + a), 1);     // accumulator full: one commit
      mbar_init(bar(kBarAccEmpty + a), 128);  // accumulator empty: the 128 threads of one epilogue group
    }
    mbar_init(bar(kBarDrain), 1);  // drain
    *abort_flag = 0;
    *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  auto tile_of = [&](int t, int& b, int& bm, int& bn) {
    b = t / per_matrix;
    const int rem = t - b * per_matrix;
    bm = rem / nbn;
    bn = rem - bm * nbn;
  };

  if (warp == 0) {
    // ---- producer ----
    if (lane == 0) {
      long long c = 0;  // chunks issued
      for (int t = blockIdx.x; t < total && !*abort_flag; t += gridDim.x) {
        int b, bm, bn;
        tile_of(t, b, bm, bn);
        if (skip && skip[b]) continue;
        const uint8_t* ab = aimg + (size_t(b) * nbm_all + bm) * kChunks * size_t(A_PLANES) * A_PLANE;
        const uint8_t* bb = bimg + (size_t(b) * nbn_all + bn) * kChunks * size_t(B_PLANES) * B_PLANE;
        bool ok = true;
        for (int ch = 0; ch < nchunks; ++ch, ++c) {
          const int st = int(c % kPStages);
          const uint32_t ph = uint32_t((c / kPStages) & 1);
          if (!mbar_wait_or_abort(bar(kBarEmpty + st), ph ^ 1u, abort_flag, err_flag, polls)) { ok = false; break; }
          const uint32_t sA = sbase + uint32_t(st) * SMEM_OPS, sB = sA + A_PLANES * A_PLANE;
          mbar_expect_tx(bar(kBarFull + st), uint32_t(SMEM_OPS));
          const uint8_t* ach = ab + size_t(ch) * A_PLANES * A_PLANE;
          const uint8_t* bch = bb + size_t(ch) * B_PLANES * B_PLANE;
          for (int p = 0; p < A_PLANES; ++p) bulk_copy(sA + p * A_PLANE, ach + size_t(p) * A_PLANE, A_PLANE, bar(kBarFull + st));
          for (int p = 0; p < B_PLANES; ++p) bulk_copy(sB + p * B_PLANE, bch + size_t(p) * B_PLANE, B_PLANE, bar(kBarFull + st));
        }
        if (!ok) break;
      }
      if (*abort_flag) {
        // copies issued but not yet seen complete by the MMA thread: wait for them (bounded)
        for (long long q = *(volatile int*)consumed; q < c; ++q) {
          const uint64_t t0 = global_ns();
          for (long long it = 0; it < kWaitLimit; ++it) {
            uint32_t done;
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                : "=r"(done)
                : "r"(bar(kBarFull + int(q % kPStages))), "r"(uint32_t((q / kPStages) & 1))
                : "memory");
            if (done || ((it & 1023) == 1023 && global_ns() - t0 > 1000000000ull)) break;
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0) {
      long long c = 0, i = 0;  // chunks consumed, tiles of this CTA
      bool issued = false;
      for (int t = blockIdx.x; t < total && !*abort_flag; t += gridDim.x) {
        int b, bm, bn;
        tile_of(t, b, bm, bn);
        if (skip && skip[b]) continue;
        const int a = int(i % kPGroups);
        if (!mbar_wait_or_abort(bar(kBarAccEmpty + a), uint32_t(((i / kPGroups) & 1) ^ 1), abort_flag, err_flag, polls))
          break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t tmem_r = tmem + uint32_t(a * 128), tmem_i = tmem_r + 64;
        bool ok = true;
        for (int ch = 0; ch < nchunks; ++ch, ++c) {
          const int st = int(c % kPStages);
          if (!mbar_wait_or_abort(bar(kBarFull + st), uint32_t((c / kPStages) & 1), abort_flag, err_flag, polls)) { ok = false; break; }
          *(volatile int*)consumed = int(c + 1);
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sA = sbase + uint32_t(st) * SMEM_OPS, sB = sA + A_PLANES * A_PLANE;
          for (int ks = 0; ks < KC / 8; ++ks) {
            const uint32_t koff = uint32_t(ks * 32);
            auto ad = [&](int p) { return umma_desc_sw(sA + p * A_PLANE + koff); };
            auto bd = [&](int p) { return umma_desc_sw(sB + p * B_PLANE + koff); };
            const uint32_t acc0 = (ch == 0 && ks == 0) ? 0u : 1u;
            // [Cr | Ci] += Ar hi [Br hi | Bi hi] + Ar hi [Br lo | Bi lo] + Ar lo [Br hi | Bi hi]
            //            + Ai hi [-Bi hi | Br hi] + Ai hi [-Bi lo | Br lo] + Ai lo [-Bi hi | Br hi],
            // i.e. Cr += Ar Br + Ai (-Bi), Ci += Ar Bi + Ai Br, each hi*hi + hi*lo + lo*hi
            (void)tmem_i;
            mma_tf32(tmem_r, ad(0), bd(1), acc0);
            mma_tf32(tmem_r, ad(0), bd(4), 1u);
            mma_tf32(tmem_r, ad(1), bd(1), 1u);
            mma_tf32(tmem_r, ad(2), bd(0), 1u);
            mma_tf32(tmem_r, ad(2), bd(3), 1u);
            mma_tf32(tmem_r, ad(3), bd(0), 1u);
          }
          issued = true;
          umma_commit(bar(kBarEmpty + st));  // the stage is free once these MMAs have read it
        }
        if (!ok) break;
        umma_commit(bar(kBarAccFull + a));  // the accumulator is complete
        ++i;
      }
      if (issued) {
        // every MMA of this CTA has completed before the tensor memory is freed
        umma_commit(bar(kBarDrain));
        const uint64_t t0 = global_ns();
        for (long long it = 0; it < kWaitLimit; ++it) {
          uint32_t done;
          asm volatile(
              "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
              : "=r"(done)
              : "r"(bar(kBarDrain))
              : "memory");
          if (done || ((it & 1023) == 1023 && global_ns() - t0 > 1000000000ull)) break;
        }
      }
    }
  } else {
    // ---- epilogue groups ----
    const int g = (warp - 2) >> 2;     // group g: warps 2 + 4g .. 5 + 4g
    const int quarter = warp & 3;      // tensor-memory lanes [32 quarter, 32 quarter + 32)
    const uint32_t lane_off = uint32_t(quarter * 32) << 16;
    long long i = 0;                   // tiles of this CTA
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
      // every branch below is uniform across the warp (tcgen05.ld is .sync.aligned)
      if (__shfl_sync(0xffffffffu, *abort_flag, 0)) break;
      int b, bm, bn;
      tile_of(t, b, bm, bn);
      if (skip && skip[b]) continue;
      const long long mine = i++;
      if (mine % kPGroups != g) continue;
      const int r0 = k + kb + bm * BM, c0 = k + kb + bn * BN;
      const int row = r0 + quarter * 32 + lane;
      const bool row_ok = row < n;
      const int ld = lay.lda;  // column offsets within a tile stay far below 2^31 elements
      float2* crow = M + size_t(b) * lay.stride + size_t(row) + size_t(lay.lda) * size_t(c0);
      // C of 16 columns at a time, the next part loaded while this one is stored
      float2 cn[16];
#pragma unroll
      for (int j = 0; j < 16; ++j)
        cn[j] = (row_ok && c0 + j < col_end) ? crow[j * ld] : make_float2(0.f, 0.f);
      const bool ready = mbar_wait_or_abort(bar(kBarAccFull + g), uint32_t((mine / kPGroups) & 1), abort_flag, err_flag, polls);
      if (!__all_sync(0xffffffffu, ready)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tmem_r = tmem + uint32_t(g * 128) + lane_off, tmem_i = tmem_r + 64;
#pragma unroll 1
      for (int part = 0; part < BN / 16; ++part) {
        float2 cc[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) cc[j] = cn[j];
        if (part + 1 < BN / 16) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = c0 + (part + 1) * 16 + j;
            cn[j] = (row_ok && col < col_end) ? crow[((part + 1) * 16 + j) * ld] : make_float2(0.f, 0.f);
          }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint32_t cr[8], ci[8];
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                       : "=r"(cr[0]), "=r"(cr[1]), "=r"(cr[2]), "=r"(cr[3]), "=r"(cr[4]), "=r"(cr[5]), "=r"(cr[6]),
                         "=r"(cr[7])
                       : "r"(tmem_r + uint32_t(part * 16 + h * 8)));
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                       : "=r"(ci[0]), "=r"(ci[1]), "=r"(ci[2]), "=r"(ci[3]), "=r"(ci[4]), "=r"(ci[5]), "=r"(ci[6]),
                         "=r"(ci[7])
                       : "r"(tmem_i + uint32_t(part * 16 + h * 8)));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (row_ok) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const int col = c0 + part * 16 + h * 8 + j;
              if (col < col_end) {
                float2 v = cc[h * 8 + j];
                v.x -= __uint_as_float(cr[j]);
                v.y -= __uint_as_float(ci[j]);
                crow[(part * 16 + h * 8 + j) * ld] = v;
              }
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(bar(kBarAccEmpty + g));  // the accumulator may be overwritten
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kPTmemCols));
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
size_t tc_image_bytes(int n, int m, int batch) {
  const int nbm = (n + BM - 1) / BM, nbn = (n + m + BN - 1) / BN;
  return size_t(batch) * kChunks * (size_t(nbm) * A_PLANES * A_PLANE + size_t(nbn) * B_PLANES * B_PLANE);
}

void tc_trailing_update(const BatchLayout& lay, int batch, int k, int kb, int col_end, float2* M, uint8_t* images,
                        int* err_flag, const int* skip, long long wait_polls, KernelSpans* spans, cudaStream_t s) {
  const int rows = lay.n - (k + kb), cols = col_end - (k + kb);
  if (rows <= 0 || cols <= 0 || kb <= 0) return;
  const int nbm_all = (lay.n + BM - 1) / BM, nbn_all = (lay.n + lay.m + BN - 1) / BN;
  uint8_t* aimg = images;
  uint8_t* bimg = images + size_t(batch) * kChunks * size_t(nbm_all) * A_PLANES * A_PLANE;
  const int nbm = (rows + BM - 1) / BM, nbn = (cols + BN - 1) / BN;
  count_launch();
  const int nch = (kb + KC - 1) / KC;
  tc_split_a_kernel<<<dim3(unsigned(nch * nbm), unsigned(batch)), 256, 0, s>>>(lay, k, kb, M, aimg, nbm_all);
  count_launch();
  tc_split_b_kernel<<<dim3(unsigned(nch * nbn), unsigned(batch)), 256, 0, s>>>(lay, k, kb, col_end, M, bimg, nbn_all);
  const int sms = current_sm_count();
  ensure_smem_limit(reinterpret_cast<const void*>(tc_update_persistent_kernel), size_t(kPSmem));
  const long long tiles = (long long)nbm * nbn * batch;
  if (tiles > 0x7fffffffLL) {  // the kernel numbers tiles with 32-bit integers
    if (err_flag) cudaMemsetAsync(err_flag, 0xff, sizeof(int), s);
    return;
  }
  const unsigned grid = unsigned(tiles < sms ? tiles : sms);
  const bool prof = spans && spans->on;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (prof) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
  }
  count_launch();
  tc_update_persistent_kernel<<<grid, kPThreads, kPSmem, s>>>(lay, k, kb, col_end, M, aimg, bimg, nbm_all, nbn_all,
                                                              nbm, nbn, batch, err_flag, skip,
                                                              wait_polls > 0 ? wait_polls : kTcWaitPolls);
  if (prof) {
    cudaEventRecord(e1, s);
    spans->spans.push_back({e0, e1});
  }
}

}  // namespace rfx
