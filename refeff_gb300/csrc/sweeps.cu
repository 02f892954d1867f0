// Fused triangular sweeps for the FP32 refinement: the whole forward (L, with
// the stored per-panel row moves) or backward (U) substitution of a group of
// right-hand-side columns runs in one CTA per (matrix, column group), with
// the right-hand sides resident in shared memory.  One launch replaces the
// ~2 x n/NB small launches of the blocked sweep, and each CTA streams its
// triangle from HBM exactly once.
//
// Reference: the solve half of complex32_faer_lu_solve
// (crates/refeff-linalg/src/lu.rs:474-529), applied to the elimination's
// factors and row moves.
#include <cuda_runtime.h>

#include "batched_lu.cuh"
#include "cplx.cuh"
#include "fms_plan.cuh"

namespace rfx {
namespace {

constexpr int kSwThreads = 512;
constexpr int kSwUnroll = 16;

template <int NB, int CG>
struct SweepSmem {
  static size_t bytes(int n) { return (size_t(n) * CG + size_t(NB) * (NB + 1) + size_t(2 * NB) * CG) * sizeof(float2); }
};

// Y[r] -= sum_j T(r, j) X[j] for rows [r_begin, r_end), j < kb, T column j at
// Mb + lda (c0 + j).  Each thread walks its rows (r_begin + tid + q kSwThreads)
// in batches of kSwUnroll columns and loads the next batch (of the same row or
// of its next row) before it multiplies the current one, so that the loads of
// one batch are in flight while the previous batch is computed.
template <int CG>
__device__ __forceinline__ void sweep_update(const float2* __restrict__ Mb, size_t lda, int c0, int kb, int r_begin,
                                             int r_end, const float2* X, float2* Y) {
  const int nfull = kb / kSwUnroll;
  if (nfull == 0) {  // a narrow last block: one column at a time
    for (int r = r_begin + int(threadIdx.x); r < r_end; r += kSwThreads) {
      float2 acc[CG];
#pragma unroll
      for (int c = 0; c < CG; ++c) acc[c] = make_float2(0.f, 0.f);
      for (int j = 0; j < kb; ++j) {
        const float2 l = Mb[size_t(r) + lda * size_t(c0 + j)];
#pragma unroll
        for (int c = 0; c < CG; ++c) cfma(acc[c], l, X[j * CG + c]);
      }
#pragma unroll
      for (int c = 0; c < CG; ++c) Y[r * CG + c] = csub(Y[r * CG + c], acc[c]);
    }
    return;
  }
  int r = r_begin + int(threadIdx.x);
  if (r >= r_end) return;
  auto load = [&](int rr, int bb, float2 (&v)[kSwUnroll]) {
#pragma unroll
    for (int u = 0; u < kSwUnroll; ++u) v[u] = Mb[size_t(rr) + lda * size_t(c0 + bb * kSwUnroll + u)];
  };
  float2 acc[CG];
#pragma unroll
  for (int c = 0; c < CG; ++c) acc[c] = make_float2(0.f, 0.f);
  float2 cur[kSwUnroll];
  load(r, 0, cur);
  int bi = 0;
  for (;;) {
    int rn = r, bn = bi + 1;
    if (bn == nfull) {
      rn = r + kSwThreads;
      bn = 0;
    }
    const bool more = rn < r_end;
    float2 nxt[kSwUnroll];
    if (more) load(rn, bn, nxt);
    const int j0 = bi * kSwUnroll;
#pragma unroll
    for (int u = 0; u < kSwUnroll; ++u)
#pragma unroll
      for (int c = 0; c < CG; ++c) cfma(acc[c], cur[u], X[(j0 + u) * CG + c]);
    if (bn == 0) {  // row r done with its full batches: the remaining columns, then the row
      for (int j = nfull * kSwUnroll; j < kb; ++j) {
        const float2 l = Mb[size_t(r) + lda * size_t(c0 + j)];
#pragma unroll
        for (int c = 0; c < CG; ++c) cfma(acc[c], l, X[j * CG + c]);
      }
#pragma unroll
      for (int c = 0; c < CG; ++c) {
        Y[r * CG + c] = csub(Y[r * CG + c], acc[c]);
        acc[c] = make_float2(0.f, 0.f);
      }
    }
    if (!more) break;
    r = rn;
    bi = bn;
#pragma unroll
    for (int u = 0; u < kSwUnroll; ++u) cur[u] = nxt[u];
  }
}

template <int NB, int CG>
__global__ void __launch_bounds__(kSwThreads) fwd_sweep_kernel(BatchLayout lay, float2* __restrict__ M, LuWork w,
                                                               const int* skip) {
  const int b = blockIdx.y, cg0 = blockIdx.x * CG;
  if (skip && skip[b]) return;
  const int n = lay.n, ncols = min(CG, lay.m - cg0);
  extern __shared__ float2 sw_sm[];
  float2* Y = sw_sm;                                // [n][CG]
  float2* T = Y + size_t(n) * CG;                   // [NB][NB + 1]
  float2* tmp = T + NB * (NB + 1);                  // [2 NB][CG]
  float2* Mb = M + size_t(b) * lay.stride;
  const size_t lda = size_t(lay.lda);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int idx = tid; idx < n * CG; idx += kSwThreads) {
    const int r = idx % n, c = idx / n;
    Y[r * CG + c] = c < ncols ? Mb[size_t(r) + lda * size_t(n + cg0 + c)] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int k = 0; k < n; k += NB) {
    const int kb = min(NB, n - k);
    // row moves of this panel, applied as one gather; with paired blocks both
    // blocks' moves are applied before the first block of the pair is solved
    // (the second block's moves only touch rows below the first block)
    const bool pair = w.pair128 && NB == 64;
    const int p0 = k / NB;
    const int nmoves = !pair ? 1 : (p0 % 2 == 1 ? 0 : (k + NB < n ? 2 : 1));
    for (int idx = tid; idx < kb * kb; idx += kSwThreads) {
      const int r = idx % kb, c = idx / kb;
      T[r * (NB + 1) + c] = Mb[size_t(k + r) + lda * size_t(k + c)];
    }
    for (int q = 0; q < nmoves; ++q) {
      const size_t pidx = size_t(b) * w.npanels + p0 + q;
      const int np = w.nperm[pidx];
      const int2* pm = w.perm + pidx * (2 * NB);
      for (int idx = tid; idx < np * CG; idx += kSwThreads) tmp[idx] = Y[pm[idx / CG].y * CG + idx % CG];
      __syncthreads();
      for (int idx = tid; idx < np * CG; idx += kSwThreads) Y[pm[idx / CG].x * CG + idx % CG] = tmp[idx];
      __syncthreads();
    }
    __syncthreads();
    // unit-lower solve of the block rows, one warp per column
    if (wid < ncols) {
      constexpr int kR = (NB + 31) / 32;
      float2 x[kR];
#pragma unroll
      for (int t = 0; t < kR; ++t) {
        const int i = lane + 32 * t;
        x[t] = i < kb ? Y[(k + i) * CG + wid] : make_float2(0.f, 0.f);
      }
      for (int p = 0; p < kb; ++p) {
        const int ot = p >> 5, ol = p & 31;
        float2 xp = make_float2(0.f, 0.f);
#pragma unroll
        for (int t = 0; t < kR; ++t) {
          const float re = __shfl_sync(0xffffffffu, x[t].x, ol);
          const float im = __shfl_sync(0xffffffffu, x[t].y, ol);
          if (t == ot) xp = make_float2(re, im);
        }
#pragma unroll
        for (int t = 0; t < kR; ++t) {
          const int i = lane + 32 * t;
          if (i > p && i < kb) cfms(x[t], T[i * (NB + 1) + p], xp);
        }
      }
#pragma unroll
      for (int t = 0; t < kR; ++t) {
        const int i = lane + 32 * t;
        if (i < kb) Y[(k + i) * CG + wid] = x[t];
      }
    }
    __syncthreads();
    sweep_update<CG>(Mb, lda, k, kb, k + kb, n, Y + size_t(k) * CG, Y);
    __syncthreads();
  }
  for (int idx = tid; idx < n * ncols; idx += kSwThreads) {
    const int r = idx % n, c = idx / n;
    Mb[size_t(r) + lda * size_t(n + cg0 + c)] = Y[r * CG + c];
  }
}

template <int NB, int CG>
__global__ void __launch_bounds__(kSwThreads) bwd_sweep_kernel(BatchLayout lay, float2* __restrict__ M,
                                                               const int* skip) {
  const int b = blockIdx.y, cg0 = blockIdx.x * CG;
  if (skip && skip[b]) return;
  const int n = lay.n, ncols = min(CG, lay.m - cg0);
  extern __shared__ float2 sw_sm[];
  float2* Y = sw_sm;
  float2* T = Y + size_t(n) * CG;
  float2* dinv = T + NB * (NB + 1);  // reciprocals of the block's diagonal (0 for a zero pivot)
  float2* Mb = M + size_t(b) * lay.stride;
  const size_t lda = size_t(lay.lda);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int idx = tid; idx < n * CG; idx += kSwThreads) {
    const int r = idx % n, c = idx / n;
    Y[r * CG + c] = c < ncols ? Mb[size_t(r) + lda * size_t(n + cg0 + c)] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int k = ((n - 1) / NB) * NB; k >= 0; k -= NB) {
    const int kb = min(NB, n - k);
    for (int idx = tid; idx < kb * kb; idx += kSwThreads) {
      const int r = idx % kb, c = idx / kb;
      const float2 v = Mb[size_t(k + r) + lda * size_t(k + c)];
      T[r * (NB + 1) + c] = v;
      if (r == c) dinv[r] = (v.x == 0.f && v.y == 0.f) ? make_float2(0.f, 0.f) : cdiv(make_float2(1.f, 0.f), v);
    }
    __syncthreads();
    if (wid < ncols) {
      constexpr int kR = (NB + 31) / 32;
      float2 x[kR];
#pragma unroll
      for (int t = 0; t < kR; ++t) {
        const int i = lane + 32 * t;
        x[t] = i < kb ? Y[(k + i) * CG + wid] : make_float2(0.f, 0.f);
      }
      for (int p = kb - 1; p >= 0; --p) {
        const int ot = p >> 5, ol = p & 31;
#pragma unroll
        for (int t = 0; t < kR; ++t)
          if (t == ot && lane == ol) x[t] = cmul(x[t], dinv[p]);
        float2 xp = make_float2(0.f, 0.f);
#pragma unroll
        for (int t = 0; t < kR; ++t) {
          const float re = __shfl_sync(0xffffffffu, x[t].x, ol);
          const float im = __shfl_sync(0xffffffffu, x[t].y, ol);
          if (t == ot) xp = make_float2(re, im);
        }
#pragma unroll
        for (int t = 0; t < kR; ++t) {
          const int i = lane + 32 * t;
          if (i < p) cfms(x[t], T[i * (NB + 1) + p], xp);
        }
      }
#pragma unroll
      for (int t = 0; t < kR; ++t) {
        const int i = lane + 32 * t;
        if (i < kb) Y[(k + i) * CG + wid] = x[t];
      }
    }
    __syncthreads();
    sweep_update<CG>(Mb, lda, k, kb, 0, k, Y + size_t(k) * CG, Y);
    __syncthreads();
  }
  for (int idx = tid; idx < n * ncols; idx += kSwThreads) {
    const int r = idx % n, c = idx / n;
    Mb[size_t(r) + lda * size_t(n + cg0 + c)] = Y[r * CG + c];
  }
}

constexpr size_t kSwSmemBudget = 200 * 1024;

template <int NB, int CG>
bool launch_sweep_cg(bool forward, const BatchLayout& lay, int batch, float2* M, const LuWork* w, const int* skip,
                     cudaStream_t s) {
  const size_t smem = SweepSmem<NB, CG>::bytes(lay.n);
  // each column group streams the whole triangle: decline narrow groups for many columns
  if (smem > kSwSmemBudget || CG < (lay.m < 4 ? lay.m : 4)) return false;
  if (forward) ensure_smem_limit(reinterpret_cast<const void*>(fwd_sweep_kernel<NB, CG>), smem);
  else ensure_smem_limit(reinterpret_cast<const void*>(bwd_sweep_kernel<NB, CG>), smem);
  dim3 grid(unsigned((lay.m + CG - 1) / CG), unsigned(batch));
  count_launch();
  if (forward) fwd_sweep_kernel<NB, CG><<<grid, kSwThreads, smem, s>>>(lay, M, *w, skip);
  else bwd_sweep_kernel<NB, CG><<<grid, kSwThreads, smem, s>>>(lay, M, skip);
  return true;
}

template <int NB>
bool launch_sweep_nb(bool forward, const BatchLayout& lay, int batch, float2* M, const LuWork* w, const int* skip,
                     cudaStream_t s) {
  return launch_sweep_cg<NB, 8>(forward, lay, batch, M, w, skip, s) ||
         launch_sweep_cg<NB, 4>(forward, lay, batch, M, w, skip, s) ||
         launch_sweep_cg<NB, 2>(forward, lay, batch, M, w, skip, s) ||
         launch_sweep_cg<NB, 1>(forward, lay, batch, M, w, skip, s);
}

}  // namespace

bool fused_forward_sweep(int nb, const BatchLayout& lay, int batch, float2* M, const LuWork& w, const int* skip,
                         cudaStream_t s) {
  if (nb == 64) return launch_sweep_nb<64>(true, lay, batch, M, &w, skip, s);
  if (nb == 32) return launch_sweep_nb<32>(true, lay, batch, M, &w, skip, s);
  return false;
}

bool fused_sweep_available(int nb, const BatchLayout& lay) {
  const int need = lay.m < 4 ? lay.m : 4;  // the narrowest column group launch_sweep_cg accepts
  if (nb == 64) return SweepSmem<64, 8>::bytes(lay.n) <= kSwSmemBudget ||
                       (need <= 4 && SweepSmem<64, 4>::bytes(lay.n) <= kSwSmemBudget) ||
                       (need <= 2 && SweepSmem<64, 2>::bytes(lay.n) <= kSwSmemBudget) ||
                       (need <= 1 && SweepSmem<64, 1>::bytes(lay.n) <= kSwSmemBudget);
  if (nb == 32) return SweepSmem<32, 8>::bytes(lay.n) <= kSwSmemBudget ||
                       (need <= 4 && SweepSmem<32, 4>::bytes(lay.n) <= kSwSmemBudget) ||
                       (need <= 2 && SweepSmem<32, 2>::bytes(lay.n) <= kSwSmemBudget) ||
                       (need <= 1 && SweepSmem<32, 1>::bytes(lay.n) <= kSwSmemBudget);
  return false;
}

bool fused_backward_sweep(int nb, const BatchLayout& lay, int batch, float2* M, const int* skip, cudaStream_t s) {
  if (nb == 64) return launch_sweep_nb<64>(false, lay, batch, M, nullptr, skip, s);
  if (nb == 32) return launch_sweep_nb<32>(false, lay, batch, M, nullptr, skip, s);
  return false;
}

}  // namespace rfx
