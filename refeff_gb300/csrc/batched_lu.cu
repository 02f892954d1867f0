// Batched blocked complex LU (partial pivoting, pivot norm |re|+|im| as in
// crates/refeff-linalg/src/lu.rs:337-345, 612-614) on augmented systems
// [A | B], batched over energy points, and the triangular sweeps that reuse
// the factors (crates/refeff-linalg/src/lu.rs:400-529 solve semantics).
//
// One elimination step k (panel width NB):
//   panel_kernel      the (n-k) x NB panel lives in the distributed shared
//                     memory of a thread-block cluster (rows split across the
//                     CTAs); one cluster barrier per column: local arg-max,
//                     cluster arg-max over DSMEM, pivot row read over DSMEM,
//                     rank-1 update of the CTA's own rows.  Rows are not moved
//                     while the panel is factored; the permutation is applied
//                     when the panel is written back, and its row moves are
//                     stored per panel.
//   rhs_lower_kernel  applies the panel's row moves to the trailing columns and
//                     solves U12 = L11^-1 A12 (one warp per column).
//   gemm_update       A22 -= L21 U12 on the trailing block (B included).
// Columns left of the panel are never permuted.  A later forward sweep
// applies each panel's moves to the new right-hand side just before that
// panel's L columns, which is the same permutation order the elimination saw.
#include <cooperative_groups.h>
#include <climits>
#include "cplx.cuh"
#include "batched_lu.cuh"

namespace cg = cooperative_groups;

namespace rfx {

constexpr int kPanelThreads = 256;

template <typename T, int NB>
static size_t panel_smem_bytes(int rpc_max, int n, bool pos_global) {
  size_t b = size_t(NB) * rpc_max * sizeof(cplx<T>);  // panel
  b += NB * sizeof(cplx<T>);                          // pivot row copy
  b += 2 * 16;                                        // arg-max slots
  b += size_t(rpc_max) * sizeof(int);                 // done flags
  if (!pos_global) b += 2 * size_t(n) * sizeof(int);  // row2pos / pos2row (rank 0)
  b += 64;                                            // scratch
  return (b + 15) / 16 * 16;
}

static size_t panel_smem_any(int elem, int nb, int rpc, int n, bool pos_global) {
  if (elem == 8) {
    switch (nb) {
      case 64: return panel_smem_bytes<float, 64>(rpc, n, pos_global);
      case 32: return panel_smem_bytes<float, 32>(rpc, n, pos_global);
      default: return panel_smem_bytes<float, 16>(rpc, n, pos_global);
    }
  }
  switch (nb) {
    case 32: return panel_smem_bytes<double, 32>(rpc, n, pos_global);
    case 16: return panel_smem_bytes<double, 16>(rpc, n, pos_global);
    default: return panel_smem_bytes<double, 8>(rpc, n, pos_global);
  }
}

template <typename T>
struct alignas(16) ArgSlot {
  T val;
  int row;
};

template <typename T>
__device__ __forceinline__ void argmax_merge(T& v, int& r, T ov, int orow) {
  if (ov > v || (ov == v && orow < r)) { v = ov; r = orow; }
}

template <typename T, int NB>
__global__ void __launch_bounds__(kPanelThreads) panel_kernel(BatchLayout lay, int k, cplx<T>* __restrict__ M,
                                                              LuWork w, int rpc_max) {
  using C = cplx<T>;
  cg::cluster_group cluster = cg::this_cluster();
  const int CL = int(cluster.num_blocks());
  const int rank = int(cluster.block_rank());
  const int b = blockIdx.y;
  const int n = lay.n;
  const int R = n - k;
  const int kb = min(NB, R);
  const int panel = k / NB;
  const int rpc = (R + CL - 1) / CL;
  const int row_lo = rank * rpc;
  const int nloc = max(0, min(R, row_lo + rpc) - row_lo);
  const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31, wid = tid >> 5;

  extern __shared__ __align__(16) unsigned char smraw[];
  C* pan = reinterpret_cast<C*>(smraw);
  C* urow = pan + size_t(NB) * rpc_max;
  int* done = reinterpret_cast<int*>(reinterpret_cast<ArgSlot<T>*>(urow + NB) + 2);  // after two reserved slots
  // row-position bookkeeping (rank 0): shared memory, or global scratch for large n
  const bool pos_global = w.pos_scratch != nullptr;
  int* row2pos = pos_global ? w.pos_scratch + size_t(b) * 2 * n : done + rpc_max;
  int* pos2row = row2pos + n;
  int* scratch = pos_global ? done + rpc_max : pos2row + n;  // [2] move count
  // per-warp arg-max slots, double-buffered by column parity
  __shared__ ArgSlot<T> wslot[2][kPanelThreads / 32];

  C* Mb = M + size_t(b) * lay.stride;
  for (int idx = tid; idx < nloc * kb; idx += nthr) {
    const int r = idx % nloc, c = idx / nloc;
    pan[size_t(c) * rpc_max + r] = Mb[size_t(k + row_lo + r) + size_t(lay.lda) * (k + c)];
  }
  for (int r = tid; r < nloc; r += nthr) done[r] = 0;
  if (rank == 0) {
    for (int q = tid; q < R; q += nthr) { row2pos[q] = q; pos2row[q] = q; }
    if (tid == 0) scratch[2] = 0;
  }
  __syncthreads();

  // Each thread keeps the same rows (r = tid, tid + nthr, ...) for the whole
  // panel, so their done flags are its own and the arg-max of column j + 1 is
  // taken while column j's update writes it.  Per column: one cluster barrier
  // (every warp has published its arg-max), one CTA barrier (the pivot row is
  // in shared memory).  Ties go to the lowest row, so the pivots do not depend
  // on the reduction order.
  const int nw = nthr / 32;
  T best = T(-1);
  int brow = INT_MAX;
  for (int r = tid; r < nloc; r += nthr) {
    T v = cabs1(pan[r]);
    if (!(v >= T(0))) v = T(0);  // a NaN entry competes as zero, so a valid row is always chosen
    argmax_merge(best, brow, v, row_lo + r);
  }
  for (int j = 0; j < kb; ++j) {
    for (int off = 16; off > 0; off >>= 1) {
      const T ov = __shfl_down_sync(0xffffffffu, best, off);
      const int orow = __shfl_down_sync(0xffffffffu, brow, off);
      argmax_merge(best, brow, ov, orow);
    }
    if (lane == 0) {
      wslot[j & 1][wid].val = best;
      wslot[j & 1][wid].row = brow;
    }
    cluster.sync();
    // every warp reduces the cluster's slots over DSMEM; the butterfly leaves the winner in every lane
    T wv = T(-1);
    int wrow = INT_MAX;
    for (int q = lane; q < CL * nw; q += 32) {
      const ArgSlot<T>* rs = cluster.map_shared_rank(&wslot[j & 1][0], q / nw);
      argmax_merge(wv, wrow, rs[q % nw].val, rs[q % nw].row);
    }
    for (int off = 16; off > 0; off >>= 1) {
      const T ov = __shfl_xor_sync(0xffffffffu, wv, off);
      const int orow = __shfl_xor_sync(0xffffffffu, wrow, off);
      argmax_merge(wv, wrow, ov, orow);
    }
    const int owner = wrow / rpc, lr = wrow % rpc;
    const C* opan = cluster.map_shared_rank(pan, owner);
    for (int c = j + tid; c < kb; c += nthr) urow[c] = opan[size_t(c) * rpc_max + lr];
    if (rank == owner && tid == lr % nthr) done[lr] = 1;
    if (rank == 0 && tid == 0) {
      const int q = row2pos[wrow];
      const int pj = pos2row[j];
      pos2row[j] = wrow;
      pos2row[q] = pj;
      row2pos[wrow] = j;
      row2pos[pj] = q;
      w.ipiv[size_t(b) * n + k + j] = k + q;
      if (!(wv > T(0))) {
        atomicMax(w.status + b, int(kDevSingular));
        atomicCAS(w.info + b, 0, k + j + 1);
      }
    }
    __syncthreads();
    // multipliers, rank-1 update of own rows, and the local arg-max of column j + 1
    const C pv = urow[j];
    const bool zero_pivot = !(cabs1(pv) > T(0));
    best = T(-1);
    brow = INT_MAX;
    for (int r = tid; r < nloc; r += nthr) {
      if (done[r]) continue;
      C l = pan[size_t(j) * rpc_max + r];
      l = zero_pivot ? mk<T>(T(0), T(0)) : cdiv(l, pv);
      pan[size_t(j) * rpc_max + r] = l;
      for (int c = j + 1; c < kb; ++c) cfms(pan[size_t(c) * rpc_max + r], l, urow[c]);
      if (j + 1 < kb) {
        T v = cabs1(pan[size_t(j + 1) * rpc_max + r]);
        if (!(v >= T(0))) v = T(0);
        argmax_merge(best, brow, v, row_lo + r);
      }
    }
  }
  cluster.sync();
  // write back in pivoted order; rank 0 publishes the row moves of this panel
  const int* r2p0 = pos_global ? row2pos : cluster.map_shared_rank(row2pos, 0);
  for (int idx = tid; idx < nloc * kb; idx += nthr) {
    const int r = idx % nloc, c = idx / nloc;
    const int dst = k + r2p0[row_lo + r];
    Mb[size_t(dst) + size_t(lay.lda) * (k + c)] = pan[size_t(c) * rpc_max + r];
  }
  if (rank == 0) {
    int2* pm = w.perm + (size_t(b) * w.npanels + panel) * (2 * NB);
    for (int q = tid; q < R; q += nthr) {
      if (pos2row[q] != q) {
        const int si = atomicAdd(&scratch[2], 1);
        if (si < 2 * NB) pm[si] = make_int2(k + q, k + pos2row[q]);
      }
    }
    __syncthreads();
    if (tid == 0) w.nperm[size_t(b) * w.npanels + panel] = min(scratch[2], 2 * NB);
  }
  cluster.sync();
}

template <typename T, int NB, bool kSolve>
__device__ __forceinline__ void rhs_lower_column(const BatchLayout& lay, int k, int kb, cplx<T>* colp, const LuWork& w,
                                                 int b, const cplx<T> (*L11)[NB + 1], int lane) {
  using C = cplx<T>;
  const int panel = k / NB;
  const size_t pidx = size_t(b) * w.npanels + panel;
  const int np = w.nperm[pidx];
  const int2* pm = w.perm + pidx * (2 * NB);
  constexpr int kMoves = (2 * NB + 31) / 32;
  C v[kMoves];
  int dst[kMoves];
#pragma unroll
  for (int t = 0; t < kMoves; ++t) {
    const int i = lane + 32 * t;
    dst[t] = -1;
    if (i < np) { const int2 mv = pm[i]; dst[t] = mv.x; v[t] = colp[mv.y]; }
  }
  __syncwarp();
#pragma unroll
  for (int t = 0; t < kMoves; ++t)
    if (dst[t] >= 0) colp[dst[t]] = v[t];
  __syncwarp();
  if constexpr (!kSolve) return;
  constexpr int kRows = (NB + 31) / 32;
  C x[kRows];
#pragma unroll
  for (int t = 0; t < kRows; ++t) {
    const int i = lane + 32 * t;
    x[t] = i < kb ? colp[k + i] : mk<T>(T(0), T(0));
  }
  for (int p = 0; p < kb; ++p) {
    const int owner_t = p >> 5, owner_l = p & 31;
    C xp = mk<T>(T(0), T(0));
#pragma unroll
    for (int t = 0; t < kRows; ++t) {
      const T re = __shfl_sync(0xffffffffu, x[t].x, owner_l);
      const T im = __shfl_sync(0xffffffffu, x[t].y, owner_l);
      if (t == owner_t) { xp.x = re; xp.y = im; }
    }
#pragma unroll
    for (int t = 0; t < kRows; ++t) {
      const int i = lane + 32 * t;
      if (i > p && i < kb) cfms(x[t], L11[i][p], xp);
    }
  }
#pragma unroll
  for (int t = 0; t < kRows; ++t) {
    const int i = lane + 32 * t;
    if (i < kb) colp[k + i] = x[t];
  }
}

// Columns [c_begin, c_end), kRhsColsPerWarp per warp (one after another, so
// that each CTA reads L11 once for 8 * kRhsColsPerWarp columns): apply the
// panel's row moves, then solve the panel rows with the unit lower L11.
constexpr int kRhsColsPerWarp = 4;

template <typename T, int NB, bool kSolve = true>
__global__ void __launch_bounds__(256) rhs_lower_kernel(BatchLayout lay, int k, int c_begin, int c_end,
                                                        cplx<T>* __restrict__ M, LuWork w, const int* skip) {
  using C = cplx<T>;
  const int b = blockIdx.y;
  if (skip && skip[b]) return;
  __shared__ C L11[kSolve ? NB : 1][NB + 1];
  const int n = lay.n;
  const int kb = min(NB, n - k);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  C* Mb = M + size_t(b) * lay.stride;
  if constexpr (kSolve) {
    for (int idx = threadIdx.x; idx < kb * kb; idx += blockDim.x) {
      const int r = idx % kb, c = idx / kb;
      L11[r][c] = Mb[size_t(k + r) + size_t(lay.lda) * (k + c)];
    }
    __syncthreads();
  }
  const int first = c_begin + blockIdx.x * (blockDim.x / 32) * kRhsColsPerWarp + wid;
  for (int cw = 0; cw < kRhsColsPerWarp; ++cw) {
    const int col = first + cw * (blockDim.x / 32);
    if (col >= c_end) return;
    rhs_lower_column<T, NB, kSolve>(lay, k, kb, Mb + size_t(lay.lda) * col, w, b, L11, lane);
  }
}
// The outer block row of the two-level FP32 elimination as a product:
// U12 = L11^-1 (P A12).  First each matrix's unit lower L11 (rows and columns
// [k, k + kb)) is inverted, one warp per column of the inverse; then each CTA
// takes kLtN columns of the block row, applies the block's composed row moves
// (rows in [k, n)) and multiplies the kb panel rows by L11^-1 from shared
// memory, each thread keeping 8 rows of one column in registers.  The
// column-by-column substitution it replaces walked a 64-step dependent chain
// of shuffles per column; here the same flops run with full instruction-level
// parallelism.  Partial pivoting keeps |L11| <= 1, so the explicit inverse is
// as good a triangular solve as substitution for the FP32 factors, which the
// FP64 refinement corrects in any case.
constexpr int kLtN = 32;  // block-row columns per CTA of rhs_lower_tile_kernel

__global__ void __launch_bounds__(256) unit_lower_inverse_kernel(BatchLayout lay, int k,
                                                                 const float2* __restrict__ M,
                                                                 float2* __restrict__ linv) {
  constexpr int NB = 64, kRows = NB / 32;
  const int b = blockIdx.x;
  __shared__ float2 L11[NB][NB + 1];
  const int kb = min(NB, lay.n - k);
  const float2* Mb = M + size_t(b) * lay.stride;
  for (int idx = threadIdx.x; idx < kb * kb; idx += blockDim.x) {
    const int r = idx % kb, c = idx / kb;
    L11[r][c] = Mb[size_t(k + r) + size_t(lay.lda) * (k + c)];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2* out = linv + size_t(b) * NB * NB;
  for (int j = wid; j < NB; j += 8) {
    float2 x[kRows];
#pragma unroll
    for (int t = 0; t < kRows; ++t) x[t] = make_float2(lane + 32 * t == j ? 1.f : 0.f, 0.f);
    for (int p = j; p < kb; ++p) {
      const int ot = p >> 5, ol = p & 31;
      float2 xp = make_float2(0.f, 0.f);
#pragma unroll
      for (int t = 0; t < kRows; ++t) {
        const float re = __shfl_sync(0xffffffffu, x[t].x, ol);
        const float im = __shfl_sync(0xffffffffu, x[t].y, ol);
        if (t == ot) xp = make_float2(re, im);
      }
#pragma unroll
      for (int t = 0; t < kRows; ++t) {
        const int i = lane + 32 * t;
        if (i > p && i < kb) cfms(x[t], L11[i][p], xp);
      }
    }
#pragma unroll
    for (int t = 0; t < kRows; ++t) {
      const int i = lane + 32 * t;
      out[i + NB * j] = (i < kb && j < kb) ? x[t] : make_float2(0.f, 0.f);
    }
  }
}

// With kprev >= 0 (paired blocks) the block is the second of a pair whose
// first block starts at kprev and whose update of these columns was deferred:
// between the row moves and the L11^-1 product the panel rows get
// A12 -= L21prev (rows [k, k + kb), columns [kprev, kprev + 64)) U12prev
// (rows [kprev, kprev + 64) of these columns).
__global__ void __launch_bounds__(256) rhs_lower_tile_kernel(BatchLayout lay, int k, int c_begin, int c_end,
                                                             float2* __restrict__ M, LuWork w,
                                                             const float2* __restrict__ linv, int kprev) {
  constexpr int NB = 64;
  const int b = blockIdx.y, cb = c_begin + blockIdx.x * kLtN;
  const int ncols = min(kLtN, c_end - cb);
  const int kb = min(NB, lay.n - k);
  extern __shared__ float2 lt_sm[];
  float2* Li = lt_sm;               // [NB][NB]: Li[i + NB * j] = (L11^-1)(i, j)
  float2* Bt = lt_sm + NB * NB;     // [NB][kLtN]: the block rows (after the moves)
  float2* Bw = Bt + NB * kLtN;      // [NB][kLtN]: rows moved below the block, then U12 of the pair's first block
  float2* Mb = M + size_t(b) * lay.stride;
  const size_t lda = size_t(lay.lda);
  const int tid = threadIdx.x;
  // The block's composed row moves (dst, src; every dst >= k) on these columns.  Each block row is read
  // straight from its source row; a row moved below the block is staged and written back.  At most NB rows
  // land below the block: each of the block's NB pivot steps moves at most one row out of it.
  __shared__ int src_of[NB];     // source row of block row i, or -1 when the row stays
  __shared__ int2 below[NB];     // (dst, src) of the moves with dst >= k + kb
  __shared__ int nbelow;
  const size_t pidx = size_t(b) * w.npanels + k / NB;
  const int np = w.nperm[pidx];
  const int2* pm = w.perm + pidx * (2 * NB);
  for (int i = tid; i < NB; i += 256) src_of[i] = -1;
  if (tid == 0) nbelow = 0;
  const float4* src = reinterpret_cast<const float4*>(linv + size_t(b) * NB * NB);
  if (kprev < 0)
    for (int idx = tid; idx < NB * NB / 2; idx += 256) reinterpret_cast<float4*>(Li)[idx] = src[idx];
  __syncthreads();
  for (int i = tid; i < np; i += 256) {
    const int2 mv = pm[i];
    if (mv.x < k + kb) {
      src_of[mv.x - k] = mv.y;
    } else {
      const int q = atomicAdd(&nbelow, 1);
      if (q < NB) below[q] = mv;
    }
  }
  __syncthreads();
  const int nbw = min(nbelow, NB);
  for (int idx = tid; idx < NB * kLtN; idx += 256) {
    const int i = idx % NB, c = idx / NB;
    const int sr = i < kb ? (src_of[i] >= 0 ? src_of[i] : k + i) : -1;
    Bt[i * kLtN + c] = (sr >= 0 && c < ncols) ? Mb[size_t(sr) + lda * size_t(cb + c)] : make_float2(0.f, 0.f);
  }
  for (int idx = tid; idx < nbw * ncols; idx += 256) {
    const int q = idx % nbw, c = idx / nbw;
    Bw[q * kLtN + c] = Mb[size_t(below[q].y) + lda * size_t(cb + c)];
  }
  __syncthreads();  // every source is read before any row is written
  for (int idx = tid; idx < nbw * ncols; idx += 256) {
    const int q = idx % nbw, c = idx / nbw;
    Mb[size_t(below[q].x) + lda * size_t(cb + c)] = Bw[q * kLtN + c];
  }
  // rows r0 .. r0 + 7 of column `col`
  const int col = tid & 31, r0 = (tid >> 5) * 8;
  if (kprev >= 0) {
    // the deferred update by the pair's first block: Li <- L21prev, Bw <- U12prev (once the rows moved
    // below the block have left it)
    __syncthreads();
    float2* Up = Bw;
    for (int idx = tid; idx < NB * NB; idx += 256) {
      const int i = idx % NB, j = idx / NB;
      Li[i + NB * j] = i < kb ? Mb[size_t(k + i) + lda * size_t(kprev + j)] : make_float2(0.f, 0.f);
    }
    for (int idx = tid; idx < NB * kLtN; idx += 256) {
      const int j = idx % NB, c = idx / NB;
      Up[j * kLtN + c] = c < ncols ? Mb[size_t(kprev + j) + lda * size_t(cb + c)] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 d[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) d[q] = Bt[(r0 + q) * kLtN + col];
    for (int j = 0; j < NB; ++j) {
      const float2 uv = Up[j * kLtN + col];
      const float4* lr = reinterpret_cast<const float4*>(Li + r0 + NB * j);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 l2 = lr[q];
        cfms(d[2 * q], make_float2(l2.x, l2.y), uv);
        cfms(d[2 * q + 1], make_float2(l2.z, l2.w), uv);
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; ++q) Bt[(r0 + q) * kLtN + col] = d[q];
    for (int idx = tid; idx < NB * NB / 2; idx += 256) reinterpret_cast<float4*>(Li)[idx] = src[idx];
  }
  __syncthreads();
  // L11^-1 is lower triangular, so j <= r0 + 7
  float2 acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = make_float2(0.f, 0.f);
  const int jend = min(kb, r0 + 8);
  for (int j = 0; j < jend; ++j) {
    const float2 bv = Bt[j * kLtN + col];
    const float4* lr = reinterpret_cast<const float4*>(Li + r0 + NB * j);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 l2 = lr[q];
      cfma(acc[2 * q], make_float2(l2.x, l2.y), bv);
      cfma(acc[2 * q + 1], make_float2(l2.z, l2.w), bv);
    }
  }
  if (col < ncols)
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (r0 + q < kb) Mb[size_t(k + r0 + q) + lda * size_t(cb + col)] = acc[q];
}

// One warp per RHS column: X[k:k+kb] = U11^-1 Y[k:k+kb] (bottom-up).
template <typename T, int NB>
__global__ void __launch_bounds__(256) rhs_upper_kernel(BatchLayout lay, int k, cplx<T>* __restrict__ M,
                                                        const int* skip) {
  using C = cplx<T>;
  const int b = blockIdx.y;
  if (skip && skip[b]) return;
  __shared__ C U11[NB][NB + 1];
  const int n = lay.n;
  const int kb = min(NB, n - k);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  C* Mb = M + size_t(b) * lay.stride;
  for (int idx = threadIdx.x; idx < kb * kb; idx += blockDim.x) {
    const int r = idx % kb, c = idx / kb;
    U11[r][c] = Mb[size_t(k + r) + size_t(lay.lda) * (k + c)];
  }
  __syncthreads();
  const int col = n + blockIdx.x * (blockDim.x / 32) + wid;
  if (col >= n + lay.m) return;
  C* colp = Mb + size_t(lay.lda) * col;
  constexpr int kRows = (NB + 31) / 32;
  C x[kRows];
#pragma unroll
  for (int t = 0; t < kRows; ++t) {
    const int i = lane + 32 * t;
    x[t] = i < kb ? colp[k + i] : mk<T>(T(0), T(0));
  }
  for (int p = kb - 1; p >= 0; --p) {
    const int owner_t = p >> 5, owner_l = p & 31;
#pragma unroll
    for (int t = 0; t < kRows; ++t)
      if (t == owner_t && lane == owner_l) {
        const C d = U11[p][p];
        x[t] = (d.x == T(0) && d.y == T(0)) ? mk<T>(T(0), T(0)) : cdiv(x[t], d);
      }
    C xp = mk<T>(T(0), T(0));
#pragma unroll
    for (int t = 0; t < kRows; ++t) {
      const T re = __shfl_sync(0xffffffffu, x[t].x, owner_l);
      const T im = __shfl_sync(0xffffffffu, x[t].y, owner_l);
      if (t == owner_t) { xp.x = re; xp.y = im; }
    }
#pragma unroll
    for (int t = 0; t < kRows; ++t) {
      const int i = lane + 32 * t;
      if (i < p) cfms(x[t], U11[i][p], xp);
    }
  }
#pragma unroll
  for (int t = 0; t < kRows; ++t) {
    const int i = lane + 32 * t;
    if (i < kb) colp[k + i] = x[t];
  }
}

// C[r_begin:r_end, c_begin:c_end] -= M[rows, ka:ka+kb] * M[ka:ka+kb, cols]
// Thread tile TM x TN complex, CTA tile (16*TM) x (16*TN), 256 threads.
template <typename T, int TM, int TN, int KMAX>
__global__ void __launch_bounds__(256) gemm_update_kernel(BatchLayout lay, int r_begin, int r_end, int c_begin,
                                                          int c_end, int ka, int kb, cplx<T>* __restrict__ M,
                                                          const int* skip) {
  using C = cplx<T>;
  constexpr int BM = 16 * TM, BN = 16 * TN;
  const int b = blockIdx.z;
  if (skip && skip[b]) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* As = reinterpret_cast<C*>(smraw);   // [KMAX][BM]
  C* Bs = As + KMAX * BM;                // [KMAX][BN]
  const int r0 = r_begin + blockIdx.x * BM;
  const int c0 = c_begin + blockIdx.y * BN;
  if (r0 >= r_end || c0 >= c_end) return;
  C* Mb = M + size_t(b) * lay.stride;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < kb * BM; idx += 256) {
    const int r = idx % BM, kk = idx / BM;
    As[kk * BM + r] = (r0 + r < r_end) ? Mb[size_t(r0 + r) + size_t(lay.lda) * (ka + kk)] : mk<T>(T(0), T(0));
  }
  for (int idx = tid; idx < kb * BN; idx += 256) {
    const int kk = idx % kb, c = idx / kb;
    Bs[kk * BN + c] = (c0 + c < c_end) ? Mb[size_t(ka + kk) + size_t(lay.lda) * (c0 + c)] : mk<T>(T(0), T(0));
  }
  __syncthreads();
  const int tx = tid & 15, ty = tid >> 4;
  C acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int jj = 0; jj < TN; ++jj) acc[i][jj] = mk<T>(T(0), T(0));
  for (int kk = 0; kk < kb; ++kk) {
    C a[TM], bb[TN];
#pragma unroll
    for (int i = 0; i < TM; ++i) a[i] = As[kk * BM + ty + 16 * i];
#pragma unroll
    for (int jj = 0; jj < TN; ++jj) bb[jj] = Bs[kk * BN + tx + 16 * jj];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int jj = 0; jj < TN; ++jj) cfma(acc[i][jj], a[i], bb[jj]);
  }
#pragma unroll
  for (int jj = 0; jj < TN; ++jj) {
    const int c = c0 + tx + 16 * jj;
    if (c >= c_end) continue;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int r = r0 + ty + 16 * i;
      if (r >= r_end) continue;
      C* p = Mb + size_t(r) + size_t(lay.lda) * c;
      C v = *p;
      v.x -= acc[i][jj].x;
      v.y -= acc[i][jj].y;
      *p = v;
    }
  }
}

template <typename T>
__global__ void absorber_solve_kernel(BatchLayout lay, const cplx<T>* __restrict__ M, double2* __restrict__ gg,
                                      const int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smraw[];
  double2* U = reinterpret_cast<double2*>(smraw);  // m x m
  const int b = blockIdx.x;
  const int n = lay.n, m = lay.m, r0 = n - m;
  const cplx<T>* Mb = M + size_t(b) * lay.stride;
  for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
    const int r = idx % m, c = idx / m;
    const cplx<T> u = Mb[size_t(r0 + r) + size_t(lay.lda) * (r0 + c)];
    U[r + m * c] = make_double2(double(u.x), double(u.y));
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (c >= m) return;
  double2* out = gg + size_t(b) * m * m + size_t(m) * c;
  for (int r = 0; r < m; ++r) {
    const cplx<T> y = Mb[size_t(r0 + r) + size_t(lay.lda) * (n + c)];
    out[r] = make_double2(double(y.x), double(y.y));
  }
  const bool bad = status && status[b] != kDevOk;
  for (int r = m - 1; r >= 0; --r) {
    double2 v = out[r];
    for (int p = r + 1; p < m; ++p) cfms(v, U[r + m * p], out[p]);
    const double2 d = U[r + m * r];
    out[r] = (bad || (d.x == 0.0 && d.y == 0.0)) ? make_double2(0.0, 0.0) : cdiv(v, d);
  }
}

// ---------------------------------------------------------------------------
// FP64 refinement kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* p, double v) {
  atomicMax(p, static_cast<unsigned long long>(__double_as_longlong(v)));
}

// R = B - A X.  A and B are stored as hi/lo float pairs (float4 per complex
// entry, exact to about 2^-48) and X in FP64; the products are accumulated in
// double-float on the FP32 pipes (GB300's FP64 rate is a small fraction of its
// FP32 rate).
//
// x (FP64) -> (hi.re, hi.im, lo.re, lo.im) once per residual, so that the
// residual CTAs read a ready split instead of each converting all of x.
__global__ void split_x_kernel(BatchLayout lay, const double2* __restrict__ X64, float4* __restrict__ Xs,
                               const int* skip) {
  const int b = blockIdx.y;
  if (skip && skip[b]) return;
  const size_t base = size_t(b) * lay.lda * lay.m;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < lay.n * lay.m; idx += gridDim.x * blockDim.x) {
    const int r = idx % lay.n, c = idx / lay.n;
    const size_t i = base + size_t(r) + size_t(lay.lda) * c;
    Xs[i] = split_hi_lo(X64[i]);
  }
}

// r = b - A x in double-float: 64 rows per CTA, each thread two rows (r, r + 32)
// and kCols right-hand sides (columns cg, cg + 8, ...), so that every a and x
// value read from shared memory feeds several complex MACs.
constexpr int kRdRows = 64, kRdK = 32;

// kGroups warps, one column group each (columns cg, cg + kGroups, ...), so
// that kCols x kGroups covers the right-hand sides with little padding (25 as
// 5 x 5, 9 as 3 x 3).
template <int kCols, int kGroups>
__global__ void __launch_bounds__(32 * kGroups) residual_df_kernel(BatchLayout lay, const float4* __restrict__ Ms,
                                                                   const float4* __restrict__ Xsp,
                                                                   double2* __restrict__ R, unsigned long long* rnorm,
                                                                   unsigned long long* bnorm, const int* skip) {
  constexpr int BR = kRdRows, BK = kRdK, XW = kCols * kGroups, kThreads = 32 * kGroups;
  const int b = blockIdx.y;
  if (skip && skip[b]) return;
  extern __shared__ float4 rd_sm[];
  float4* As = rd_sm;            // [BK][BR]
  float4* Xs = rd_sm + BK * BR;  // [BK][XW]
  const int n = lay.n, m = lay.m;
  const int r0 = blockIdx.x * BR;
  const float4* A = Ms + size_t(b) * lay.stride;
  const float4* X = Xsp + size_t(b) * lay.lda * m;
  double2* Rb = R + size_t(b) * lay.lda * m;
  const int tid = threadIdx.x, rp = tid & 31, cg = tid >> 5;
  df acc[2][kCols][2];
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int q = 0; q < kCols; ++q) acc[h][q][0] = acc[h][q][1] = {0.f, 0.f};
  for (int k0 = 0; k0 < n; k0 += BK) {
    const int kk_n = min(BK, n - k0);
    __syncthreads();
    for (int idx = tid; idx < BK * BR; idx += kThreads) {
      const int r = idx % BR, kk = idx / BR;
      As[kk * BR + r] = (r0 + r < n && kk < kk_n) ? A[size_t(r0 + r) + size_t(lay.lda) * (k0 + kk)]
                                                  : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int idx = tid; idx < BK * XW; idx += kThreads) {
      const int kk = idx % BK, c = idx / BK;
      Xs[kk * XW + c] = (kk < kk_n && c < m) ? X[size_t(k0 + kk) + size_t(lay.lda) * c] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    for (int kk = 0; kk < kk_n; ++kk) {
      const float4 a0 = As[kk * BR + rp], a1 = As[kk * BR + rp + 32];
#pragma unroll
      for (int q = 0; q < kCols; ++q) {
        const float4 x = Xs[kk * XW + cg + kGroups * q];
        dot2_mac(acc[0][q][0], a0.x, a0.z, x.x, x.z);    // re += a.re x.re
        dot2_mac(acc[0][q][0], -a0.y, -a0.w, x.y, x.w);  // re -= a.im x.im
        dot2_mac(acc[0][q][1], a0.x, a0.z, x.y, x.w);    // im += a.re x.im
        dot2_mac(acc[0][q][1], a0.y, a0.w, x.x, x.z);    // im += a.im x.re
        dot2_mac(acc[1][q][0], a1.x, a1.z, x.x, x.z);
        dot2_mac(acc[1][q][0], -a1.y, -a1.w, x.y, x.w);
        dot2_mac(acc[1][q][1], a1.x, a1.z, x.y, x.w);
        dot2_mac(acc[1][q][1], a1.y, a1.w, x.x, x.z);
      }
    }
  }
  double rmax = 0.0, bmax = 0.0;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int row = r0 + rp + 32 * h;
    if (row >= n) continue;
#pragma unroll
    for (int q = 0; q < kCols; ++q) {
      const int c = cg + kGroups * q;
      if (c >= m) continue;
      const double2 bv = join_hi_lo(A[size_t(row) + size_t(lay.lda) * (n + c)]);
      const double ax = double(acc[h][q][0].hi) + double(acc[h][q][0].lo);
      const double ay = double(acc[h][q][1].hi) + double(acc[h][q][1].lo);
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
  if ((tid & 31) == 0) {
    atomic_max_nonneg(rnorm + b, rmax);
    atomic_max_nonneg(bnorm + b, bmax);
  }
}

__device__ __forceinline__ double norm_scale(const unsigned long long* rnorm, int b) {
  const double r = __longlong_as_double(static_cast<long long>(rnorm[b]));
  return r > 0.0 ? r : 1.0;
}

__global__ void residual_to_rhs32_kernel(BatchLayout lay, const double2* __restrict__ R,
                                         const unsigned long long* rnorm, float2* __restrict__ M32, const int* skip) {
  const int b = blockIdx.y;
  if (skip && skip[b]) return;
  const int n = lay.n, m = lay.m;
  const double inv = 1.0 / norm_scale(rnorm, b);
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n * m; idx += gridDim.x * blockDim.x) {
    const int r = idx % n, c = idx / n;
    const double2 v = R[size_t(b) * lay.lda * m + size_t(r) + size_t(lay.lda) * c];
    M32[size_t(b) * lay.stride + size_t(r) + size_t(lay.lda) * (n + c)] = make_float2(float(v.x * inv), float(v.y * inv));
  }
}

__global__ void accumulate_correction_kernel(BatchLayout lay, const float2* __restrict__ M32,
                                             const unsigned long long* rnorm, double2* __restrict__ X64, int init,
                                             const int* skip, unsigned long long* dnorm, unsigned long long* xnorm) {
  const int b = blockIdx.y;
  if (skip && skip[b]) return;
  const int n = lay.n, m = lay.m;
  const double sc = init ? 1.0 : norm_scale(rnorm, b);
  double dmax = 0.0, xmax = 0.0;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n * m; idx += gridDim.x * blockDim.x) {
    const int r = idx % n, c = idx / n;
    const float2 d = M32[size_t(b) * lay.stride + size_t(r) + size_t(lay.lda) * (n + c)];
    double2& x = X64[size_t(b) * lay.lda * m + size_t(r) + size_t(lay.lda) * c];
    const double2 dd = make_double2(double(d.x) * sc, double(d.y) * sc);
    if (init) x = dd;
    else { x.x += dd.x; x.y += dd.y; }
    dmax = fmax(dmax, cabs1(dd));
    xmax = fmax(xmax, cabs1(x));
  }
  if (!dnorm) return;
  for (int off = 16; off > 0; off >>= 1) {
    dmax = fmax(dmax, __shfl_down_sync(0xffffffffu, dmax, off));
    xmax = fmax(xmax, __shfl_down_sync(0xffffffffu, xmax, off));
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_nonneg(dnorm + b, dmax);
    atomic_max_nonneg(xnorm + b, xmax);
  }
}

// Stopping rule of the refinement, per system not yet finished (done == 0):
// record relres = |r| / |b| of this step's residual and count the step.  The
// corrections shrink geometrically, |d_k+1| ~ rho |d_k| with rho = |d_k| /
// |d_k-1| (the initial solve counts as d_0 = x), so the error left after
// applying d_k is about |d_k|^2 / |d_k-1|.  Stop with done = 1 when that
// estimate, or the correction itself, is within tol |x|; stop with done = 2
// when the corrections stop shrinking (|d| > 0.5 |d_prev|): such systems go
// to the FP64 LU.
__global__ void ir_check_kernel(int batch, const unsigned long long* rnorm, const unsigned long long* bnorm,
                                const unsigned long long* dnorm, const unsigned long long* xnorm, double tol,
                                int* done, int* iters, double* relres, double* dprev) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch || done[b]) return;
  auto v = [](const unsigned long long* p, int i) { return __longlong_as_double(static_cast<long long>(p[i])); };
  const double r = v(rnorm, b), bn = v(bnorm, b), d = v(dnorm, b), x = v(xnorm, b);
  relres[b] = bn > 0.0 ? r / bn : r;
  const int it = iters[b]++;
  const double prev = it > 0 ? dprev[b] : x;
  if (d <= tol * x || d * d <= tol * x * prev) done[b] = 1;
  else if (it > 0 && d > 0.5 * prev) done[b] = 2;
  dprev[b] = d;
}

__global__ void extract_absorber_kernel(BatchLayout lay, const double2* __restrict__ X64, double2* __restrict__ gg) {
  const int b = blockIdx.x;
  const int n = lay.n, m = lay.m;
  for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
    const int r = idx % m, c = idx / m;
    gg[size_t(b) * m * m + idx] = X64[size_t(b) * lay.lda * m + size_t(n - m + r) + size_t(lay.lda) * c];
  }
}

__global__ void copy_rhs64_kernel(BatchLayout lay, const double2* __restrict__ M64, double2* __restrict__ X64) {
  const int b = blockIdx.y;
  const int n = lay.n, m = lay.m;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n * m; idx += gridDim.x * blockDim.x) {
    const int r = idx % n, c = idx / n;
    X64[size_t(b) * lay.lda * m + size_t(r) + size_t(lay.lda) * c] =
        M64[size_t(b) * lay.stride + size_t(r) + size_t(lay.lda) * (n + c)];
  }
}

// In place: M (double2 per entry) -> hi/lo float4 per entry, and M32 <- hi.
__global__ void split_system_kernel(BatchLayout lay, double2* __restrict__ M, float2* __restrict__ M32) {
  const int b = blockIdx.y;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < lay.stride; i += size_t(gridDim.x) * blockDim.x) {
    const size_t g = size_t(b) * lay.stride + i;
    const float4 v = split_hi_lo(M[g]);
    reinterpret_cast<float4*>(M)[g] = v;
    M32[g] = make_float2(v.x, v.y);
  }
}

void launch_split_system(const BatchLayout& lay, int batch, double2* M, float2* M32, cudaStream_t s) {
  dim3 grid(256, unsigned(batch));
  count_launch();
  split_system_kernel<<<grid, 256, 0, s>>>(lay, M, M32);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// First panel configuration of width nb that fits the shared-memory budget:
// smallest cluster with the bookkeeping in shared memory, else with it in
// global scratch.
// The smallest cluster whose panel fits a CTA's shared memory, preferring
// panels of at most 100 KB within a portable cluster (two CTAs per SM:
// measured 3% faster elimination at n = 2256 than one CTA of up to 200 KB;
// 16-CTA clusters were slower) and falling back to 200 KB and 16 CTAs.
static bool fit_panel(int elem, int nb, int n, int& cluster, int& rpc, int& smem, int& pos_global,
                      bool global_first = false) {
  for (int pass = 0; pass < 2; ++pass)
    for (int g = global_first ? 1 : 0; g < (pass == 0 && !global_first ? 1 : 2); ++g)  // bookkeeping in global memory only as the last resort
      for (int cl = 1; cl <= (pass == 0 ? 8 : 16); cl *= 2) {
        const size_t budget = size_t(pass == 0 ? 100 : 200) * 1024;
        const int r = (n + cl - 1) / cl;
        const size_t bsz = panel_smem_any(elem, nb, r, n, g == 1);
        if (bsz <= budget) {
          cluster = cl;
          rpc = r;
          smem = int(bsz);
          pos_global = g;
          return true;
        }
      }
  return false;
}

template <typename T>
PanelConfig choose_panel(int n, int inner_pref) {
  PanelConfig pc;
  pc.cluster = 0;
  const bool forced = inner_pref == 16 || inner_pref == 32;
  if (sizeof(T) == 4 && ((inner_pref == 0 && n >= 512) || (forced && n >= 128))) {
    // two-level: 64-column blocks of 16- or 32-column cluster panels.  16 columns
    // halve the shared memory of a panel, and with the row bookkeeping in global
    // scratch a 4-CTA panel takes 72 KB per CTA, three CTAs per SM: about three
    // times as many panels (energies) are factored at once as with 32 columns
    // and the bookkeeping in shared memory.  The panel's column chain, not its
    // arithmetic, bounds it (measured at n = 2256: elimination 103.8 -> 90.8 ms).
    const int order[2] = {inner_pref == 32 ? 32 : 16, inner_pref == 32 ? 16 : 32};
    for (int iw : order)
      if (fit_panel(8, iw, n, pc.inner_cluster, pc.inner_rpc, pc.inner_smem, pc.inner_pos_global, iw == 16)) {
        pc.nb = 64;
        pc.inner_nb = iw;
        pc.cluster = pc.inner_cluster;
        pc.pos_global = pc.inner_pos_global;
        return pc;
      }
    return pc;
  }
  const int elem = int(sizeof(cplx<T>));
  const int widths[3] = {32, 16, sizeof(T) == 4 ? 16 : 8};
  for (int nb : widths)
    if (fit_panel(elem, nb, n, pc.cluster, pc.rpc_max, pc.smem, pc.pos_global)) {
      pc.nb = nb;
      return pc;
    }
  pc.cluster = 0;  // too large for one cluster
  return pc;
}

template <typename T, int NB>
static cudaError_t launch_panel(const PanelConfig& pc, const BatchLayout& lay, int batch, int k, cplx<T>* M,
                                const LuWork& w, cudaStream_t s) {
  auto kern = panel_kernel<T, NB>;
  cudaError_t err = ensure_smem_limit(reinterpret_cast<const void*>(kern), size_t(pc.smem));
  if (err != cudaSuccess) return err;
  if (pc.cluster > 8) {
    err = ensure_nonportable_clusters(reinterpret_cast<const void*>(kern));
    if (err != cudaSuccess) return err;
  }
  // the trailing rows shrink as k grows: the smallest cluster whose CTAs still hold them (same
  // shared memory, rpc_max rows each), so that late panels pay fewer or no cluster barriers
  int cl = pc.cluster;
  const int R = lay.n - k;
  while (cl > 1 && (R + cl / 2 - 1) / (cl / 2) <= pc.rpc_max) cl /= 2;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(cl), unsigned(batch), 1);
  cfg.blockDim = dim3(kPanelThreads, 1, 1);
  cfg.dynamicSmemBytes = size_t(pc.smem);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = unsigned(cl);
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  count_launch();
  return cudaLaunchKernelEx(&cfg, kern, lay, k, M, w, pc.rpc_max);
}

template <typename T, int NB, bool kSolve = true>
static void launch_rhs_lower(const BatchLayout& lay, int batch, int k, int c_begin, int c_end, cplx<T>* M,
                             const LuWork& w, const int* skip, cudaStream_t s) {
  const int ncols = c_end - c_begin;
  if (ncols <= 0) return;
  const int per_cta = 8 * kRhsColsPerWarp;
  dim3 grid(unsigned((ncols + per_cta - 1) / per_cta), unsigned(batch));
  count_launch();
  rhs_lower_kernel<T, NB, kSolve><<<grid, 256, 0, s>>>(lay, k, c_begin, c_end, M, w, skip);
}

// Composes the row moves of the P inner panels of an outer block into one
// gather list: after all of them, row d holds the original row
// f(d) = src_0(src_1(...src_{P-1}(d))).  One CTA of 128 threads per matrix,
// the lists in shared memory (P * 2 * IW <= 128 entries).
__global__ void __launch_bounds__(128) compose_moves_kernel(int k, int iw, int P, LuWork w_out, LuWork w_in) {
  const int b = blockIdx.x;
  __shared__ int2 mv[128];
  __shared__ int cntl[4];
  __shared__ int cnt;
  const int per = 2 * iw, p0 = k / iw;
  const int t = threadIdx.x;
  if (t < P) cntl[t] = w_in.nperm[size_t(b) * w_in.npanels + p0 + t];
  if (t == 0) cnt = 0;
  __syncthreads();
  {
    const int p = t / per, e = t % per;
    if (p < P && e < cntl[p]) mv[t] = w_in.perm[(size_t(b) * w_in.npanels + p0 + p) * per + e];
  }
  __syncthreads();
  int2* out = w_out.perm + (size_t(b) * w_out.npanels + k / 64) * 128;
  const int p = t / per, e = t % per;
  int d = -1;
  if (p < P && e < cntl[p]) {
    d = mv[t].x;
    for (int q = 0; q < p && d >= 0; ++q)  // a row moved by an earlier panel is handled there
      for (int x = 0; x < cntl[q]; ++x)
        if (mv[q * per + x].x == d) { d = -1; break; }
  }
  if (d >= 0) {
    int f = d;
    for (int q = P - 1; q >= 0; --q)
      for (int x = 0; x < cntl[q]; ++x)
        if (mv[q * per + x].x == f) { f = mv[q * per + x].y; break; }
    if (f != d) {
      const int slot = atomicAdd(&cnt, 1);
      if (slot < 128) out[slot] = make_int2(d, f);
    }
  }
  __syncthreads();
  if (t == 0) w_out.nperm[size_t(b) * w_out.npanels + k / 64] = min(cnt, 128);
}

template <typename T, int TM, int TN, int KMAX>
static void launch_gemm(const BatchLayout& lay, int batch, int r_begin, int r_end, int c_begin, int c_end, int ka,
                        int kb, cplx<T>* M, const int* skip, cudaStream_t s) {
  constexpr int BM = 16 * TM, BN = 16 * TN;
  const int rows = r_end - r_begin, cols = c_end - c_begin;
  if (rows <= 0 || cols <= 0 || kb <= 0) return;
  const size_t smem = size_t(KMAX) * (BM + BN) * sizeof(cplx<T>);
  auto kern = gemm_update_kernel<T, TM, TN, KMAX>;
  ensure_smem_limit(reinterpret_cast<const void*>(kern), smem);
  dim3 grid(unsigned((rows + BM - 1) / BM), unsigned((cols + BN - 1) / BN), unsigned(batch));
  count_launch();
  kern<<<grid, 256, smem, s>>>(lay, r_begin, r_end, c_begin, c_end, ka, kb, M, skip);
}

template <typename T>
static void gemm_any(int nb, const BatchLayout& lay, int batch, int r_begin, int r_end, int c_begin, int c_end, int ka,
                     int kb, cplx<T>* M, const int* skip, cudaStream_t s) {
  // Skinny right-hand sides (m columns) use a narrow tile; KMAX = panel width.
  const bool skinny = (c_end - c_begin) <= 32;
#define RFX_GEMM(TM, TN, K) launch_gemm<T, TM, TN, K>(lay, batch, r_begin, r_end, c_begin, c_end, ka, kb, M, skip, s)
  if (sizeof(T) == 8) {
    switch (nb) {
      case 64: skinny ? RFX_GEMM(4, 2, 64) : RFX_GEMM(4, 4, 64); break;
      case 32: skinny ? RFX_GEMM(4, 2, 32) : RFX_GEMM(4, 4, 32); break;
      case 16: skinny ? RFX_GEMM(4, 2, 16) : RFX_GEMM(4, 4, 16); break;
      default: skinny ? RFX_GEMM(4, 2, 8) : RFX_GEMM(4, 4, 8); break;
    }
  } else {
    switch (nb) {
      case 64: skinny ? RFX_GEMM(8, 2, 64) : RFX_GEMM(8, 4, 64); break;
      case 32: skinny ? RFX_GEMM(8, 2, 32) : RFX_GEMM(8, 4, 32); break;
      default: skinny ? RFX_GEMM(8, 2, 16) : RFX_GEMM(8, 4, 16); break;
    }
  }
#undef RFX_GEMM
}

template <typename T, bool kSolve = true>
static void rhs_lower_any(int nb, const BatchLayout& lay, int batch, int k, int c_begin, int c_end, cplx<T>* M,
                          const LuWork& w, const int* skip, cudaStream_t s) {
  switch (nb) {
    case 64: launch_rhs_lower<T, 64, kSolve>(lay, batch, k, c_begin, c_end, M, w, skip, s); break;
    case 32: launch_rhs_lower<T, 32, kSolve>(lay, batch, k, c_begin, c_end, M, w, skip, s); break;
    case 16: launch_rhs_lower<T, 16, kSolve>(lay, batch, k, c_begin, c_end, M, w, skip, s); break;
    default:
      if constexpr (sizeof(T) == 8) launch_rhs_lower<T, 8, kSolve>(lay, batch, k, c_begin, c_end, M, w, skip, s);
      break;
  }
}

// Cluster panel of width nb: FP32 uses 32 / 16, FP64 32 / 16 / 8.
template <typename T>
static cudaError_t panel_any(const PanelConfig& pc, int nb, const BatchLayout& lay, int batch, int k, cplx<T>* M,
                             const LuWork& w, cudaStream_t s) {
  if (nb == 32) return launch_panel<T, 32>(pc, lay, batch, k, M, w, s);
  if (nb == 16) return launch_panel<T, 16>(pc, lay, batch, k, M, w, s);
  if constexpr (sizeof(T) == 8) {
    if (nb == 8) return launch_panel<T, 8>(pc, lay, batch, k, M, w, s);
  }
  return cudaErrorInvalidValue;
}

// FP32 elimination with two-level blocking: each 64-column outer block is
// factored as P = 64 / IW cluster panels of width IW (32, or 16 for large n),
// which keeps the on-chip panel footprint small enough for many matrices per
// wave; inside the block each panel updates the block's remaining columns
// (rank-IW), and its row moves are applied to the earlier panels' L columns,
// so that the block's L is in one row order.  The panels' moves are composed,
// and the trailing matrix (right-hand sides included) gets one K = 64 update:
// on the tensor cores when operand images are available, else on CUDA cores.
//
// Paired blocks (pc.pair128, tensor cores): the blocks are taken two at a
// time, a = [k, k + 64) and b = [k + 64, k + 128).  Block a's update reaches
// only b's columns (K = 64 over 64 columns); b is factored with its moves also
// applied to a's L; b's block row gets a's deferred update inside the
// L11^-1 product (rhs_lower_tile_kernel, kprev = k); and one K = 128 update
// covers everything beyond the pair.  Each trailing entry is read and written
// once per pair instead of once per block, which halves the traffic of the
// dominant kernel for the same flops.
static cudaError_t lu_eliminate_two_level(const PanelConfig& pc, const BatchLayout& lay, int batch, float2* M,
                                          const LuWork& w, cudaStream_t s) {
  const int n = lay.n, col_end = lay.n + lay.m, iw = pc.inner_nb;
  if (pc.nb != 64 || w.nb != 64 || (iw != 32 && iw != 16) || !w.perm_in) return cudaErrorInvalidValue;
  PanelConfig pin;
  pin.nb = iw;
  pin.cluster = pc.inner_cluster;
  pin.rpc_max = pc.inner_rpc;
  pin.smem = pc.inner_smem;
  pin.pos_global = pc.inner_pos_global;
  LuWork wi = w;
  wi.perm = w.perm_in;
  wi.nperm = w.nperm_in;
  wi.nb = iw;
  wi.npanels = panel_count(n, iw);
  if (!pin.pos_global) wi.pos_scratch = nullptr;
  const bool pair = pc.pair128 && w.pair128 && w.tc_images && w.linv;
  // the inner panels of block [k, k + kb); their row moves also reach the L columns [l_begin, k)
  auto factor_block = [&](int k, int kb, int l_begin) -> cudaError_t {
    int P = 0;
    for (int ki = k; ki < k + kb; ki += iw, ++P) {
      const int kbi = min(iw, k + kb - ki);
      cudaError_t err = panel_any<float>(pin, iw, lay, batch, ki, M, wi, s);
      if (err != cudaSuccess) return err;
      if (ki > l_begin) rhs_lower_any<float, false>(iw, lay, batch, ki, l_begin, ki, M, wi, nullptr, s);  // moves on earlier L
      if (ki + kbi < k + kb) {
        // the block's remaining columns: this panel's moves and L11, then its rank-IW update
        rhs_lower_any<float>(iw, lay, batch, ki, ki + kbi, k + kb, M, wi, nullptr, s);
        gemm_any<float>(iw, lay, batch, ki + kbi, n, ki + kbi, k + kb, ki, kbi, M, nullptr, s);
      }
    }
    count_launch();
    compose_moves_kernel<<<batch, 128, 0, s>>>(k, iw, P, w, wi);
    return cudaSuccess;
  };
  // the block row of block [k, k + kb) for every column beyond it: moves, then U12 = L11^-1 (P A12)
  auto block_row = [&](int k, int kb, int kprev) {
    if (!w.linv) {
      launch_rhs_lower<float, 64>(lay, batch, k, k + kb, col_end, M, w, nullptr, s);
      return;
    }
    count_launch();
    unit_lower_inverse_kernel<<<batch, 256, 0, s>>>(lay, k, M, w.linv);
    const int ncols = col_end - (k + kb);
    if (ncols > 0) {
      constexpr int smem = (64 * 64 + 2 * 64 * kLtN) * int(sizeof(float2));
      ensure_smem_limit(reinterpret_cast<const void*>(rhs_lower_tile_kernel), size_t(smem));
      count_launch();
      rhs_lower_tile_kernel<<<dim3(unsigned((ncols + kLtN - 1) / kLtN), unsigned(batch)), 256, smem, s>>>(
          lay, k, k + kb, col_end, M, w, w.linv, kprev);
    }
  };
  auto update = [&](int k, int kb, int c_end) {
    if (w.tc_images) tc_trailing_update(lay, batch, k, kb, c_end, M, w.tc_images, w.tc_err, nullptr, w.tc_wait_polls,
                                        w.tc_spans, s);
    else gemm_any<float>(64, lay, batch, k + kb, n, k + kb, c_end, k, kb, M, nullptr, s);
  };
  for (int k = 0; k < n; k += pair ? 128 : 64) {
    const int kb = min(64, n - k);
    cudaError_t err = factor_block(k, kb, k);
    if (err != cudaSuccess) return err;
    block_row(k, kb, -1);
    const int k2 = k + kb;
    if (!pair || k2 >= n) {
      update(k, kb, col_end);
    } else {
      const int kb2 = min(64, n - k2);
      update(k, kb, k2 + kb2);              // block a into block b's columns only
      err = factor_block(k2, kb2, k);       // b's moves also on a's L
      if (err != cudaSuccess) return err;
      block_row(k2, kb2, k);                // with a's deferred update of b's block row
      update(k, kb + kb2, col_end);         // K = kb + kb2 over everything beyond the pair
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

template <typename T>
cudaError_t lu_eliminate(const PanelConfig& pc, const BatchLayout& lay, int batch, cplx<T>* M, const LuWork& w,
                         cudaStream_t s) {
  const int n = lay.n, col_end = lay.n + lay.m;
  if (pc.cluster <= 0 || w.nb != pc.nb) return cudaErrorInvalidValue;
  if constexpr (sizeof(T) == 4) {
    if (pc.inner_nb) return lu_eliminate_two_level(pc, lay, batch, M, w, s);
  }
  LuWork wl = w;
  if (!pc.pos_global) wl.pos_scratch = nullptr;
  for (int k = 0; k < n; k += pc.nb) {
    const int kb = min(pc.nb, n - k);
    cudaError_t err = panel_any<T>(pc, pc.nb, lay, batch, k, M, wl, s);
    if (err != cudaSuccess) return err;
    rhs_lower_any<T>(pc.nb, lay, batch, k, k + kb, col_end, M, wl, nullptr, s);
    if constexpr (sizeof(T) == 4) {
      if (w.tc_images) {
        tc_trailing_update(lay, batch, k, kb, col_end, M, w.tc_images, w.tc_err, nullptr, w.tc_wait_polls, w.tc_spans, s);
        err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        continue;
      }
    }
    gemm_any<T>(pc.nb, lay, batch, k + kb, n, k + kb, col_end, k, kb, M, nullptr, s);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

template <typename T>
void lu_forward_rhs(const PanelConfig& pc, const BatchLayout& lay, int batch, cplx<T>* M, const LuWork& w,
                    const int* skip, cudaStream_t s) {
  const int n = lay.n, col_end = lay.n + lay.m;
  for (int k = 0; k < n; k += pc.nb) {
    const int kb = min(pc.nb, n - k);
    rhs_lower_any<T>(pc.nb, lay, batch, k, n, col_end, M, w, skip, s);
    gemm_any<T>(pc.nb, lay, batch, k + kb, n, n, col_end, k, kb, M, skip, s);
  }
}

template <typename T>
void lu_backward_rhs(const PanelConfig& pc, const BatchLayout& lay, int batch, cplx<T>* M, const int* skip,
                     cudaStream_t s) {
  const int n = lay.n, col_end = lay.n + lay.m;
  const int last = ((n - 1) / pc.nb) * pc.nb;
  dim3 grid(unsigned((lay.m + 7) / 8), unsigned(batch));
  for (int k = last; k >= 0; k -= pc.nb) {
    const int kb = min(pc.nb, n - k);
    count_launch();
    switch (pc.nb) {
      case 64: rhs_upper_kernel<T, 64><<<grid, 256, 0, s>>>(lay, k, M, skip); break;
      case 32: rhs_upper_kernel<T, 32><<<grid, 256, 0, s>>>(lay, k, M, skip); break;
      case 16: rhs_upper_kernel<T, 16><<<grid, 256, 0, s>>>(lay, k, M, skip); break;
      default:
        if constexpr (sizeof(T) == 8) rhs_upper_kernel<T, 8><<<grid, 256, 0, s>>>(lay, k, M, skip);
        break;
    }
    gemm_any<T>(pc.nb, lay, batch, 0, k, n, col_end, k, kb, M, skip, s);
  }
}

template <typename T>
void launch_absorber_solve(const BatchLayout& lay, int batch, const cplx<T>* M, double2* gg, const int* status,
                           cudaStream_t s) {
  const int threads = ((lay.m + 31) / 32) * 32;
  const size_t smem = size_t(lay.m) * lay.m * sizeof(double2);
  count_launch();
  absorber_solve_kernel<T><<<unsigned(batch), threads, smem, s>>>(lay, M, gg, status);
}

template <int kCols, int kGroups>
static void launch_residual_df(const BatchLayout& lay, int batch, const float4* Ms, const float4* Xs, double2* R,
                               unsigned long long* rnorm_bits, unsigned long long* bnorm_bits, const int* skip,
                               cudaStream_t s) {
  constexpr size_t smem = size_t(kRdK) * (kRdRows + kCols * kGroups) * sizeof(float4);
  ensure_smem_limit(reinterpret_cast<const void*>(residual_df_kernel<kCols, kGroups>), smem);
  dim3 grid(unsigned((lay.n + kRdRows - 1) / kRdRows), unsigned(batch));
  count_launch();
  residual_df_kernel<kCols, kGroups><<<grid, 32 * kGroups, smem, s>>>(lay, Ms, Xs, R, rnorm_bits, bnorm_bits, skip);
}

void launch_residual(const BatchLayout& lay, int batch, const float4* Ms, const double2* X64, float4* Xsplit,
                     double2* R, unsigned long long* rnorm_bits, unsigned long long* bnorm_bits, const int* skip,
                     cudaStream_t s, const ResidualTc* tc) {
  if (tc && launch_residual_tc(lay, batch, Ms, X64, *tc, R, rnorm_bits, bnorm_bits, skip, s)) return;
  {
    dim3 grid(unsigned(min(64, (lay.n * lay.m + 255) / 256)), unsigned(batch));
    count_launch();
    split_x_kernel<<<grid, 256, 0, s>>>(lay, X64, Xsplit, skip);
  }
  // column groups sized to the right-hand sides: 9 (lmax 2) and 25 (lmax 4) without padding
  if (lay.m <= 8) launch_residual_df<1, 8>(lay, batch, Ms, Xsplit, R, rnorm_bits, bnorm_bits, skip, s);
  else if (lay.m == 9) launch_residual_df<3, 3>(lay, batch, Ms, Xsplit, R, rnorm_bits, bnorm_bits, skip, s);
  else if (lay.m <= 16) launch_residual_df<2, 8>(lay, batch, Ms, Xsplit, R, rnorm_bits, bnorm_bits, skip, s);
  else if (lay.m <= 24) launch_residual_df<3, 8>(lay, batch, Ms, Xsplit, R, rnorm_bits, bnorm_bits, skip, s);
  else if (lay.m == 25) launch_residual_df<5, 5>(lay, batch, Ms, Xsplit, R, rnorm_bits, bnorm_bits, skip, s);
  else if (lay.m <= 32) launch_residual_df<4, 8>(lay, batch, Ms, Xsplit, R, rnorm_bits, bnorm_bits, skip, s);
  else launch_residual_df<8, 8>(lay, batch, Ms, Xsplit, R, rnorm_bits, bnorm_bits, skip, s);
}

void launch_residual_to_rhs32(const BatchLayout& lay, int batch, const double2* R,
                              const unsigned long long* rnorm_bits, float2* M32, const int* skip, cudaStream_t s) {
  dim3 grid(unsigned(min(64, (lay.n * lay.m + 255) / 256)), unsigned(batch));
  count_launch();
  residual_to_rhs32_kernel<<<grid, 256, 0, s>>>(lay, R, rnorm_bits, M32, skip);
}

void launch_accumulate_correction(const BatchLayout& lay, int batch, const float2* M32,
                                  const unsigned long long* rnorm_bits, double2* X64, bool init, const int* skip,
                                  unsigned long long* dnorm_bits, unsigned long long* xnorm_bits, cudaStream_t s) {
  dim3 grid(unsigned(min(64, (lay.n * lay.m + 255) / 256)), unsigned(batch));
  count_launch();
  accumulate_correction_kernel<<<grid, 256, 0, s>>>(lay, M32, rnorm_bits, X64, init ? 1 : 0, skip, dnorm_bits,
                                                    xnorm_bits);
}

void launch_ir_check(int batch, const unsigned long long* rnorm_bits, const unsigned long long* bnorm_bits,
                     const unsigned long long* dnorm_bits, const unsigned long long* xnorm_bits, double tol,
                     int* done, int* iters, double* relres, double* dprev, cudaStream_t s) {
  count_launch();
  ir_check_kernel<<<unsigned((batch + 127) / 128), 128, 0, s>>>(batch, rnorm_bits, bnorm_bits, dnorm_bits, xnorm_bits,
                                                                tol, done, iters, relres, dprev);
}

__global__ void extract_blocks_kernel(BatchLayout lay, const double2* __restrict__ X64, const SolvedBlock* blocks,
                                      int nblocks, int per_matrix, double2* __restrict__ out,
                                      const int* __restrict__ status) {
  const int b = blockIdx.x;
  const bool bad = status && status[b] != kDevOk;
  for (int q = 0; q < nblocks; ++q) {
    const SolvedBlock bl = blocks[q];
    for (int idx = threadIdx.x; idx < bl.size * bl.size; idx += blockDim.x) {
      const int r = idx % bl.size, c = idx / bl.size;
      out[size_t(b) * per_matrix + bl.pack + idx] =
          bad ? make_double2(0.0, 0.0) : X64[size_t(b) * lay.lda * lay.m + size_t(bl.row + r) + size_t(lay.lda) * (bl.col + c)];
    }
  }
}

void launch_extract_blocks(const BatchLayout& lay, int batch, const double2* X64, const SolvedBlock* blocks, int nblocks,
                           int per_matrix, double2* out, const int* status, cudaStream_t s) {
  count_launch();
  extract_blocks_kernel<<<unsigned(batch), 256, 0, s>>>(lay, X64, blocks, nblocks, per_matrix, out, status);
}

void launch_extract_absorber(const BatchLayout& lay, int batch, const double2* X64, double2* gg, cudaStream_t s) {
  count_launch();
  extract_absorber_kernel<<<unsigned(batch), 256, 0, s>>>(lay, X64, gg);
}

void launch_copy_rhs64(const BatchLayout& lay, int batch, const double2* M64, double2* X64, cudaStream_t s) {
  dim3 grid(unsigned(min(64, (lay.n * lay.m + 255) / 256)), unsigned(batch));
  count_launch();
  copy_rhs64_kernel<<<grid, 256, 0, s>>>(lay, M64, X64);
}

template PanelConfig choose_panel<double>(int, int);
template PanelConfig choose_panel<float>(int, int);
template cudaError_t lu_eliminate<double>(const PanelConfig&, const BatchLayout&, int, double2*, const LuWork&,
                                          cudaStream_t);
template cudaError_t lu_eliminate<float>(const PanelConfig&, const BatchLayout&, int, float2*, const LuWork&,
                                         cudaStream_t);
template void lu_forward_rhs<double>(const PanelConfig&, const BatchLayout&, int, double2*, const LuWork&, const int*,
                                     cudaStream_t);
template void lu_forward_rhs<float>(const PanelConfig&, const BatchLayout&, int, float2*, const LuWork&, const int*,
                                    cudaStream_t);
template void lu_backward_rhs<double>(const PanelConfig&, const BatchLayout&, int, double2*, const int*,
                                      cudaStream_t);
template void lu_backward_rhs<float>(const PanelConfig&, const BatchLayout&, int, float2*, const int*, cudaStream_t);
template void launch_absorber_solve<double>(const BatchLayout&, int, const double2*, double2*, const int*,
                                            cudaStream_t);
template void launch_absorber_solve<float>(const BatchLayout&, int, const float2*, double2*, const int*,
                                           cudaStream_t);

}  // namespace rfx
