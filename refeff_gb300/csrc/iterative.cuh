// Iterative FMS forms (FEFF minv != 0): launch interface.
#pragma once
#include <cuda_runtime.h>

#include "fms_plan.cuh"

namespace rfx {

// Vectors of n entries each solver keeps per (energy, column) in its scratch slab.
constexpr int kIterVectors = 10;

struct IterArgs {
  int n = 0, m = 0;
  size_t lda = 0, stride = 0;
  const void* W = nullptr;     // system per energy, cplx<R>, column-major (lda, stride)
  const void* grow = nullptr;  // the solved blocks' rows of G0 per energy, cplx<R>, m x n column-major
  void* scratch = nullptr;     // batch * m * kIterVectors * n cplx<R>
  const SolvedBlock* blocks = nullptr;  // the potentials' blocks; their columns partition [0, m)
  int nblocks = 0;
  int gg_per = 0;              // packed blocks per energy
  double2* gg = nullptr;       // batch * gg_per, block q at gg[e][pack + row + size * col]
  int* status = nullptr;       // per energy, DevStatus (max-reduced)
  const int* skip = nullptr;
  double tol1 = 0.0;
};

// Builds W from G0 (in place for FP64, into W32 for the Complex32 form), then
// solves every column of the solved blocks (lay.m in all) of every energy with
// the `minv` method (1 ggbi, 2 ggrm, 3 gggm, else ggtf) and writes each block
// of gg.  t: per-state T table (band 0, band 1) in device order; partner: spin
// partner per state (-1 none).  grow / scratch are sized for double even in
// the FP32 form.
cudaError_t launch_iterative(bool fp64, int minv, const BatchLayout& lay, int batch, double2* G0, float2* W32,
                             const double2* t, const int* partner, double tol1, double tol2, void* grow, void* scratch,
                             const SolvedBlock* blocks, int nblocks, int gg_per, double2* gg, int* status,
                             cudaStream_t s);

}  // namespace rfx
