// Batched right-preconditioned BiCGSTAB on the FP32 system matrices of a batch.
#pragma once
#include <cuda_runtime.h>

#include "fms_plan.cuh"

namespace rfx {

// Vectors kept per (matrix, column): x, r (also s), r-hat, p, v, p-hat, s-hat, t.
constexpr int kBicgVectors = 8;
// Doubles kept per (matrix, column): rho, alpha, omega, |b|^2, and accumulators.
constexpr int kBicgScalars = 16;
// Column slices of the matrix-vector product (partial products summed by the
// dot kernels): slices of at least 512 columns, at most 16, on the CUDA cores;
// slices of 256 columns on the tensor cores, whose FP32 accumulation is
// exact only for short sums.  bicg_slices gives the count for n.
constexpr int kBicgMaxSplit = 16;
constexpr int kBicgTcSliceCols = 256;
int bicg_slices(int n, bool tensor, int* chunk = nullptr);

struct BicgWork {
  float2* vec = nullptr;     // kBicgVectors * batch * lda * m
  double* sc = nullptr;      // batch * m * kBicgScalars
  int* state = nullptr;      // batch * m: 0 running, 1 converged, 2 breakdown
  int* done = nullptr;       // batch: every column finished
  int* iters = nullptr;      // batch: iterations of the slowest column
  int* active = nullptr;     // 1 int: matrices still running (host poll)
  float2* part = nullptr;    // (slices - 1) * batch * lda * m: partial products of the split product
  int* act = nullptr;        // batch: compacted list of running matrices
  int* tc_err = nullptr;     // 1 int: set when a wait of the tensor-core product gave up
  int tensor = 0;            // products on the tensor cores (up to 32 right-hand sides)
};

// Solves A X = B for every matrix of the batch whose skip flag is clear:
// A = the first n columns of M32, B = its last m columns, X written over B.
// Right preconditioner: diagonal D (batch * lda complex, NULL for none) or the
// block diagonal blk, i.e. BiCGSTAB on A P y = b, x = P y.  Stops a column when |r|_2 <= tol |b|_2;
// after max_iter iterations, or on a breakdown, the matrix's flag in
// `failed` is set to 2 (the caller's fallback marker) and its X is left as the
// last iterate.  The host polls the number of running matrices every
// `poll` iterations (one small device-to-host copy), so the call is not
// capturable into a CUDA graph.
// Block-diagonal right preconditioner: per matrix and atom a C x C block
// B[(b N + atom) C^2 + q C + q'] acting on the atom's states [atom_off[a],
// atom_off[a + 1]); state_atom[i] is the atom of state i (device order).
struct BlockPrecond {
  const float2* B = nullptr;
  const int* state_atom = nullptr;
  const int* atom_off = nullptr;
  int N = 0, C = 0;
};
// blk (nullable) replaces D when given.
cudaError_t bicgstab_solve(const BatchLayout& lay, int batch, float2* M32, const float2* D, const BlockPrecond* blk,
                           const BicgWork& w, double tol, int max_iter, int poll, const int* skip, int* failed,
                           cudaStream_t s);

}  // namespace rfx
