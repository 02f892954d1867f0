// Allocation-free dense FP64 solve on caller-owned device buffers.
//
// The same elimination as refeff_complex_lu_solve_batched with the FP64 LU
// form (cluster-panel LU of the augmented [A | B] system, then the backward
// sweep), but its scratch -- the padded augmented systems, the pivot and
// row-move lists, the per-system status words -- lives in one file-scope
// device array instead of memory obtained from cudaMalloc.  Nothing here
// allocates: no cudaMalloc / cudaFree, no allocating library routine.
//
// Set-up: the first call made on a device (the calling thread's current
// device) looks the array's address up with cudaGetSymbolAddress and keeps it
// for that device; later calls reuse it.  Calls are asynchronous on the
// caller's stream and share the one array per device, so two calls whose
// work overlaps on the GPU race on it: order them (one stream, or events).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/refeff_fms.h"
#include "batched_lu.cuh"
#include "fms_plan.cuh"

namespace rfx {
namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[REFEFF_FMS_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mu;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Copies the caller's column-major systems into the padded augmented layout
// (rows n..lda-1 zero) and clears the status and first-zero-pivot words,
// which the elimination only raises.
__global__ void noalloc_pack_kernel(BatchLayout lay, const double2* __restrict__ A, const double2* __restrict__ B,
                                    double2* __restrict__ M, int* __restrict__ status, int* __restrict__ info) {
  const int b = blockIdx.y, n = lay.n, m = lay.m;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    status[b] = 0;
    info[b] = 0;
  }
  const size_t total = size_t(lay.lda) * size_t(n + m);
  double2* Mb = M + size_t(b) * lay.stride;
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total; idx += size_t(gridDim.x) * blockDim.x) {
    const int r = int(idx % size_t(lay.lda));
    const int c = int(idx / size_t(lay.lda));
    double2 v = make_double2(0.0, 0.0);
    if (r < n) v = c < n ? A[size_t(b) * n * n + size_t(r) + size_t(n) * c]
                         : B[size_t(b) * n * m + size_t(r) + size_t(n) * (c - n)];
    Mb[idx] = v;
  }
}

__device__ int public_status(int dev) {
  switch (dev) {
    case kDevOk: return REFEFF_FMS_OK;
    case kDevSingular: return REFEFF_FMS_ERR_SINGULAR_MATRIX;
    case kDevNonfinite: return REFEFF_FMS_ERR_NONFINITE_INPUT;
    case kDevZeroRho: return REFEFF_FMS_ERR_ZERO_RHO;
    case kDevNotConverged: return REFEFF_FMS_ERR_NOT_CONVERGED;
    default: return REFEFF_FMS_ERR_CUDA;
  }
}

// X (column-major, leading dimension n) <- solution columns of the augmented
// system; per-system status and first zero pivot in the public codes.
__global__ void noalloc_unpack_kernel(BatchLayout lay, const double2* __restrict__ M, double2* __restrict__ X,
                                      const int* __restrict__ status, const int* __restrict__ info,
                                      int32_t* __restrict__ status_out, int32_t* __restrict__ pivot_out) {
  const int b = blockIdx.y, n = lay.n, m = lay.m;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (status_out) status_out[b] = public_status(status[b]);
    if (pivot_out) pivot_out[b] = info[b];
  }
  const double2* Mb = M + size_t(b) * lay.stride + size_t(lay.lda) * n;
  for (size_t idx = size_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < size_t(n) * m;
       idx += size_t(gridDim.x) * blockDim.x) {
    const int r = int(idx % size_t(n)), c = int(idx / size_t(n));
    X[size_t(b) * n * m + idx] = Mb[size_t(r) + size_t(lay.lda) * c];
  }
}

// The array's device address for the current device, looked up on first use.
int scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return REFEFF_FMS_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return REFEFF_FMS_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return REFEFF_FMS_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_ptr[dev]);
  return REFEFF_FMS_OK;
}

}  // namespace
}  // namespace rfx

using namespace rfx;

extern "C" int refeff_complex_lu_solve_device_noalloc(int n, int m, int batch, const refeff_complex128* d_A,
                                                      const refeff_complex128* d_B, refeff_complex128* d_X,
                                                      int32_t* d_status, int32_t* d_pivot, void* stream) {
  if (n <= 0 || m <= 0 || m > 64 || batch <= 0 || batch > 65535 || !d_A || !d_B || !d_X)
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  BatchLayout lay;
  lay.n = n;
  lay.m = m;
  lay.lda = (n + 31) / 32 * 32;
  lay.stride = size_t(lay.lda) * size_t(n + m);
  const PanelConfig pc = choose_panel<double>(n);
  if (pc.cluster <= 0 || pc.pos_global) return REFEFF_FMS_ERR_UNSUPPORTED;
  const int npanels = panel_count(n, pc.nb);
  // scratch carve-up, each piece 256-byte aligned
  const size_t off_ipiv = align256(size_t(batch) * lay.stride * sizeof(double2));
  const size_t off_perm = off_ipiv + align256(size_t(batch) * n * sizeof(int));
  const size_t off_nperm = off_perm + align256(size_t(batch) * npanels * 2 * pc.nb * sizeof(int2));
  const size_t off_status = off_nperm + align256(size_t(batch) * npanels * sizeof(int));
  const size_t off_info = off_status + align256(size_t(batch) * sizeof(int));
  const size_t need = off_info + align256(size_t(batch) * sizeof(int));
  if (need > size_t(REFEFF_FMS_NOALLOC_SCRATCH_BYTES)) return REFEFF_FMS_ERR_SCRATCH_LIMIT;

  unsigned char* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  double2* M = reinterpret_cast<double2*>(base);
  LuWork w;
  w.ipiv = reinterpret_cast<int*>(base + off_ipiv);
  w.perm = reinterpret_cast<int2*>(base + off_perm);
  w.nperm = reinterpret_cast<int*>(base + off_nperm);
  w.status = reinterpret_cast<int*>(base + off_status);
  w.info = reinterpret_cast<int*>(base + off_info);
  w.nb = pc.nb;
  w.npanels = npanels;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  const unsigned gx = unsigned(std::min<size_t>(256, (size_t(lay.lda) * (n + m) + 255) / 256));
  count_launch();
  noalloc_pack_kernel<<<dim3(gx, unsigned(batch)), 256, 0, s>>>(lay, reinterpret_cast<const double2*>(d_A),
                                                               reinterpret_cast<const double2*>(d_B), M, w.status,
                                                               w.info);
  if (cudaGetLastError() != cudaSuccess) return REFEFF_FMS_ERR_CUDA;
  if (lu_eliminate<double>(pc, lay, batch, M, w, s) != cudaSuccess) return REFEFF_FMS_ERR_CUDA;
  lu_backward_rhs<double>(pc, lay, batch, M, nullptr, s);
  const unsigned ux = unsigned(std::min<size_t>(256, (size_t(n) * m + 255) / 256));
  count_launch();
  noalloc_unpack_kernel<<<dim3(ux, unsigned(batch)), 256, 0, s>>>(lay, M, reinterpret_cast<double2*>(d_X), w.status,
                                                                 w.info, d_status, d_pivot);
  return cudaGetLastError() == cudaSuccess ? REFEFF_FMS_OK : REFEFF_FMS_ERR_CUDA;
}
