// Learned diagonal preconditioner for the BiCGSTAB form.
//
// A small MLP maps, per (energy, atom), the wave number, the atom's t_l, and
// the shell geometry around the atom (neighbour counts, mean distances and
// the neighbours' mean t_l in three shells) to the channel diagonal of the
// atom's block of (I - G0 T)^-1, predicted as a deviation from 1.  The
// BiCGSTAB form applies it as a right preconditioner.  Training and inference
// run here on the GPU: forward, backward and Adam kernels over row-major
// FP32 activations; the gradients are checked against a CPU restatement in
// the tests.  There is no counterpart in the reference (its BiCGSTAB form,
// crates/refeff-core/src/fms/internals/iterative.rs:181-254, is
// unpreconditioned).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/refeff_fms.h"
#include "cplx.cuh"
#include "host_internal.h"
#include "precond_mlp.cuh"

namespace rfx {
namespace {

constexpr int kTile = 16;

// C = act(opA(A) opB(B) + bias), or C += opA(A) opB(B) when `accumulate`.
// opA(A)(i, k) = TA ? A[k * lda + i] : A[i * lda + k]; likewise for B.
template <bool TA, bool TB>
__global__ void gemm_kernel(int M, int N, int K, const float* __restrict__ A, int lda, const float* __restrict__ B,
                            int ldb, float* __restrict__ C, int ldc, const float* __restrict__ bias, bool act_tanh,
                            bool accumulate) {
  __shared__ float As[kTile][kTile + 1], Bs[kTile][kTile + 1];
  const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile;
  const int i = blockIdx.y * kTile + ty, j = blockIdx.x * kTile + tx;
  float acc = 0.f;
  for (int k0 = 0; k0 < K; k0 += kTile) {
    {
      const int ai = blockIdx.y * kTile + ty, ak = k0 + tx;  // As[ty][tx] = opA(ai, ak)
      float v = 0.f;
      if (ai < M && ak < K) v = TA ? A[size_t(ak) * lda + ai] : A[size_t(ai) * lda + ak];
      As[ty][tx] = v;
      const int bk = k0 + ty, bj = blockIdx.x * kTile + tx;  // Bs[ty][tx] = opB(bk, bj)
      float w = 0.f;
      if (bk < K && bj < N) w = TB ? B[size_t(bj) * ldb + bk] : B[size_t(bk) * ldb + bj];
      Bs[ty][tx] = w;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTile; ++kk) acc = fmaf(As[ty][kk], Bs[kk][tx], acc);
    __syncthreads();
  }
  if (i >= M || j >= N) return;
  float* c = C + size_t(i) * ldc + j;
  if (accumulate) {
    *c += acc;
    return;
  }
  if (bias) acc += bias[j];
  *c = act_tanh ? tanhf(acc) : acc;
}

template <bool TA, bool TB>
void gemm(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc, const float* bias,
          bool act_tanh, bool accumulate, cudaStream_t s) {
  if (M <= 0 || N <= 0) return;
  const dim3 grid(unsigned((N + kTile - 1) / kTile), unsigned((M + kTile - 1) / kTile));
  count_launch();
  gemm_kernel<TA, TB><<<grid, kTile * kTile, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, act_tanh, accumulate);
}

// dy = 2 (y - t) / (S O); loss += sum (y - t)^2 / (S O)
__global__ void mse_grad_kernel(size_t total, const float* __restrict__ y, const float* __restrict__ t,
                                float* __restrict__ dy, double* loss) {
  __shared__ double red[8];
  double part = 0.0;
  const double scale = 1.0 / double(total);
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const float d = y[i] - t[i];
    dy[i] = float(2.0 * double(d) * scale);
    part += double(d) * d * scale;
  }
  for (int off = 16; off > 0; off >>= 1) part += __shfl_down_sync(0xffffffffu, part, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t2 = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) t2 += red[w];
    atomicAdd(loss, t2);
  }
}

// d = d * (1 - h^2) (tanh derivative), in place
__global__ void tanh_back_kernel(size_t total, const float* __restrict__ h, float* __restrict__ d) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x)
    d[i] *= 1.f - h[i] * h[i];
}

// db[j] = sum_s d[s][j]
__global__ void colsum_kernel(int S, int N, const float* __restrict__ d, float* __restrict__ db) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  float acc = 0.f;
  for (int s = 0; s < S; ++s) acc += d[size_t(s) * N + j];
  db[j] = acc;
}

__global__ void adam_kernel(size_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = v;
    p[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
  }
}

unsigned grid_for(size_t total, unsigned threads) {
  return unsigned(std::min<size_t>((total + threads - 1) / threads, 4096));
}

struct Offsets {
  size_t W1, b1, W2, b2, W3, b3;
};
Offsets offsets(const MlpShape& sh) {
  Offsets o;
  o.W1 = 0;
  o.b1 = o.W1 + size_t(sh.H) * sh.F;
  o.W2 = o.b1 + sh.H;
  o.b2 = o.W2 + size_t(sh.H) * sh.H;
  o.W3 = o.b2 + sh.H;
  o.b3 = o.W3 + size_t(sh.O) * sh.H;
  return o;
}

// t = (e^{2 i delta} - 1) / (2 i)
__device__ __forceinline__ float2 t_of_phase(double2 d) {
  const double a = exp(-2.0 * d.y);
  double sn, cs;
  sincos(2.0 * d.x, &sn, &cs);
  const double zr = a * cs, zi = a * sn;
  return make_float2(float(zi / 2.0), float(-(zr - 1.0) / 2.0));
}

__global__ void features_kernel(int batch, int N, int L, int nsp, int npot, int F, const double2* __restrict__ k,
                                const double2* __restrict__ xph, const int* __restrict__ atom_pot,
                                const float* __restrict__ shell_info, const float* __restrict__ shell_pots,
                                float* __restrict__ X) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= batch * N) return;
  const int b = idx / N, d = idx % N, D = 2 * L + 1, nl = L + 1;
  float* f = X + size_t(idx) * F;
  const double2 kk = k[size_t(b) * nsp];
  f[0] = float(kk.x);
  f[1] = float(kk.y);
  const double2* xe = xph + size_t(b) * nsp * D * npot;
  auto tl = [&](int p, int l) { return t_of_phase(xe[size_t(nsp) * (size_t(l + L) + size_t(D) * p)]); };
  const int pd = atom_pot[d];
  for (int l = 0; l < nl; ++l) {
    const float2 t = tl(pd, l);
    f[2 + 2 * l] = t.x;
    f[3 + 2 * l] = t.y;
  }
  int o = 2 + 2 * nl;
  for (int j = 0; j < kShells; ++j) {
    f[o++] = shell_info[(size_t(d) * kShells + j) * 2];
    f[o++] = shell_info[(size_t(d) * kShells + j) * 2 + 1];
    const float* fr = shell_pots + (size_t(d) * kShells + j) * npot;
    for (int l = 0; l < nl; ++l) {
      float2 acc = make_float2(0.f, 0.f);
      for (int p = 0; p < npot; ++p)
        if (fr[p] != 0.f) {
          const float2 t = tl(p, l);
          acc.x += fr[p] * t.x;
          acc.y += fr[p] * t.y;
        }
      f[o++] = acc.x;
      f[o++] = acc.y;
    }
  }
}

// Energies whose E - E_ref = Re((k a0)^2) / 2 Hartree (wave number of spin 0)
// lies outside [e_lo, e_hi] eV get D = 1: no preconditioning there.
__global__ void scatter_diag_kernel(int batch, int N, int L, int nsp, int lda, const int* __restrict__ atom_off,
                                    const int* __restrict__ atom_lmax, const float* __restrict__ Y,
                                    const double2* __restrict__ k, double e_lo, double e_hi, float2* __restrict__ D) {
  const int per = nsp * (L + 1) * (L + 1), O = 2 * (L + 1) * (L + 1);
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)batch * N * per) return;
  const int q = int(idx % per);
  const int d = int((idx / per) % N);
  const int b = int(idx / per / N);
  const int lm = atom_lmax[d];
  if (q >= nsp * (lm + 1) * (lm + 1)) return;
  const int c = q / nsp;
  const float* y = Y + (size_t(b) * N + d) * O;
  bool on = true;
  if (k) {
    constexpr double kBohr = 0.529177249, kHartreeEv = 27.211396;
    const double2 kk = k[size_t(b) * nsp];
    const double e_ev = 0.5 * (kk.x * kk.x - kk.y * kk.y) * kBohr * kBohr * kHartreeEv;
    on = e_ev >= e_lo && e_ev <= e_hi;
  }
  D[size_t(b) * lda + atom_off[d] + q] = on ? make_float2(1.f + y[2 * c], y[2 * c + 1]) : make_float2(1.f, 0.f);
}

}  // namespace

// ---------------------------------------------------------------------------
// host-side pieces used by the plan
// ---------------------------------------------------------------------------
int feature_count(int L) { return 2 + 2 * (L + 1) + kShells * (2 + 2 * (L + 1)); }
int output_count(int L, int kind) {
  const int C = (L + 1) * (L + 1);
  return kind == kPrecondBlock ? 2 * C * C : 2 * C;
}

ShellTables shell_tables(int N, int npot, const float* pos, const int* pot) {
  static const double edges[kShells + 1] = {0.0, 2.9, 3.7, 4.6};
  ShellTables t;
  t.info.assign(size_t(N) * kShells * 2, 0.f);
  t.pots.assign(size_t(N) * kShells * npot, 0.f);
  std::vector<double> cnt(static_cast<size_t>(kShells)), sum(static_cast<size_t>(kShells));
  std::vector<double> pc(static_cast<size_t>(kShells) * npot);
  for (int d = 0; d < N; ++d) {
    std::fill(cnt.begin(), cnt.end(), 0.0);
    std::fill(sum.begin(), sum.end(), 0.0);
    std::fill(pc.begin(), pc.end(), 0.0);
    for (int e = 0; e < N; ++e) {
      if (e == d) continue;
      const double dx = double(pos[3 * e]) - pos[3 * d], dy = double(pos[3 * e + 1]) - pos[3 * d + 1],
                   dz = double(pos[3 * e + 2]) - pos[3 * d + 2];
      const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
      for (int j = 0; j < kShells; ++j)
        if (r >= edges[j] && r < edges[j + 1]) {
          cnt[size_t(j)] += 1.0;
          sum[size_t(j)] += r;
          pc[size_t(j) * npot + pot[e]] += 1.0;
        }
    }
    for (int j = 0; j < kShells; ++j) {
      const size_t base = size_t(d) * kShells + j;
      t.info[base * 2] = float(cnt[size_t(j)] / 12.0);
      t.info[base * 2 + 1] = cnt[size_t(j)] > 0 ? float(sum[size_t(j)] / cnt[size_t(j)] / 5.0) : 0.f;
      for (int p = 0; p < npot; ++p)
        t.pots[base * npot + p] = cnt[size_t(j)] > 0 ? float(pc[size_t(j) * npot + p] / cnt[size_t(j)]) : 0.f;
    }
  }
  return t;
}

void launch_features(int batch, int N, int L, int nsp, int npot, const double2* k, const double2* xph,
                     const int* atom_pot, const float* shell_info, const float* shell_pots, float* X, cudaStream_t s) {
  const int total = batch * N;
  count_launch();
  features_kernel<<<(total + 127) / 128, 128, 0, s>>>(batch, N, L, nsp, npot, feature_count(L), k, xph, atom_pot,
                                                      shell_info, shell_pots, X);
}

// Dblk[(b N + atom) C^2 + q C + q'] = delta(q, q') + (Y[b*N + atom][2 (q C + q')] + i Y[..][2 (q C + q') + 1])
// for q, q' below the atom's channel count, zero beyond it; identity outside the energy window.
__global__ void scatter_block_kernel(int batch, int N, int L, const int* __restrict__ atom_lmax,
                                     const float* __restrict__ Y, const double2* __restrict__ k, double e_lo,
                                     double e_hi, float2* __restrict__ B) {
  const int C = (L + 1) * (L + 1), CC = C * C;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)batch * N * CC) return;
  const int e = int(idx % CC), d = int((idx / CC) % N), b = int(idx / CC / N);
  const int q = e / C, q2 = e % C;
  const int cnt = (atom_lmax[d] + 1) * (atom_lmax[d] + 1);
  bool on = true;
  if (k) {
    constexpr double kBohr = 0.529177249, kHartreeEv = 27.211396;
    const double2 kk = k[b];
    const double e_ev = 0.5 * (kk.x * kk.x - kk.y * kk.y) * kBohr * kBohr * kHartreeEv;
    on = e_ev >= e_lo && e_ev <= e_hi;
  }
  float2 v = make_float2(q == q2 ? 1.f : 0.f, 0.f);
  if (q >= cnt || q2 >= cnt) v = make_float2(0.f, 0.f);
  else if (on) {
    const float* y = Y + (size_t(b) * N + d) * 2 * CC + 2 * e;
    v.x += y[0];
    v.y += y[1];
  }
  B[idx] = v;
}

void launch_scatter_block(int batch, int N, int L, const int* atom_lmax, const float* Y, const double2* k, double e_lo,
                          double e_hi, float2* B, cudaStream_t s) {
  const int C = (L + 1) * (L + 1);
  const long long total = (long long)batch * N * C * C;
  count_launch();
  scatter_block_kernel<<<unsigned((total + 255) / 256), 256, 0, s>>>(batch, N, L, atom_lmax, Y, k, e_lo, e_hi, B);
}

void launch_scatter_diag(int batch, int N, int L, int nsp, int lda, const int* atom_off, const int* atom_lmax,
                         const float* Y, const double2* k, double e_lo, double e_hi, float2* D, cudaStream_t s) {
  const long long total = (long long)batch * N * nsp * (L + 1) * (L + 1);
  count_launch();
  scatter_diag_kernel<<<unsigned((total + 255) / 256), 256, 0, s>>>(batch, N, L, nsp, lda, atom_off, atom_lmax, Y, k,
                                                                    e_lo, e_hi, D);
}

cudaError_t MlpScratch::ensure(const MlpShape& sh, int S) {
  if (S <= capacity && sh.H == H && sh.O == O) return cudaSuccess;
  release();
  const size_t sh1 = size_t(S) * sh.H, so = size_t(S) * sh.O;
  cudaError_t e = cudaMalloc(&h1, sh1 * sizeof(float));
  if (!e) e = cudaMalloc(&h2, sh1 * sizeof(float));
  if (!e) e = cudaMalloc(&y, so * sizeof(float));
  if (!e) e = cudaMalloc(&d1, sh1 * sizeof(float));
  if (!e) e = cudaMalloc(&d2, sh1 * sizeof(float));
  if (!e) e = cudaMalloc(&dy, so * sizeof(float));
  if (!e) e = cudaMalloc(&loss, sizeof(double));
  if (e) {
    release();
    return e;
  }
  capacity = S;
  H = sh.H;
  O = sh.O;
  return cudaSuccess;
}

void MlpScratch::release() {
  for (float** p : {&h1, &h2, &y, &d1, &d2, &dy})
    if (*p) {
      cudaFree(*p);
      *p = nullptr;
    }
  if (loss) cudaFree(loss);
  loss = nullptr;
  capacity = 0;
}

cudaError_t mlp_forward(const MlpShape& sh, const float* P, int S, const float* X, MlpScratch& w, float* Y,
                        cudaStream_t s) {
  cudaError_t e = w.ensure(sh, S);
  if (e) return e;
  const Offsets o = offsets(sh);
  gemm<false, true>(S, sh.H, sh.F, X, sh.F, P + o.W1, sh.F, w.h1, sh.H, P + o.b1, true, false, s);
  gemm<false, true>(S, sh.H, sh.H, w.h1, sh.H, P + o.W2, sh.H, w.h2, sh.H, P + o.b2, true, false, s);
  gemm<false, true>(S, sh.O, sh.H, w.h2, sh.H, P + o.W3, sh.H, Y ? Y : w.y, sh.O, P + o.b3, false, false, s);
  return cudaGetLastError();
}

cudaError_t mlp_loss_grad(const MlpShape& sh, const float* P, int S, const float* X, const float* T, MlpScratch& w,
                          float* G, cudaStream_t s) {
  cudaError_t e = mlp_forward(sh, P, S, X, w, nullptr, s);
  if (e) return e;
  const Offsets o = offsets(sh);
  const size_t so = size_t(S) * sh.O, sh1 = size_t(S) * sh.H;
  cudaMemsetAsync(w.loss, 0, sizeof(double), s);
  count_launch();
  mse_grad_kernel<<<grid_for(so, 256), 256, 0, s>>>(so, w.y, T, w.dy, w.loss);
  // layer 3: dW3 = dy^T h2, db3 = colsum(dy), dh2 = dy W3
  cudaMemsetAsync(G, 0, sh.n_params() * sizeof(float), s);
  gemm<true, false>(sh.O, sh.H, S, w.dy, sh.O, w.h2, sh.H, G + o.W3, sh.H, nullptr, false, true, s);
  count_launch();
  colsum_kernel<<<(sh.O + 127) / 128, 128, 0, s>>>(S, sh.O, w.dy, G + o.b3);
  gemm<false, false>(S, sh.H, sh.O, w.dy, sh.O, P + o.W3, sh.H, w.d2, sh.H, nullptr, false, false, s);
  count_launch();
  tanh_back_kernel<<<grid_for(sh1, 256), 256, 0, s>>>(sh1, w.h2, w.d2);
  // layer 2
  gemm<true, false>(sh.H, sh.H, S, w.d2, sh.H, w.h1, sh.H, G + o.W2, sh.H, nullptr, false, true, s);
  count_launch();
  colsum_kernel<<<(sh.H + 127) / 128, 128, 0, s>>>(S, sh.H, w.d2, G + o.b2);
  gemm<false, false>(S, sh.H, sh.H, w.d2, sh.H, P + o.W2, sh.H, w.d1, sh.H, nullptr, false, false, s);
  count_launch();
  tanh_back_kernel<<<grid_for(sh1, 256), 256, 0, s>>>(sh1, w.h1, w.d1);
  // layer 1
  gemm<true, false>(sh.H, sh.F, S, w.d1, sh.H, X, sh.F, G + o.W1, sh.F, nullptr, false, true, s);
  count_launch();
  colsum_kernel<<<(sh.H + 127) / 128, 128, 0, s>>>(S, sh.H, w.d1, G + o.b1);
  return cudaGetLastError();
}

cudaError_t mlp_adam(size_t n, float* P, const float* G, float* m1, float* m2, int step, float lr, float b1, float b2,
                     float eps, cudaStream_t s) {
  const float c1 = 1.f - std::pow(b1, float(step)), c2 = 1.f - std::pow(b2, float(step));
  count_launch();
  adam_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, P, G, m1, m2, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

}  // namespace rfx

// ---------------------------------------------------------------------------
// C ABI: the model object
// ---------------------------------------------------------------------------
using namespace rfx;

struct refeff_fms_precond_model {
  refeff_fms_context* ctx = nullptr;
  int L = 0;
  int kind = kPrecondDiagonal;
  MlpShape shape;
  float* params = nullptr;
  float* grad = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  int step = 0;
  MlpScratch scratch;
  ~refeff_fms_precond_model() {
    cudaSetDevice(context_device(ctx));
    cudaStreamSynchronize(context_stream(ctx));
    for (float* p : {params, grad, m1, m2})
      if (p) cudaFree(p);
    scratch.release();
  }
};

namespace rfx {
const MlpShape* model_shape(const refeff_fms_precond_model* m) { return m ? &m->shape : nullptr; }
const float* model_params(const refeff_fms_precond_model* m) { return m ? m->params : nullptr; }
int model_lmax(const refeff_fms_precond_model* m) { return m ? m->L : -1; }
int model_kind(const refeff_fms_precond_model* m) { return m ? m->kind : kPrecondDiagonal; }
}  // namespace rfx

namespace rfx {
namespace {

// a device float buffer freed with its scope
struct DevFloats {
  float* p = nullptr;
  ~DevFloats() { if (p) cudaFree(p); }
};

uint64_t splitmix(uint64_t& x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

double uniform01(uint64_t& x) { return double(splitmix(x) >> 11) * (1.0 / 9007199254740992.0); }

int set_device(refeff_fms_precond_model* m) {
  return cudaSetDevice(context_device(m->ctx)) == cudaSuccess ? REFEFF_FMS_OK : REFEFF_FMS_ERR_CUDA;
}

}  // namespace
}  // namespace rfx

extern "C" int refeff_fms_precond_model_create_kind(refeff_fms_context* ctx, int lmax, int hidden, int kind,
                                                    unsigned long long seed, refeff_fms_precond_model** out) {
  if (!ctx || !out || lmax < 0 || lmax > 6 || hidden < 1 || hidden > 1024 ||
      (kind != kPrecondDiagonal && kind != kPrecondBlock) || (kind == kPrecondBlock && lmax > 4))
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  auto m = new refeff_fms_precond_model;
  m->ctx = ctx;
  m->L = lmax;
  m->kind = kind;
  m->shape.F = feature_count(lmax);
  m->shape.H = hidden;
  m->shape.O = output_count(lmax, kind);
  const size_t np = m->shape.n_params();
  if (set_device(m) || cudaMalloc(&m->params, np * sizeof(float)) || cudaMalloc(&m->grad, np * sizeof(float)) ||
      cudaMalloc(&m->m1, np * sizeof(float)) || cudaMalloc(&m->m2, np * sizeof(float))) {
    delete m;
    return REFEFF_FMS_ERR_OUT_OF_MEMORY;
  }
  // Glorot-uniform weights, zero biases; the last layer starts at zero so the
  // untrained model is the identity preconditioner
  std::vector<float> h(np, 0.f);
  uint64_t st = seed;
  const Offsets o = offsets(m->shape);
  auto fill = [&](size_t off, int fan_out, int fan_in) {
    const double a = std::sqrt(6.0 / double(fan_in + fan_out));
    for (size_t i = 0; i < size_t(fan_out) * fan_in; ++i) h[off + i] = float((2.0 * uniform01(st) - 1.0) * a);
  };
  fill(o.W1, m->shape.H, m->shape.F);
  fill(o.W2, m->shape.H, m->shape.H);
  cudaMemcpy(m->params, h.data(), np * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemset(m->m1, 0, np * sizeof(float));
  cudaMemset(m->m2, 0, np * sizeof(float));
  if (cudaGetLastError() != cudaSuccess) {
    delete m;
    return REFEFF_FMS_ERR_CUDA;
  }
  context_retain(ctx);
  *out = m;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_precond_model_create(refeff_fms_context* ctx, int lmax, int hidden, unsigned long long seed,
                                               refeff_fms_precond_model** out) {
  return refeff_fms_precond_model_create_kind(ctx, lmax, hidden, kPrecondDiagonal, seed, out);
}

extern "C" void refeff_fms_precond_model_destroy(refeff_fms_precond_model* m) {
  if (!m) return;
  refeff_fms_context* ctx = m->ctx;
  delete m;
  context_release(ctx);
}

extern "C" int refeff_fms_precond_model_query(const refeff_fms_precond_model* m, int* n_features, int* hidden,
                                              int* n_outputs, long long* n_params) {
  if (!m) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (n_features) *n_features = m->shape.F;
  if (hidden) *hidden = m->shape.H;
  if (n_outputs) *n_outputs = m->shape.O;
  if (n_params) *n_params = (long long)m->shape.n_params();
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_precond_get_params(const refeff_fms_precond_model* m, float* out) {
  if (!m || !out) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(context_device(m->ctx)) != cudaSuccess) return REFEFF_FMS_ERR_CUDA;
  return cudaMemcpy(out, m->params, m->shape.n_params() * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
             ? REFEFF_FMS_OK
             : REFEFF_FMS_ERR_CUDA;
}

extern "C" int refeff_fms_precond_set_params(refeff_fms_precond_model* m, const float* in) {
  if (!m || !in) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (set_device(m)) return REFEFF_FMS_ERR_CUDA;
  const size_t np = m->shape.n_params();
  for (size_t i = 0; i < np; ++i)
    if (!std::isfinite(in[i])) return REFEFF_FMS_ERR_NONFINITE_INPUT;
  if (cudaMemcpy(m->params, in, np * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return REFEFF_FMS_ERR_CUDA;
  cudaMemset(m->m1, 0, np * sizeof(float));
  cudaMemset(m->m2, 0, np * sizeof(float));
  m->step = 0;
  return cudaGetLastError() == cudaSuccess ? REFEFF_FMS_OK : REFEFF_FMS_ERR_CUDA;
}

namespace rfx {
namespace {
int upload(const float* host, size_t n, DevFloats& dev, cudaStream_t s) {
  if (cudaMalloc(&dev.p, std::max<size_t>(n, 1) * sizeof(float)) != cudaSuccess) return REFEFF_FMS_ERR_OUT_OF_MEMORY;
  return cudaMemcpyAsync(dev.p, host, n * sizeof(float), cudaMemcpyHostToDevice, s) == cudaSuccess ? REFEFF_FMS_OK
                                                                                                    : REFEFF_FMS_ERR_CUDA;
}
}  // namespace
}  // namespace rfx

extern "C" int refeff_fms_precond_loss_grad(refeff_fms_precond_model* m, int n_samples, const float* X, const float* T,
                                            double* loss, float* grad) {
  if (!m || n_samples <= 0 || !X || !T) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (set_device(m)) return REFEFF_FMS_ERR_CUDA;
  cudaStream_t s = context_stream(m->ctx);
  DevFloats dx, dt;
  int rc = upload(X, size_t(n_samples) * m->shape.F, dx, s);
  if (!rc) rc = upload(T, size_t(n_samples) * m->shape.O, dt, s);
  if (rc) return rc;
  if (mlp_loss_grad(m->shape, m->params, n_samples, dx.p, dt.p, m->scratch, m->grad, s) != cudaSuccess)
    return REFEFF_FMS_ERR_CUDA;
  double l = 0.0;
  if ((loss && cudaMemcpyAsync(&l, m->scratch.loss, sizeof(double), cudaMemcpyDeviceToHost, s)) ||
      (grad && cudaMemcpyAsync(grad, m->grad, m->shape.n_params() * sizeof(float), cudaMemcpyDeviceToHost, s)) ||
      cudaStreamSynchronize(s))
    return REFEFF_FMS_ERR_CUDA;
  if (loss) *loss = l;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_precond_predict(refeff_fms_precond_model* m, int n_samples, const float* X, float* Y) {
  if (!m || n_samples <= 0 || !X || !Y) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (set_device(m)) return REFEFF_FMS_ERR_CUDA;
  cudaStream_t s = context_stream(m->ctx);
  DevFloats dx, dy;
  int rc = upload(X, size_t(n_samples) * m->shape.F, dx, s);
  if (rc) return rc;
  if (cudaMalloc(&dy.p, size_t(n_samples) * m->shape.O * sizeof(float)) != cudaSuccess) return REFEFF_FMS_ERR_OUT_OF_MEMORY;
  if (mlp_forward(m->shape, m->params, n_samples, dx.p, m->scratch, dy.p, s) != cudaSuccess ||
      cudaMemcpyAsync(Y, dy.p, size_t(n_samples) * m->shape.O * sizeof(float), cudaMemcpyDeviceToHost, s) ||
      cudaStreamSynchronize(s))
    return REFEFF_FMS_ERR_CUDA;
  return REFEFF_FMS_OK;
}

namespace rfx {
namespace {
// rows idx[i] of src (rows of `width` floats) -> dst row i
__global__ void gather_rows_kernel(int rows, int width, const int* __restrict__ idx, const float* __restrict__ src,
                                   float* __restrict__ dst) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)rows * width) return;
  const int r = int(t / width), c = int(t % width);
  dst[t] = src[size_t(idx[r]) * width + c];
}
}  // namespace
}  // namespace rfx

extern "C" int refeff_fms_precond_train(refeff_fms_precond_model* m, int n_samples, const float* X, const float* T,
                                        int epochs, int batch_size, float learning_rate, unsigned long long seed,
                                        double* epoch_loss) {
  if (!m || n_samples <= 0 || !X || !T || epochs < 0 || batch_size <= 0 || !(learning_rate > 0.f))
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (set_device(m)) return REFEFF_FMS_ERR_CUDA;
  cudaStream_t s = context_stream(m->ctx);
  const MlpShape& sh = m->shape;
  const int B = std::min(batch_size, n_samples);
  DevFloats dx, dt, bx, bt;
  int* didx = nullptr;
  int rc = upload(X, size_t(n_samples) * sh.F, dx, s);
  if (!rc) rc = upload(T, size_t(n_samples) * sh.O, dt, s);
  if (rc) return rc;
  if (cudaMalloc(&bx.p, size_t(B) * sh.F * sizeof(float)) || cudaMalloc(&bt.p, size_t(B) * sh.O * sizeof(float)) ||
      cudaMalloc(&didx, size_t(n_samples) * sizeof(int)))
    return REFEFF_FMS_ERR_OUT_OF_MEMORY;
  std::vector<int> perm(static_cast<size_t>(n_samples));
  std::iota(perm.begin(), perm.end(), 0);
  uint64_t st = seed;
  double* dloss = nullptr;
  cudaMalloc(&dloss, sizeof(double) * size_t(std::max(epochs, 1)));
  cudaMemsetAsync(dloss, 0, sizeof(double) * size_t(std::max(epochs, 1)), s);
  int result = REFEFF_FMS_OK;
  for (int ep = 0; ep < epochs && result == REFEFF_FMS_OK; ++ep) {
    for (int i = n_samples - 1; i > 0; --i) std::swap(perm[size_t(i)], perm[size_t(splitmix(st) % uint64_t(i + 1))]);
    if (cudaMemcpyAsync(didx, perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice, s)) {
      result = REFEFF_FMS_ERR_CUDA;
      break;
    }
    for (int b0 = 0; b0 + B <= n_samples; b0 += B) {
      count_launch();
      gather_rows_kernel<<<unsigned((size_t(B) * sh.F + 255) / 256), 256, 0, s>>>(B, sh.F, didx + b0, dx.p, bx.p);
      count_launch();
      gather_rows_kernel<<<unsigned((size_t(B) * sh.O + 255) / 256), 256, 0, s>>>(B, sh.O, didx + b0, dt.p, bt.p);
      if (mlp_loss_grad(sh, m->params, B, bx.p, bt.p, m->scratch, m->grad, s) != cudaSuccess) {
        result = REFEFF_FMS_ERR_CUDA;
        break;
      }
      if (mlp_adam(sh.n_params(), m->params, m->grad, m->m1, m->m2, ++m->step, learning_rate, 0.9f, 0.999f, 1e-8f, s) !=
          cudaSuccess) {
        result = REFEFF_FMS_ERR_CUDA;
        break;
      }
    }
    if (epoch_loss) {
      // loss of the full training set with the epoch's parameters
      if (mlp_forward(sh, m->params, n_samples, dx.p, m->scratch, nullptr, s) != cudaSuccess) {
        result = REFEFF_FMS_ERR_CUDA;
        break;
      }
      cudaMemsetAsync(m->scratch.loss, 0, sizeof(double), s);
      count_launch();
      mse_grad_kernel<<<grid_for(size_t(n_samples) * sh.O, 256), 256, 0, s>>>(size_t(n_samples) * sh.O, m->scratch.y,
                                                                              dt.p, m->scratch.dy, m->scratch.loss);
      cudaMemcpyAsync(dloss + ep, m->scratch.loss, sizeof(double), cudaMemcpyDeviceToDevice, s);
    }
  }
  if (result == REFEFF_FMS_OK && epoch_loss && epochs > 0 &&
      (cudaMemcpyAsync(epoch_loss, dloss, sizeof(double) * size_t(epochs), cudaMemcpyDeviceToHost, s) ||
       cudaStreamSynchronize(s)))
    result = REFEFF_FMS_ERR_CUDA;
  cudaStreamSynchronize(s);
  cudaFree(dloss);
  cudaFree(didx);
  if (result == REFEFF_FMS_OK && cudaGetLastError() != cudaSuccess) result = REFEFF_FMS_ERR_CUDA;
  return result;
}
