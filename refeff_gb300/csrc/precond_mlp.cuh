// Learned diagonal preconditioner for the BiCGSTAB form: a small MLP, its
// GPU training and inference kernels, and the per-atom features it reads.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "fms_plan.cuh"

struct refeff_fms_precond_model;  // the C ABI's model object (precond_mlp.cu)

namespace rfx {

// Three dense layers, F -> H -> H -> O, tanh after the first two.  Parameters
// are one float vector: W1[H][F], b1[H], W2[H][H], b2[H], W3[O][H], b3[O].
struct MlpShape {
  int F = 0, H = 0, O = 0;
  size_t n_params() const { return size_t(H) * F + H + size_t(H) * H + H + size_t(O) * H + O; }
};

// Device scratch for one forward (+ backward) pass over S samples.
struct MlpScratch {
  float *h1 = nullptr, *h2 = nullptr, *y = nullptr;   // S x H, S x H, S x O
  float *d1 = nullptr, *d2 = nullptr, *dy = nullptr;  // deltas, same shapes
  double* loss = nullptr;                             // 1
  int capacity = 0, H = 0, O = 0;  // sized for S <= capacity samples of this width
  cudaError_t ensure(const MlpShape& sh, int S);
  void release();
  ~MlpScratch() { release(); }
};

// Y = MLP(X): X S x F row-major, Y S x O.
cudaError_t mlp_forward(const MlpShape& sh, const float* params, int S, const float* X, MlpScratch& w, float* Y,
                        cudaStream_t s);
// Mean squared error against T (S x O) and its gradient (n_params floats,
// overwritten) by backpropagation; loss (double, device) overwritten.
cudaError_t mlp_loss_grad(const MlpShape& sh, const float* params, int S, const float* X, const float* T,
                          MlpScratch& w, float* grad, cudaStream_t s);
// One Adam step (bias-corrected, step >= 1).
cudaError_t mlp_adam(size_t n, float* params, const float* grad, float* m1, float* m2, int step, float lr, float beta1,
                     float beta2, float eps, cudaStream_t s);

// Per-atom shell tables of a cluster for the features (host side, device order).
constexpr int kShells = 3;
struct ShellTables {
  std::vector<float> info;  // [N][kShells][2]: neighbour count / 12, mean distance / 5 A
  std::vector<float> pots;  // [N][kShells][npot]: neighbour fraction per potential
};
ShellTables shell_tables(int N, int npot, const float* pos_dev_order, const int* pot_dev_order);
int feature_count(int L);
// Model kinds: the channel diagonal of each atom's block of A^-1, or the whole block.
constexpr int kPrecondDiagonal = 0, kPrecondBlock = 1;
int output_count(int L, int kind = kPrecondDiagonal);

// Features of every (energy, device atom): S = batch * N rows of feature_count(L).
// k: batch * nsp wave numbers; xph: batch * xph_per_energy phase shifts.
void launch_features(int batch, int N, int L, int nsp, int npot, const double2* k, const double2* xph,
                     const int* atom_pot, const float* shell_info, const float* shell_pots, float* X, cudaStream_t s);
// The model's shape, device parameters and the lmax its features are built for.
const MlpShape* model_shape(const refeff_fms_precond_model* m);
const float* model_params(const refeff_fms_precond_model* m);
int model_lmax(const refeff_fms_precond_model* m);
int model_kind(const refeff_fms_precond_model* m);

// D[b][state] = 1 + (Y[b*N + atom][2c] + i Y[..][2c+1]), c = channel of the state (spin-independent);
// with k (batch * nsp wave numbers), energies with E - E_ref outside [e_lo, e_hi] eV get D = 1.
void launch_scatter_diag(int batch, int N, int L, int nsp, int lda, const int* atom_off, const int* atom_lmax,
                         const float* Y, const double2* k, double e_lo, double e_hi, float2* D, cudaStream_t s);
// Block kind (one spin channel): Bblk[(b N + atom) C^2 + q C + q'] = I + the network's block, C = (L+1)^2,
// identity outside [e_lo, e_hi] eV (k: batch wave numbers), zero rows / columns beyond the atom's channels.
void launch_scatter_block(int batch, int N, int L, const int* atom_lmax, const float* Y, const double2* k, double e_lo,
                          double e_hi, float2* B, cudaStream_t s);

}  // namespace rfx
