// Host runtime behind include/refeff_fms.h: context, cluster preparation,
// plan construction (energy-independent tables resident in HBM), batched
// execution of the FMS solve on the GPU (captured as CUDA graphs), and the
// dense batched solve.
//
// Reference interfaces replaced here:
//   fms_yprep_cluster / sort_representative_atoms  crates/refeff-core/src/fms/cluster.rs:10-195
//   fms_real_space_plan / fms_driver_setup         crates/refeff-core/src/fms/driver.rs:4-140
//   construct_state_kets_with_limit                crates/refeff-core/src/state.rs:97-148
//   fms_real_space_spectrum                        crates/refeff-core/src/fms/driver.rs:231-239
//   fms_gg_section_values                          crates/refeff-engine/src/fms.rs:2004-2047
//   complex32_faer_lu_factor / _solve              crates/refeff-linalg/src/lu.rs:385-490
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "../../include/refeff_fms.h"
#include "batched_lu.cuh"
#include "bicgstab.cuh"
#include "precond_mlp.cuh"
#include "cplx.cuh"
#include "fms_plan.cuh"
#include "host_internal.h"
#include "iterative.cuh"

using namespace rfx;

namespace {
std::atomic<unsigned long long> g_launches{0};
// Bumped by every device (re)allocation and release of the solve's buffers
// and by every option or plan setting a captured graph bakes in: the
// many-cluster graph (which holds device pointers and kernel arguments of
// several plans) is replayed only while it has not moved.
std::atomic<unsigned long long> g_state_epoch{1};
void bump_epoch() { g_state_epoch.fetch_add(1, std::memory_order_relaxed); }
}

void rfx::count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

namespace {
std::mutex g_attr_mu;
std::map<std::pair<int, const void*>, size_t> g_smem_limit;
std::set<std::pair<int, const void*>> g_nonportable;
std::map<int, int> g_sm_count;
}  // namespace

cudaError_t rfx::ensure_smem_limit(const void* kernel, size_t bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_attr_mu);
  size_t& granted = g_smem_limit[{dev, kernel}];
  if (bytes <= granted) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (e == cudaSuccess) granted = bytes;
  return e;
}

cudaError_t rfx::ensure_nonportable_clusters(const void* kernel) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_attr_mu);
  if (g_nonportable.count({dev, kernel})) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e == cudaSuccess) g_nonportable.insert({dev, kernel});
  return e;
}

int rfx::current_sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lock(g_attr_mu);
  auto it = g_sm_count.find(dev);
  if (it != g_sm_count.end()) return it->second;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 1;
  g_sm_count[dev] = sms;
  return sms;
}

extern "C" unsigned long long refeff_fms_kernel_launches(void) { return g_launches.load(); }

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct refeff_fms_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  int sm_count = 0;
  int use_tensor_cores = 1;  // FP32 trailing updates on tcgen05 (REFEFF_FMS_OPT_TENSOR_CORES)
  int dense_refinement = 10; // corrections of the dense FP32 solve (REFEFF_FMS_OPT_DENSE_REFINEMENT)
  long long tc_wait_polls = kTcWaitPolls;  // REFEFF_FMS_OPT_TC_WAIT_POLLS
  int paired_blocks = 1;     // REFEFF_FMS_OPT_PAIRED_BLOCKS
  int multi_streams = 4;     // REFEFF_FMS_OPT_MULTI_STREAMS
  int dual_streams = 1;      // REFEFF_FMS_OPT_DUAL_STREAMS
  int bicg_tensor = 1;       // REFEFF_FMS_OPT_BICG_TENSOR
  int residual_tensor = 1;   // REFEFF_FMS_OPT_RESIDUAL_TENSOR
  std::vector<cudaStream_t> pool;  // extra streams for the multi-cluster spectrum (created on first use)
  std::vector<cudaEvent_t> pool_join;  // one per pool stream: joins it back into a capture
  cudaEvent_t fork_ev = nullptr;
  // the many-cluster call's device work as one CUDA graph (REFEFF_FMS_OPT_MULTI_GRAPH): captured on
  // the second call with the same plans, energy counts, batch sizes and form, replayed after that
  // while g_state_epoch is unchanged
  int multi_graph = 1;
  std::vector<long long> mg_key, mg_seen;
  unsigned long long mg_epoch = 0, mg_launches = 0, mg_seen_epoch = 0;
  cudaGraphExec_t mg_exec = nullptr;
  long long mg_captures = 0, mg_replays = 0;
  // the caller's handle plus one per live plan and model: the context is torn
  // down when the last of them is destroyed, in whatever order that happens
  std::atomic<int> refs{1};
};

void rfx::set_last_error(refeff_fms_context* ctx, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
}

int rfx::context_device(const refeff_fms_context* ctx) { return ctx->device; }
cudaStream_t rfx::context_stream(const refeff_fms_context* ctx) { return ctx->stream; }

extern "C" int refeff_fms_context_set_option(refeff_fms_context* ctx, int option, long long value) {
  if (!ctx) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  bump_epoch();
  switch (option) {
    case REFEFF_FMS_OPT_MULTI_GRAPH: ctx->multi_graph = value != 0; return REFEFF_FMS_OK;
    case REFEFF_FMS_OPT_BICG_TENSOR:
      if (value < 0 || value > 2) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
      ctx->bicg_tensor = int(value);
      return REFEFF_FMS_OK;
    case REFEFF_FMS_OPT_TENSOR_CORES: ctx->use_tensor_cores = value != 0; return REFEFF_FMS_OK;
    case REFEFF_FMS_OPT_RESIDUAL_TENSOR: ctx->residual_tensor = value != 0; return REFEFF_FMS_OK;
    case REFEFF_FMS_OPT_DENSE_REFINEMENT:
      if (value < 0 || value > 1000) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
      ctx->dense_refinement = int(value);
      return REFEFF_FMS_OK;
    case REFEFF_FMS_OPT_PAIRED_BLOCKS: ctx->paired_blocks = value != 0; return REFEFF_FMS_OK;
    case REFEFF_FMS_OPT_DUAL_STREAMS: ctx->dual_streams = value != 0; return REFEFF_FMS_OK;
    case REFEFF_FMS_OPT_MULTI_STREAMS:
      if (value < 1 || value > 64) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
      ctx->multi_streams = int(value);
      return REFEFF_FMS_OK;
    case REFEFF_FMS_OPT_TC_WAIT_POLLS:
      if (value < 0) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
      ctx->tc_wait_polls = value == 0 ? kTcWaitPolls : value;
      return REFEFF_FMS_OK;
    default: return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
}

namespace {

int fail(refeff_fms_context* ctx, int code, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

int cuda_fail(refeff_fms_context* ctx, cudaError_t err, const char* where) {
  const int code = (err == cudaErrorMemoryAllocation) ? REFEFF_FMS_ERR_OUT_OF_MEMORY : REFEFF_FMS_ERR_CUDA;
  return fail(ctx, code, std::string(where) + ": " + cudaGetErrorString(err));
}

#define RF_CUDA(ctx, expr)                                   \
  do {                                                       \
    cudaError_t rf_err_ = (expr);                            \
    if (rf_err_ != cudaSuccess) return cuda_fail(ctx, rf_err_, #expr); \
  } while (0)

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) {
      cudaFree(p);
      bump_epoch();
    }
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    bump_epoch();
    return e;
  }
  cudaError_t upload(const T* h, size_t count, cudaStream_t s) {
    cudaError_t e = alloc(count);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s);
  }
};

struct Atom {
  float pos[3];
  int pot;
};

// athep radial sort (crates/refeff-core/src/fms/internals/geometry.rs:30-36,
// cluster.rs:91-107): stable sort by r^2 + (index+1)*1e-6 in f64.
void athep_sort(std::vector<Atom>& atoms) {
  std::vector<std::pair<double, size_t>> keyed(atoms.size());
  for (size_t i = 0; i < atoms.size(); ++i) {
    const double x = atoms[i].pos[0], y = atoms[i].pos[1], z = atoms[i].pos[2];
    keyed[i] = {x * x + y * y + z * z + (double(i) + 1.0) * 1.0e-6, i};
  }
  std::stable_sort(keyed.begin(), keyed.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  std::vector<Atom> out(atoms.size());
  for (size_t i = 0; i < atoms.size(); ++i) out[i] = atoms[keyed[i].second];
  atoms.swap(out);
}

bool finite3(const float* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

}  // namespace

extern "C" int refeff_fms_abi_version(void) { return REFEFF_FMS_ABI_VERSION; }

extern "C" int refeff_fms_context_create(int device, refeff_fms_context** out) {
  if (!out) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || device < 0 || device >= count) return REFEFF_FMS_ERR_CUDA;
  auto* ctx = new refeff_fms_context();
  ctx->device = device;
  if ((e = cudaSetDevice(device)) != cudaSuccess || (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    delete ctx;
    return REFEFF_FMS_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  *out = ctx;
  return REFEFF_FMS_OK;
}

void rfx::context_retain(refeff_fms_context* ctx) { ctx->refs.fetch_add(1, std::memory_order_relaxed); }

void rfx::context_release(refeff_fms_context* ctx) {
  if (!ctx || ctx->refs.fetch_sub(1, std::memory_order_acq_rel) != 1) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  for (cudaStream_t q : ctx->pool) {
    cudaStreamSynchronize(q);
    cudaStreamDestroy(q);
  }
  for (cudaEvent_t ev : ctx->pool_join) cudaEventDestroy(ev);
  if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
  if (ctx->mg_exec) cudaGraphExecDestroy(ctx->mg_exec);
  delete ctx;
}

extern "C" void refeff_fms_context_destroy(refeff_fms_context* ctx) { context_release(ctx); }

extern "C" const char* refeff_fms_last_error(const refeff_fms_context* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

// ---------------------------------------------------------------------------
// cluster preparation (FEFF yprep + sortat)
// ---------------------------------------------------------------------------
extern "C" int refeff_fms_yprep_cluster(int central_potential, int max_potential, int n_rows, const int* potentials,
                                        const float* positions_xyz, float cluster_radius, int cluster_capacity,
                                        float* out_positions_xyz, int* out_potentials, int* out_count) {
  if (n_rows <= 0 || !potentials || !positions_xyz || !out_positions_xyz || !out_potentials || !out_count)
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (!std::isfinite(cluster_radius) || cluster_radius < 0.0f) return REFEFF_FMS_ERR_INVALID_CLUSTER_RADIUS;
  if (cluster_capacity <= 0) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  // cluster.rs:34-50: first atom with the central potential; duplicate absorbers rejected
  long central = -1;
  for (int i = 0; i < n_rows; ++i) {
    if (potentials[i] == central_potential) {
      if (central_potential == 0 && central >= 0) return REFEFF_FMS_ERR_DUPLICATE_ABSORBER;
      if (central < 0) central = i;
    }
  }
  if (central < 0) return REFEFF_FMS_ERR_MISSING_CENTRAL_ATOM;
  const float* c = positions_xyz + 3 * central;
  if (!finite3(c)) return REFEFF_FMS_ERR_NONFINITE_COORDINATE;
  std::vector<Atom> atoms(static_cast<size_t>(n_rows));
  for (int i = 0; i < n_rows; ++i) {
    for (int a = 0; a < 3; ++a) atoms[size_t(i)].pos[a] = positions_xyz[3 * i + a] - c[a];
    if (!finite3(atoms[size_t(i)].pos)) return REFEFF_FMS_ERR_NONFINITE_COORDINATE;
    atoms[size_t(i)].pot = potentials[i];
  }
  athep_sort(atoms);
  const float r2 = cluster_radius * cluster_radius;
  size_t first_outside = atoms.size();
  for (size_t i = 0; i < atoms.size(); ++i) {
    const float* p = atoms[i].pos;
    if (p[0] * p[0] + p[1] * p[1] + p[2] * p[2] > r2) { first_outside = i; break; }
  }
  const size_t untruncated = first_outside == 0 ? atoms.size() : first_outside;
  atoms.resize(std::min(untruncated, size_t(cluster_capacity)));
  // sortat (cluster.rs:115-195): representatives of each potential into the prefix
  if (central_potential < 0 || central_potential > max_potential) return REFEFF_FMS_ERR_POTENTIAL_OUT_OF_RANGE;
  for (auto& a : atoms)
    if (a.pot < 0 || a.pot > max_potential) return REFEFF_FMS_ERR_POTENTIAL_OUT_OF_RANGE;
  std::vector<long> rep(size_t(max_potential) + 1, -1);
  rep[size_t(central_potential)] = 0;
  for (int p = 0; p <= max_potential; ++p) {
    if (p == central_potential) continue;
    for (size_t i = 1; i < atoms.size(); ++i)
      if (atoms[i].pot == p) { rep[size_t(p)] = long(i); break; }
  }
  for (int p = 0; p <= max_potential; ++p) {
    const long point = rep[size_t(p)];
    if (point < 0 || point <= p) continue;
    std::swap(atoms[size_t(p)], atoms[size_t(point)]);
    for (int q = p + 1; q <= max_potential; ++q)
      if (rep[size_t(q)] == p) rep[size_t(q)] = point;
    rep[size_t(p)] = p;
  }
  const size_t prefix = std::min(atoms.size(), size_t(max_potential) + 1);
  for (int p = 0; p <= max_potential; ++p) {
    const long point = rep[size_t(p)];
    if (point < 0) continue;
    long last = -1;
    for (size_t i = 0; i < prefix; ++i)
      if (atoms[i].pot == p) last = long(i);
    if (last >= 0 && last != point) {
      float tmp[3];
      std::memcpy(tmp, atoms[size_t(last)].pos, sizeof tmp);
      std::memcpy(atoms[size_t(last)].pos, atoms[size_t(point)].pos, sizeof tmp);
      std::memcpy(atoms[size_t(point)].pos, tmp, sizeof tmp);
      rep[size_t(p)] = last;
    }
  }
  for (size_t i = 0; i < atoms.size(); ++i) {
    std::memcpy(out_positions_xyz + 3 * i, atoms[i].pos, 3 * sizeof(float));
    out_potentials[i] = atoms[i].pot;
  }
  *out_count = int(atoms.size());
  return REFEFF_FMS_OK;
}

// ---------------------------------------------------------------------------
// plan
// ---------------------------------------------------------------------------
namespace {

// FEFF's associated-Legendre normalization (crates/refeff-core/src/angular/harmonics.rs:51-75).
double xnlm_value(int l, int m) {
  if (m > l) return 0.0;
  double den = 1.0;
  for (int k = l - m + 1; k <= l + m; ++k) den *= double(k);
  return std::sqrt(double(2 * l + 1) / den);
}

// Doubled-argument Wigner 3j by the Racah sum over log-factorials and the
// t3jp / t3jm coefficients (crates/refeff-core/src/angular/coupling.rs:4-40).
double wigner3j_doubled(int j1, int j2, int j3, int m1, int m2) {
  const int m3 = -m1 - m2;
  if (std::abs(m1) + std::abs(m2) == 0 && (j1 + j2 + j3) % 4 != 0) return 0.0;
  int v[12] = {j1 + j2 - j3, j2 + j3 - j1, j3 + j1 - j2, j1 + m1, j1 - m1, j2 + m2,
               j2 - m2,      j3 + m3,      j3 - m3,      j1 + j2 + j3 + 2, j2 - j3 - m1, j1 - j3 + m2};
  for (int i = 0; i < 12; ++i) {
    if (i < 10 && v[i] < 0) return 0.0;
    v[i] /= 2;
  }
  double lf[64];
  lf[0] = 0.0;
  for (int i = 1; i < 64; ++i) lf[i] = lf[i - 1] + std::log(double(i));
  const int kmin = std::max(std::max(v[10], v[11]), 0), kmax = std::min(std::min(v[0], v[4]), v[5]);
  if (kmin > kmax) return 0.0;
  double sign = (kmin % 2 == 0) ? 1.0 : -1.0;
  double c = -lf[v[9]];
  for (int i = 0; i < 9; ++i) c += lf[v[i]];
  c /= 2.0;
  double coef = 0.0;
  for (int k = kmin; k <= kmax; ++k) {
    coef += sign * std::exp(c - (lf[k] + lf[v[0] - k] + lf[v[4] - k] + lf[v[5] - k] + lf[k - v[10]] + lf[k - v[11]]));
    sign = -sign;
  }
  if ((j1 - j2 - m3) % 4 != 0) coef = -coef;
  return coef;
}

double so_coefficient(bool plus, int l, int m, int spin) {
  const int j1 = 2 * l, j2 = 1, j3 = plus ? j1 + 1 : j1 - 1, m1 = 2 * m, m2 = 2 * spin - 3;
  const int phase = (j2 - j1 - m1 - m2) / 2;
  return ((phase % 2 == 0) ? 1.0 : -1.0) * std::sqrt(double(j3 + 1)) * wigner3j_doubled(j1, j2, j3, m1, m2);
}

}  // namespace

// Per-plan choices of the FP32 elimination (set by the caller or the
// autotuner): the inner panel width preference of choose_panel and whether
// 64-column blocks are paired (-1: the context's REFEFF_FMS_OPT_PAIRED_BLOCKS).
struct TunePrefs {
  int inner = 0;
  int paired = -1;
};

struct Workspace {
  int batch = 0;
  bool fp32 = false;
  BatchLayout lay;
  PanelConfig pc64, pc32;
  int inner_pref = 0;    // choose_panel<float> preference the workspace was built with
  int paired_pref = 1;   // pairing asked for (context or plan)
  DevBuf<double2> M64;
  DevBuf<float2> M32;
  DevBuf<double2> X64, R;
  DevBuf<float4> Xsplit;  // x as hi/lo float pairs for the residual
  DevBuf<double2> t_tab, grow, iter_scratch;  // iterative forms (minv != 0)
  DevBuf<unsigned long long> rnorm, bnorm, dnorm, xnorm;
  DevBuf<double> dprev;
  DevBuf<int> converged, iters;
  DevBuf<double> relres;
  DevBuf<int> ipiv, nperm, status, info;
  bool use_tc = false;               // FP32 trailing update on the tensor cores
  DevBuf<uint8_t> tc_images;         // operand images of the tensor-core update (and the residual's X digits)
  size_t tc_image_size = 0;
  int residual_pref = 1;             // refinement residual on the tensor cores (baked into graphs)
  DevBuf<int> tc_err;                // set by a tensor-core wait that timed out
  long long tc_wait_polls = kTcWaitPolls;  // poll budget of the tensor-core update's role waits (baked into graphs)
  KernelSpans tc_spans;              // events around this workspace's tensor-core updates (profiling)
  DevBuf<int2> perm;
  DevBuf<int2> perm_in;              // row moves of the inner panels (two-level FP32 LU)
  DevBuf<float2> linv;               // inverse of each outer block's unit lower L11 (two-level FP32 LU)
  DevBuf<int> nperm_in;
  DevBuf<int> pos_scratch;           // panel row-position bookkeeping for large n
  // BiCGSTAB form: solver vectors and scalars, the preconditioner diagonal,
  // per-atom features and network outputs
  DevBuf<float2> bicg_vec, precond_D;
  DevBuf<float2> bicg_part;  // partial products of the split matrix-vector product
  DevBuf<int> bicg_act;      // compacted list of the running matrices
  DevBuf<int> bicg_err;      // set when a wait of the tensor-core product gave up
  DevBuf<float2> precond_B;  // block-diagonal learned preconditioner: batch x N x C^2
  DevBuf<double> bicg_sc;
  DevBuf<int> bicg_state, bicg_done, bicg_iters, bicg_active, bicg_total;
  DevBuf<float> feat_X, feat_Y;
  MlpScratch mlp;
  // staging so that a captured graph can be replayed on every batch
  DevBuf<double2> k_stage, x_stage, gg_stage;
  DevBuf<double2> full_stage;  // save_gg_slice outputs of a batch (full plans)
  DevBuf<double2> hank;        // pair prefactors and Hankel tables of a batch (pair_hankel_kernel)
  DevBuf<int> hflag;
  std::map<int, cudaGraphExec_t> graphs;  // key: form * 65536 + energies in the batch
  std::map<int, unsigned long long> graph_launches;  // kernel launches per replay
  void drop_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    bump_epoch();
  }
  ~Workspace() { drop_graphs(); }
};

struct refeff_fms_plan {
  refeff_fms_context* ctx = nullptr;
  int N = 0, L = 0, nsp = 1, ispin = 0, npot = 0, lfms = 0, minv = 0;
  int n = 0, m = 0, C = 0, abs_pot = 0, abs_lmax = 0;
  // m: right-hand sides (the representative blocks of every potential in the solved range);
  // m_abs: the absorber block; gg_per: packed size of one energy's solved blocks
  int m_abs = 0, gg_per = 0;
  std::vector<SolvedBlock> blocks;   // per potential of the range, in potential order
  std::vector<int> block_pot;        // the potential of each block
  // full scattering (save_gg_slice): B = G0 entirely (m = n), and per energy the
  // b x n slice of the absorber's rows plus every atom's b x b diagonal block
  bool full = false;
  int full_per = 0;
  DevBuf<double2> d_full_all;
  DevBuf<SolvedBlock> d_blocks;
  DevBuf<int> d_bcol;
  std::vector<int> pot_lmax;
  std::vector<long> rep_offsets;  // reference state order
  int max_batch = 0;
  int refine_iters = 10;
  double refine_tol = 1.0e-10;  // stop when the correction, or its estimated remaining error, <= tol * max|x|
  // per-energy refinement outcome of the last spectrum call (FP32_REFINED)
  DevBuf<double> d_relres_all;
  DevBuf<int> d_iters_all;
  std::vector<double> last_relres;
  std::vector<int> last_iters;
  std::vector<int> last_fallback;  // energies re-solved with the FP64 LU after refinement missed
  int last_fallbacks = 0;
  // device tables
  PlanDev P;
  DevBuf<float> d_pos;
  DevBuf<int> d_atom_pot, d_atom_off, d_atom_lmax;
  DevBuf<double> d_sigsqr, d_dist, d_phi, d_dsmall, d_xnlm, d_xnlm_w, d_t3p, d_t3m;
  DevBuf<double2> d_eph;
  DevBuf<float2> d_dsmall_df, d_xnlm_df, d_xnlm_w_df;
  DevBuf<float4> d_eph_df;
  DevBuf<double2> d_k_all, d_x_all, d_gg_all;
  DevBuf<int> d_status_all;
  DevBuf<int> d_partner;  // spin partner per state, device order (-1 none)
  double toler1 = 0.0, toler2 = 0.0;  // iterative forms: convergence and G0 drop tolerances (f32 values)
  // BiCGSTAB form
  std::vector<float> pos_dev;         // positions, device atom order (host copy)
  std::vector<int> pot_dev;           // potentials, device atom order (host copy)
  std::vector<int> off_dev;           // first state of each atom, device order (host copy, N + 1)
  refeff_fms_precond_model* model = nullptr;  // learned preconditioner (not owned), NULL: none
  double precond_e_lo = -1e300, precond_e_hi = 1e300;  // energies (E - E_ref, eV) where the model is applied
  double bicg_e_lo = -1e300, bicg_e_hi = 1e300;  // energies the BiCGSTAB form iterates on; the rest go to the LU
  DevBuf<float> d_shell_info, d_shell_pots;
  DevBuf<int> d_state_atom;  // device atom of each state (device order), for the block preconditioner
  int bicg_max_iter = 400;
  double bicg_tol = 1.0e-6;
  int bicg_poll = 8;
  DevBuf<int> d_bicg_iters_all;
  std::vector<int> last_bicg_iters;
  // BiCGSTAB-form energies handed to the refined LU: 1 missed the tolerance, 2 outside the window
  std::vector<int> bicg_lu;
  std::vector<int> bicg_order;  // energies of the last BiCGSTAB-form call that iterated (window routing)
  TunePrefs tune;  // per-plan FP32 elimination choices (refeff_fms_plan_set_tuning, the autotuner)
  Workspace ws;
  // the second workspace and stream of two-stream batching, and its fork / join events (created on first use)
  Workspace ws2;
  cudaStream_t s2 = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  ~refeff_fms_plan() {
    if (s2) {
      cudaStreamSynchronize(s2);
      cudaStreamDestroy(s2);
    }
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
  }
  bool profiling = false;
  double phase_ms[REFEFF_FMS_PHASES] = {0, 0, 0, 0, 0, 0};
  size_t xph_per_energy() const { return size_t(nsp) * size_t(2 * L + 1) * size_t(npot); }
};

namespace {

int plan_create(refeff_fms_context* ctx, const refeff_fms_plan_input* in, bool full, refeff_fms_plan** out) {
  if (!ctx || !in || !out) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  ctx->last_error.clear();
  if (in->n_atoms <= 0) return fail(ctx, REFEFF_FMS_ERR_EMPTY_CLUSTER, "empty cluster");
  if (!in->positions_xyz || !in->potentials || !in->raw_potential_lmax)
    return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "null plan input array");
  if (in->spin_channels < 1 || in->spin_channels > 2)
    return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "spin_channels must be 1 or 2");
  if (in->max_potential < 0) return fail(ctx, REFEFF_FMS_ERR_POTENTIAL_OUT_OF_RANGE, "negative max_potential");
  if (in->global_lmax < 0 || in->global_lmax > kMaxL)
    return fail(ctx, REFEFF_FMS_ERR_INVALID_ANGULAR_LIMIT, "global_lmax outside 0..6");
  if (!std::isfinite(in->direct_cutoff) || in->direct_cutoff < 0.0f)
    return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "invalid direct cutoff");
  if (!std::isfinite(in->zero_tolerance) || in->zero_tolerance < 0.0f)
    return fail(ctx, REFEFF_FMS_ERR_INVALID_TOLERANCE, "invalid toler2");
  if (in->minv != 0 && (!std::isfinite(in->convergence_tolerance) || in->convergence_tolerance < 0.0f))
    return fail(ctx, REFEFF_FMS_ERR_INVALID_TOLERANCE, "invalid toler1");
  auto plan = std::make_unique<refeff_fms_plan>();
  refeff_fms_plan& p = *plan;
  p.ctx = ctx;
  p.N = in->n_atoms;
  p.L = in->global_lmax;
  p.nsp = in->spin_channels;
  p.ispin = in->spin_selector;
  p.npot = in->max_potential + 1;
  p.lfms = in->lfms;
  // a full scattering matrix forces the LU form (fms_scattering_method_selection, driver.rs:72-96)
  p.minv = full ? 0 : in->minv;
  p.full = full;
  p.toler1 = double(in->convergence_tolerance);
  p.toler2 = double(in->zero_tolerance);
  const int N = p.N, L = p.L, nsp = p.nsp;
  // driver.rs:25-31, validation.rs:69-75: clamp lipotx
  p.pot_lmax.resize(size_t(p.npot));
  for (int q = 0; q < p.npot; ++q) {
    const int v = in->raw_potential_lmax[q];
    p.pot_lmax[size_t(q)] = v < 0 ? L : std::min(v, L);
  }
  std::vector<int> atom_pot(static_cast<size_t>(N));
  for (int a = 0; a < N; ++a) {
    const int pot = in->potentials[a];
    if (pot < 0 || pot > in->max_potential)
      return fail(ctx, REFEFF_FMS_ERR_POTENTIAL_OUT_OF_RANGE, "atom " + std::to_string(a) + " potential out of range");
    if (!finite3(in->positions_xyz + 3 * a)) return fail(ctx, REFEFF_FMS_ERR_NONFINITE_COORDINATE, "non-finite coordinate");
    atom_pot[size_t(a)] = pot;
  }
  // state kets (state.rs:97-148) in reference order: offsets per potential
  p.rep_offsets.assign(size_t(p.npot), -1);
  std::vector<int> ref_off(static_cast<size_t>(N) + 1, 0);
  for (int a = 0; a < N; ++a) {
    const int pot = atom_pot[size_t(a)];
    if (p.rep_offsets[size_t(pot)] < 0) p.rep_offsets[size_t(pot)] = ref_off[size_t(a)];
    const int lm = std::min(L, p.pot_lmax[size_t(pot)]);
    ref_off[size_t(a) + 1] = ref_off[size_t(a)] + nsp * (lm + 1) * (lm + 1);
  }
  p.n = ref_off[size_t(N)];
  p.abs_pot = atom_pot[0];
  p.abs_lmax = std::min(L, p.pot_lmax[size_t(p.abs_pot)]);
  p.m_abs = nsp * (p.abs_lmax + 1) * (p.abs_lmax + 1);
  p.C = nsp * (L + 1) * (L + 1);
  // driver.rs:36-60: active potential range must have representatives
  const int pstart = p.lfms == 0 ? p.abs_pot : 0, pend = p.lfms == 0 ? p.abs_pot : in->max_potential;
  for (int q = pstart; q <= pend; ++q)
    if (p.rep_offsets[size_t(q)] < 0)
      return fail(ctx, REFEFF_FMS_ERR_MISSING_REPRESENTATIVE, "no atom for potential " + std::to_string(q));
  if (full && p.n != N * p.C)
    return fail(ctx, REFEFF_FMS_ERR_UNSUPPORTED,
                "save_gg_slice requires fixed-width atom blocks: got " + std::to_string(p.n) + " state(s), expected " +
                    std::to_string(N * p.C) + " from " + std::to_string(N) + " atom(s) and block dimension " +
                    std::to_string(p.C));
  if (N < 2) return fail(ctx, REFEFF_FMS_ERR_UNSUPPORTED, "a single-atom cluster has no scattering");

  // device atom order: reference atom 0 (absorber) last
  auto dev = [N](int a) { return a == 0 ? N - 1 : a - 1; };
  std::vector<float> pos(static_cast<size_t>(3 * N));
  std::vector<int> dpot(static_cast<size_t>(N)), doff(static_cast<size_t>(N) + 1, 0), dlmax(static_cast<size_t>(N));
  for (int a = 0; a < N; ++a) {
    const int d = dev(a);
    std::memcpy(&pos[size_t(3 * d)], in->positions_xyz + 3 * a, 3 * sizeof(float));
    dpot[size_t(d)] = atom_pot[size_t(a)];
    dlmax[size_t(d)] = std::min(L, p.pot_lmax[size_t(atom_pot[size_t(a)])]);
  }
  for (int d = 0; d < N; ++d) doff[size_t(d) + 1] = doff[size_t(d)] + nsp * (dlmax[size_t(d)] + 1) * (dlmax[size_t(d)] + 1);
  // solved blocks (fms_lu_scattering, solvers.rs:366-484): for each potential of the range, the
  // representative's states (its first atom in cluster order) are right-hand sides, and its block
  // of the solution is the scattering table entry of that potential.  A full plan solves for
  // every column of G0 (solvers.rs:473-479), so B = G0 and each block sits at its own columns.
  std::vector<int> bcol(static_cast<size_t>(N), -1);
  if (full)
    for (int d = 0; d < N; ++d) bcol[size_t(d)] = doff[size_t(d)];
  {
    int col = 0, pack = 0;
    for (int q = pstart; q <= pend; ++q) {
      int a = 0;
      while (atom_pot[size_t(a)] != q) ++a;
      const int d = dev(a);
      const int size = doff[size_t(d) + 1] - doff[size_t(d)];
      if (!full) bcol[size_t(d)] = col;
      p.blocks.push_back({doff[size_t(d)], full ? doff[size_t(d)] : col, size, pack});
      p.block_pot.push_back(q);
      col += size;
      pack += size * size;
    }
    p.m = full ? p.n : col;
    p.gg_per = pack;
    p.full_per = full ? p.C * p.n + N * p.C * p.C : 0;
  }
  if (!full && p.m > 64)
    return fail(ctx, REFEFF_FMS_ERR_UNSUPPORTED, "more than 64 right-hand sides in the potential range");
  // sigma^2 table, device order [a2 + N a1] (engine/fms.rs:4394-4426)
  std::vector<double> sig(static_cast<size_t>(N) * N, 0.0);
  for (int a1 = 0; a1 < N; ++a1)
    for (int a2 = 0; a2 < N; ++a2) {
      if (a1 == a2) continue;
      const float v = in->mean_square_displacements ? in->mean_square_displacements[size_t(a2) + size_t(N) * a1] : in->sig2g;
      if (!std::isfinite(v)) return fail(ctx, REFEFF_FMS_ERR_NONFINITE_INPUT, "non-finite mean-square displacement");
      sig[size_t(dev(a2)) + size_t(N) * dev(a1)] = double(v);
    }
  // xnlm narrowed to f32 like the reference (pairs.rs:678)
  std::vector<double> xnlm(static_cast<size_t>((L + 1) * (L + 1)), 0.0);
  for (int l = 0; l <= L; ++l)
    for (int mu = 0; mu <= l; ++mu) xnlm[size_t(mu + (L + 1) * l)] = double(float(xnlm_value(l, mu)));
  const int D = 2 * L + 1;
  std::vector<double> t3p(size_t(L + 1) * D * 2, 0.0), t3m(size_t(L + 1) * D * 2, 0.0);
  for (int l = 0; l <= L; ++l)
    for (int mm = -l; mm <= l; ++mm)
      for (int s = 1; s <= 2; ++s) {
        const size_t idx = size_t(l) + size_t(L + 1) * (size_t(mm + L) + size_t(D) * size_t(s - 1));
        t3p[idx] = double(float(so_coefficient(true, l, mm, s)));
        t3m[idx] = double(float(so_coefficient(false, l, mm, s)));
      }

  RF_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const int ds = 2 * (L + 1) * (2 * L + 1) * (2 * L + 3) / 3;
  RF_CUDA(ctx, p.d_pos.upload(pos.data(), pos.size(), s));
  p.pos_dev = pos;
  p.pot_dev = dpot;
  p.off_dev = doff;
  RF_CUDA(ctx, p.d_atom_pot.upload(dpot.data(), dpot.size(), s));
  RF_CUDA(ctx, p.d_atom_off.upload(doff.data(), doff.size(), s));
  RF_CUDA(ctx, p.d_atom_lmax.upload(dlmax.data(), dlmax.size(), s));
  RF_CUDA(ctx, p.d_bcol.upload(bcol.data(), bcol.size(), s));
  RF_CUDA(ctx, p.d_blocks.upload(p.blocks.data(), p.blocks.size(), s));
  RF_CUDA(ctx, p.d_sigsqr.upload(sig.data(), sig.size(), s));
  RF_CUDA(ctx, p.d_xnlm.upload(xnlm.data(), xnlm.size(), s));
  {
    std::vector<double> w(xnlm.size(), 0.0);
    for (int l = 0; l <= L; ++l)
      for (int mu = 0; mu <= l; ++mu) w[size_t(mu + (L + 1) * l)] = double(2 * l + 1) / xnlm[size_t(mu + (L + 1) * l)];
    RF_CUDA(ctx, p.d_xnlm_w.upload(w.data(), w.size(), s));
    // double-float copies (hi = fl32(v), lo = fl32(v - hi)) for the refined form's build
    auto split = [](const std::vector<double>& v) {
      std::vector<float2> o(v.size());
      for (size_t i = 0; i < v.size(); ++i) {
        const float h = float(v[i]);
        o[i] = make_float2(h, float(v[i] - double(h)));
      }
      return o;
    };
    const std::vector<float2> xd = split(xnlm), wd = split(w);
    RF_CUDA(ctx, p.d_xnlm_df.upload(xd.data(), xd.size(), s));
    RF_CUDA(ctx, p.d_xnlm_w_df.upload(wd.data(), wd.size(), s));
    RF_CUDA(ctx, cudaStreamSynchronize(s));  // the host vectors go out of scope
  }
  RF_CUDA(ctx, p.d_t3p.upload(t3p.data(), t3p.size(), s));
  RF_CUDA(ctx, p.d_t3m.upload(t3m.data(), t3m.size(), s));
  {
    // fms_spin_partner_index (internals/linear.rs:163-201): (l, m, 1) <-> (l, m - 1, 2)
    std::vector<int> partner(static_cast<size_t>(p.n), -1);
    for (int d = 0; d < N; ++d)
      for (int q = 0; q < doff[size_t(d) + 1] - doff[size_t(d)]; ++q) {
        if (nsp != 2) break;
        const int sp = q % 2 + 1, lm = q / 2;
        int l = 0;
        while ((l + 1) * (l + 1) <= lm) ++l;
        const int m = lm - l * l - l;
        if (sp == 1 && m > -l) partner[size_t(doff[size_t(d)] + q)] = doff[size_t(d)] + q - 1;
        if (sp == 2 && m < l) partner[size_t(doff[size_t(d)] + q)] = doff[size_t(d)] + q + 1;
      }
    RF_CUDA(ctx, p.d_partner.upload(partner.data(), partner.size(), s));
  }
  RF_CUDA(ctx, p.d_dist.alloc(size_t(N) * N));
  RF_CUDA(ctx, p.d_phi.alloc(size_t(N) * N));
  RF_CUDA(ctx, p.d_eph.alloc(size_t(N) * N * (4 * L + 1)));
  RF_CUDA(ctx, p.d_dsmall.alloc(size_t(N) * N * ds));
  RF_CUDA(ctx, p.d_eph_df.alloc(size_t(N) * N * (4 * L + 1)));
  RF_CUDA(ctx, p.d_dsmall_df.alloc(size_t(N) * N * ds));
  PlanDev& P = p.P;
  P.N = N; P.L = L; P.nsp = nsp; P.ispin = p.ispin; P.npot = p.npot; P.n = p.n; P.m = p.m; P.ds = ds;
  P.pos = p.d_pos.p; P.atom_pot = p.d_atom_pot.p; P.atom_off = p.d_atom_off.p; P.atom_lmax = p.d_atom_lmax.p;
  P.sigsqr = p.d_sigsqr.p; P.pair_dist = p.d_dist.p; P.pair_phi = p.d_phi.p; P.pair_dsmall = p.d_dsmall.p;
  P.xnlm = p.d_xnlm.p; P.xnlm_w = p.d_xnlm_w.p; P.t3p = p.d_t3p.p; P.t3m = p.d_t3m.p; P.pair_eph = p.d_eph.p;
  P.bcol = p.d_bcol.p;
  P.pair_dsmall_df = p.d_dsmall_df.p; P.pair_eph_df = p.d_eph_df.p;
  P.xnlm_df = p.d_xnlm_df.p; P.xnlm_w_df = p.d_xnlm_w_df.p;
  P.rdirec2 = double(in->direct_cutoff) * double(in->direct_cutoff);
  launch_plan_geometry(P, s);
  launch_plan_df_tables(P, s);
  RF_CUDA(ctx, cudaGetLastError());
  RF_CUDA(ctx, cudaStreamSynchronize(s));
  context_retain(ctx);
  *out = plan.release();
  return REFEFF_FMS_OK;
}

}  // namespace

extern "C" int refeff_fms_real_space_plan_create(refeff_fms_context* ctx, const refeff_fms_plan_input* in,
                                                 refeff_fms_plan** out) {
  return plan_create(ctx, in, false, out);
}

extern "C" int refeff_fms_real_space_plan_create_full(refeff_fms_context* ctx, const refeff_fms_plan_input* in,
                                                      refeff_fms_plan** out) {
  return plan_create(ctx, in, true, out);
}

extern "C" void refeff_fms_real_space_plan_destroy(refeff_fms_plan* plan) {
  if (!plan) return;
  bump_epoch();
  refeff_fms_context* ctx = plan->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete plan;
  context_release(ctx);
}

extern "C" int refeff_fms_plan_set_profiling(refeff_fms_plan* plan, int enable) {
  if (!plan) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  bump_epoch();
  plan->profiling = enable != 0;
  for (double& v : plan->phase_ms) v = 0.0;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_phase_times(const refeff_fms_plan* plan, double* ms_out, int n_phases) {
  if (!plan || !ms_out || n_phases < 0) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < n_phases && i < REFEFF_FMS_PHASES; ++i) ms_out[i] = plan->phase_ms[i];
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_query(const refeff_fms_plan* plan, int* n_states, int* channel_count, int* absorber_block,
                                     int* n_potentials) {
  if (!plan) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (n_states) *n_states = plan->n;
  if (channel_count) *channel_count = plan->C;
  if (absorber_block) *absorber_block = plan->m_abs;
  if (n_potentials) *n_potentials = plan->npot;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_set_tuning(refeff_fms_plan* plan, int inner_width, int paired_blocks) {
  if (!plan || !(inner_width == 0 || inner_width == 1 || inner_width == 16 || inner_width == 32) || paired_blocks < -1 ||
      paired_blocks > 1)
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  bump_epoch();
  plan->tune.inner = inner_width;
  plan->tune.paired = paired_blocks;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_get_tuning(const refeff_fms_plan* plan, int* inner_width, int* paired_blocks) {
  if (!plan) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (inner_width) *inner_width = plan->tune.inner;
  if (paired_blocks) *paired_blocks = plan->tune.paired;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_set_batch(refeff_fms_plan* plan, int max_batch) {
  if (!plan || max_batch < 0) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  bump_epoch();
  plan->max_batch = max_batch;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_set_refinement(refeff_fms_plan* plan, int max_iterations, double tolerance) {
  if (!plan || max_iterations < 0 || !(tolerance > 0.0)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  plan->refine_iters = max_iterations;
  plan->refine_tol = tolerance;
  plan->ws.drop_graphs();
  return REFEFF_FMS_OK;
}

// ---------------------------------------------------------------------------
// batched execution
// ---------------------------------------------------------------------------
namespace {

BatchLayout make_layout(int n, int m) {
  BatchLayout lay;
  lay.n = n;
  lay.m = m;
  lay.lda = (n + 31) / 32 * 32;
  lay.stride = size_t(lay.lda) * size_t(n + m);
  return lay;
}

size_t bytes_per_system(const BatchLayout& lay, bool fp32) {
  size_t b = lay.stride * sizeof(double2);
  if (fp32) b += lay.stride * sizeof(float2) + 2 * size_t(lay.lda) * lay.m * sizeof(double2);
  return b;
}

// Paired 64-column blocks (one K = 128 tensor-core update per pair) when the
// tensor cores run the FP32 LU and the fused forward sweep replays its moves.
int want_pair128(const Workspace& ws) {
  return ws.paired_pref && ws.fp32 && ws.use_tc && ws.pc32.inner_nb && fused_sweep_available(ws.pc32.nb, ws.lay)
             ? 1 : 0;
}

int ensure_workspace_impl(refeff_fms_context* ctx, Workspace& ws, int n, int m, int batch, bool fp32,
                          const TunePrefs* tune) {
  const BatchLayout lay = make_layout(n, m);
  if (ws.tc_wait_polls != ctx->tc_wait_polls) {  // a kernel argument: captured graphs hold the old budget
    ws.drop_graphs();
    ws.tc_wait_polls = ctx->tc_wait_polls;
  }
  if (ws.residual_pref != ctx->residual_tensor) {  // the residual's launch sequence changes: recapture
    ws.drop_graphs();
    ws.residual_pref = ctx->residual_tensor;
  }
  const int inner = tune ? tune->inner : 0;
  ws.paired_pref = tune && tune->paired >= 0 ? tune->paired : ctx->paired_blocks;
  if (ws.batch >= batch && ws.lay.n == n && ws.lay.m == m && (ws.fp32 || !fp32) && ws.inner_pref == inner) {
    const int pair = want_pair128(ws);
    if (pair != ws.pc32.pair128) {  // the elimination's launch sequence changes: recapture
      ws.drop_graphs();
      ws.pc32.pair128 = pair;
    }
    return REFEFF_FMS_OK;
  }
  ws.drop_graphs();
  ws.inner_pref = inner;
  ws.batch = std::max(batch, ws.lay.n == n && ws.lay.m == m ? ws.batch : 0);
  ws.fp32 = fp32 || (ws.lay.n == n && ws.lay.m == m && ws.fp32);
  ws.lay = lay;
  const int B = ws.batch;
  ws.pc64 = choose_panel<double>(n);
  ws.pc32 = choose_panel<float>(n, inner);
  if (ws.pc64.cluster <= 0 || (ws.fp32 && ws.pc32.cluster <= 0))
    return fail(ctx, REFEFF_FMS_ERR_UNSUPPORTED, "system too large for the cluster panel factorization");
  const int nb_min = std::min(ws.pc64.nb, ws.pc32.nb);
  const int nb_max = std::max(ws.pc64.nb, ws.pc32.nb);
  const int npanels = panel_count(n, nb_min);
  RF_CUDA(ctx, ws.M64.alloc(size_t(B) * lay.stride));
  if (ws.fp32) {
    RF_CUDA(ctx, ws.M32.alloc(size_t(B) * lay.stride));
    RF_CUDA(ctx, ws.X64.alloc(size_t(B) * lay.lda * m));
    RF_CUDA(ctx, ws.R.alloc(size_t(B) * lay.lda * m));
    RF_CUDA(ctx, ws.Xsplit.alloc(size_t(B) * lay.lda * m));
    RF_CUDA(ctx, ws.rnorm.alloc(size_t(B)));
    RF_CUDA(ctx, ws.bnorm.alloc(size_t(B)));
    RF_CUDA(ctx, ws.dnorm.alloc(size_t(B)));
    RF_CUDA(ctx, ws.xnorm.alloc(size_t(B)));
    RF_CUDA(ctx, ws.dprev.alloc(size_t(B)));
    RF_CUDA(ctx, ws.converged.alloc(size_t(B)));
    RF_CUDA(ctx, ws.iters.alloc(size_t(B)));
    RF_CUDA(ctx, ws.relres.alloc(size_t(B)));
  }
  if (ws.pc64.pos_global || (ws.fp32 && ws.pc32.pos_global)) RF_CUDA(ctx, ws.pos_scratch.alloc(size_t(B) * 2 * n));
  if (ws.fp32 && ws.pc32.inner_nb) {
    RF_CUDA(ctx, ws.perm_in.alloc(size_t(B) * panel_count(n, ws.pc32.inner_nb) * 2 * ws.pc32.inner_nb));
    RF_CUDA(ctx, ws.nperm_in.alloc(size_t(B) * panel_count(n, ws.pc32.inner_nb)));
    RF_CUDA(ctx, ws.linv.alloc(size_t(B) * 64 * 64));
  }
  RF_CUDA(ctx, ws.ipiv.alloc(size_t(B) * n));
  RF_CUDA(ctx, ws.perm.alloc(size_t(B) * npanels * 2 * nb_max));
  RF_CUDA(ctx, ws.nperm.alloc(size_t(B) * npanels));
  RF_CUDA(ctx, ws.status.alloc(size_t(B)));
  RF_CUDA(ctx, ws.info.alloc(size_t(B)));
  ws.use_tc = ws.fp32 && ctx->use_tensor_cores != 0;
  if (ws.use_tc) {
    ws.tc_image_size = tc_image_bytes(n, m, B);
    RF_CUDA(ctx, ws.tc_images.alloc(ws.tc_image_size));
    RF_CUDA(ctx, ws.tc_err.alloc(1));
    RF_CUDA(ctx, cudaMemset(ws.tc_err.p, 0, sizeof(int)));
  }
  ws.pc32.pair128 = want_pair128(ws);
  return REFEFF_FMS_OK;
}

// A workspace whose (re)configuration failed part-way (an allocation) is left
// unconfigured, so that the next call configures it again instead of running
// on buffers sized for another shape.
int ensure_workspace(refeff_fms_context* ctx, Workspace& ws, int n, int m, int batch, bool fp32,
                     const TunePrefs* tune = nullptr) {
  const int rc = ensure_workspace_impl(ctx, ws, n, m, batch, fp32, tune);
  if (rc) {
    ws.drop_graphs();
    ws.batch = 0;
    ws.lay.n = -1;
  }
  return rc;
}

LuWork lu_work(Workspace& ws, const PanelConfig& pc) {
  LuWork w;
  w.ipiv = ws.ipiv.p;
  w.perm = ws.perm.p;
  w.nperm = ws.nperm.p;
  w.status = ws.status.p;
  w.info = ws.info.p;
  w.nb = pc.nb;
  w.npanels = panel_count(ws.lay.n, pc.nb);
  w.pos_scratch = ws.pos_scratch.p;
  if (&pc == &ws.pc32) {
    w.perm_in = ws.perm_in.p;
    w.nperm_in = ws.nperm_in.p;
    w.linv = ws.linv.p;
    w.pair128 = pc.pair128;
  }
  if (&pc == &ws.pc32 && ws.use_tc) {
    w.tc_images = ws.tc_images.p;
    w.tc_err = ws.tc_err.p;
    w.tc_wait_polls = ws.tc_wait_polls;
    w.tc_spans = &ws.tc_spans;
  }
  return w;
}

using Spans = std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>>;

// Iterative refinement of X64 for the split system [A | B] in M64 with the
// FP32 factors in M32 (eliminated; RHS columns of M32 hold Y32).  Each step:
// r = b - A x (double-float), d = LU^-1 r (FP32), x += d; stop per system when
// |d| <= tol |x| (converged[b] = 1) or when |d| stops halving (converged[b] = 2,
// handed to the FP64 LU by the caller).  With `spans`, events bracket the
// sweeps (phase 2) and the residuals (phase 3).
// The tensor-core residual's arguments when the workspace runs it (the
// tensor-core update's images hold its scratch), else null: the Dot2 residual.
const ResidualTc* residual_tc(const Workspace& ws, ResidualTc& out) {
  if (!ws.use_tc || !ws.residual_pref || !ws.tc_images.p) return nullptr;
  out.images = ws.tc_images.p;
  out.bytes = ws.tc_image_size;
  out.err = ws.tc_err.p;
  out.polls = ws.tc_wait_polls;
  return &out;
}

cudaError_t refine_fp32(Workspace& ws, int batch, int iters, double tol, cudaStream_t s, Spans* spans = nullptr) {
  ResidualTc rtc;
  const BatchLayout& lay = ws.lay;
  const LuWork w32 = lu_work(ws, ws.pc32);
  auto span = [&](int phase, auto&& fn) {
    cudaEvent_t a = nullptr, b = nullptr;
    if (spans) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, s);
    }
    fn();
    if (spans) {
      cudaEventRecord(b, s);
      spans->push_back({phase, {a, b}});
    }
  };
  const size_t nb8 = size_t(batch) * sizeof(unsigned long long);
  // fused one-CTA-per-(matrix, column group) sweeps when the right-hand sides fit in shared memory
  auto forward = [&](const int* skip) {
    if (!fused_forward_sweep(ws.pc32.nb, lay, batch, ws.M32.p, w32, skip, s))
      lu_forward_rhs<float>(ws.pc32, lay, batch, ws.M32.p, w32, skip, s);
  };
  auto backward = [&](const int* skip) {
    if (!fused_backward_sweep(ws.pc32.nb, lay, batch, ws.M32.p, skip, s))
      lu_backward_rhs<float>(ws.pc32, lay, batch, ws.M32.p, skip, s);
  };
  span(2, [&] {
    backward(nullptr);
    launch_accumulate_correction(lay, batch, ws.M32.p, ws.rnorm.p, ws.X64.p, true, nullptr, nullptr, nullptr, s);
  });
  cudaMemsetAsync(ws.converged.p, 0, size_t(batch) * sizeof(int), s);
  cudaMemsetAsync(ws.iters.p, 0, size_t(batch) * sizeof(int), s);
  for (int it = 0; it < iters; ++it) {
    span(3, [&] {
      cudaMemsetAsync(ws.rnorm.p, 0, nb8, s);
      cudaMemsetAsync(ws.bnorm.p, 0, nb8, s);
      launch_residual(lay, batch, reinterpret_cast<const float4*>(ws.M64.p), ws.X64.p, ws.Xsplit.p, ws.R.p, ws.rnorm.p,
                      ws.bnorm.p, ws.converged.p, s, residual_tc(ws, rtc));
    });
    span(2, [&] {
      cudaMemsetAsync(ws.dnorm.p, 0, nb8, s);
      cudaMemsetAsync(ws.xnorm.p, 0, nb8, s);
      launch_residual_to_rhs32(lay, batch, ws.R.p, ws.rnorm.p, ws.M32.p, ws.converged.p, s);
      forward(ws.converged.p);
      backward(ws.converged.p);
      launch_accumulate_correction(lay, batch, ws.M32.p, ws.rnorm.p, ws.X64.p, false, ws.converged.p, ws.dnorm.p,
                                   ws.xnorm.p, s);
      launch_ir_check(batch, ws.rnorm.p, ws.bnorm.p, ws.dnorm.p, ws.xnorm.p, tol, ws.converged.p, ws.iters.p,
                      ws.relres.p, ws.dprev.p, s);
    });
  }
  return cudaGetLastError();
}

__global__ void add_iterations_kernel(int batch, const int* iters, int* total) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch) total[b] += iters[b];
}

BicgWork bicg_work(Workspace& ws) {
  BicgWork w;
  w.vec = ws.bicg_vec.p;
  w.sc = ws.bicg_sc.p;
  w.state = ws.bicg_state.p;
  w.done = ws.bicg_done.p;
  w.iters = ws.bicg_iters.p;
  w.active = ws.bicg_active.p;
  w.part = ws.bicg_part.p;
  w.act = ws.bicg_act.p;
  w.tc_err = ws.bicg_err.p;
  return w;
}

// BiCGSTAB form: the same refinement as refine_fp32 with the FP32 LU solves
// replaced by preconditioned BiCGSTAB solves on the unfactored FP32 matrix
// (M32 holds A and, in its last m columns, the right-hand side).  A system
// whose BiCGSTAB solve misses its tolerance within the iteration cap is
// marked converged = 2 and handed to the refined LU by the caller.
cudaError_t refine_bicgstab(Workspace& ws, int batch, const float2* D, const BlockPrecond* blk, int iters, double tol,
                            int max_iter, double inner_tol, int poll, int tensor, cudaStream_t s,
                            Spans* spans = nullptr) {
  const BatchLayout& lay = ws.lay;
  ResidualTc rtc;
  BicgWork w = bicg_work(ws);
  w.tensor = tensor;
  auto span = [&](int phase, auto&& fn) -> cudaError_t {
    cudaEvent_t a = nullptr, b = nullptr;
    if (spans) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, s);
    }
    cudaError_t e = fn();
    if (spans) {
      cudaEventRecord(b, s);
      spans->push_back({phase, {a, b}});
    }
    return e;
  };
  const size_t nb8 = size_t(batch) * sizeof(unsigned long long);
  cudaMemsetAsync(ws.converged.p, 0, size_t(batch) * sizeof(int), s);
  cudaMemsetAsync(ws.iters.p, 0, size_t(batch) * sizeof(int), s);
  cudaMemsetAsync(ws.bicg_total.p, 0, size_t(batch) * sizeof(int), s);
  auto solve = [&]() -> cudaError_t {
    cudaError_t e = bicgstab_solve(lay, batch, ws.M32.p, D, blk, w, inner_tol, max_iter, poll, ws.converged.p,
                                   ws.converged.p, s);
    count_launch();
    add_iterations_kernel<<<(batch + 127) / 128, 128, 0, s>>>(batch, ws.bicg_iters.p, ws.bicg_total.p);
    return e != cudaSuccess ? e : cudaGetLastError();
  };
  cudaError_t e = span(1, [&] {
    cudaError_t e1 = solve();
    launch_accumulate_correction(lay, batch, ws.M32.p, ws.rnorm.p, ws.X64.p, true, nullptr, nullptr, nullptr, s);
    return e1;
  });
  if (e != cudaSuccess) return e;
  for (int it = 0; it < iters; ++it) {
    span(3, [&] {
      cudaMemsetAsync(ws.rnorm.p, 0, nb8, s);
      cudaMemsetAsync(ws.bnorm.p, 0, nb8, s);
      launch_residual(lay, batch, reinterpret_cast<const float4*>(ws.M64.p), ws.X64.p, ws.Xsplit.p, ws.R.p, ws.rnorm.p,
                      ws.bnorm.p, ws.converged.p, s, residual_tc(ws, rtc));
      return cudaGetLastError();
    });
    e = span(1, [&] {
      cudaMemsetAsync(ws.dnorm.p, 0, nb8, s);
      cudaMemsetAsync(ws.xnorm.p, 0, nb8, s);
      launch_residual_to_rhs32(lay, batch, ws.R.p, ws.rnorm.p, ws.M32.p, ws.converged.p, s);
      cudaError_t e1 = solve();
      launch_accumulate_correction(lay, batch, ws.M32.p, ws.rnorm.p, ws.X64.p, false, ws.converged.p, ws.dnorm.p,
                                   ws.xnorm.p, s);
      launch_ir_check(batch, ws.rnorm.p, ws.bnorm.p, ws.dnorm.p, ws.xnorm.p, tol, ws.converged.p, ws.iters.p,
                      ws.relres.p, ws.dprev.p, s);
      return e1;
    });
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

// save_gg_slice outputs of one batch (build_saved_fms_scattering_outputs,
// engine/fms.rs:4154-4216) from X = (I - G0 T)^-1 G0, in reference state order:
// reference atom a is device atom a - 1 and the absorber (a = 0) device atom
// N - 1; every atom carries b states.  Per energy: rows [0, b) of X over every
// column (b x n, column-major), then the b x b diagonal block of each atom
// (column-major); zeros for energies that failed.
__global__ void extract_full_kernel(BatchLayout lay, int N, int b, const double2* __restrict__ X64, int per,
                                    double2* __restrict__ out, const int* status) {
  const int e = blockIdx.y;
  const bool bad = status[e] != kDevOk;
  const int n = lay.n;
  const size_t xb = size_t(e) * lay.lda * lay.m;
  auto dstate = [N, b](int st) {
    const int a = st / b;
    return (a == 0 ? N - 1 : a - 1) * b + (st - a * b);
  };
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < per; idx += gridDim.x * blockDim.x) {
    int r, c;
    if (idx < b * n) {
      r = idx % b;
      c = idx / b;
    } else {
      const int j = idx - b * n, a = j / (b * b), q = j - a * b * b;
      r = a * b + q % b;
      c = a * b + q / b;
    }
    out[size_t(e) * per + idx] =
        bad ? make_double2(0.0, 0.0) : X64[xb + size_t(dstate(r)) + size_t(lay.lda) * size_t(dstate(c))];
  }
}

__global__ void status_not_converged_kernel(int batch, const int* converged, int* status) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < batch && converged[b] != 1 && status[b] == kDevOk) status[b] = kDevNotConverged;
}

// One batch of energies from the staging buffers (k_stage, x_stage) into gg_stage/status.
// With profiling on, CUDA events bracket each phase (see refeff_fms_plan_phase_times).
cudaError_t run_fms_batch(refeff_fms_plan& p, Workspace& ws, int batch, refeff_fms_form form, cudaStream_t s) {
  const BatchLayout& lay = ws.lay;
  BuildScratch bscratch;
  bscratch.hank = ws.hank.p;
  bscratch.hflag = ws.hflag.p;
  const BuildScratch* bs = ws.hank.p && ws.hflag.p ? &bscratch : nullptr;
  cudaMemsetAsync(ws.status.p, 0, size_t(batch) * sizeof(int), s);
  cudaMemsetAsync(ws.info.p, 0, size_t(batch) * sizeof(int), s);
  const bool prof = p.profiling;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> spans;
  ws.tc_spans.on = prof;
  auto tick = [&](int phase, auto&& fn) -> cudaError_t {
    cudaEvent_t a = nullptr, b = nullptr;
    if (prof) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, s);
    }
    cudaError_t e = fn();
    if (prof) {
      cudaEventRecord(b, s);
      spans.push_back({phase, {a, b}});
    }
    return e;
  };
  cudaError_t e = cudaSuccess;
  if (p.minv != 0) {
    // FEFF iterative forms: G0 and the per-state T table, then one CTA per
    // (energy, absorber column) runs the minv solver on W = I - T G0
    tick(0, [&] {
      launch_build_g0(p.P, batch, ws.k_stage.p, lay, ws.M64.p, ws.status.p, s, bs);
      launch_t_table(p.P, batch, ws.x_stage.p, ws.t_tab.p, ws.status.p, s);
      return cudaGetLastError();
    });
    e = tick(1, [&] {
      return launch_iterative(form == REFEFF_FMS_FORM_FP64_LU, p.minv, lay, batch, ws.M64.p, ws.M32.p, ws.t_tab.p,
                              p.d_partner.p, p.toler1, p.toler2, ws.grow.p, ws.iter_scratch.p, p.d_blocks.p,
                              int(p.blocks.size()), p.gg_per, ws.gg_stage.p, ws.status.p, s);
    });
    if (e != cudaSuccess) return e;
  } else if (form == REFEFF_FMS_FORM_FP64_LU) {
    tick(0, [&] {
      launch_build_system(p.P, batch, ws.k_stage.p, ws.x_stage.p, lay, ws.M64.p, nullptr, ws.status.p, s, bs);
      return cudaGetLastError();
    });
    e = tick(1, [&] { return lu_eliminate<double>(ws.pc64, lay, batch, ws.M64.p, lu_work(ws, ws.pc64), s); });
    if (e != cudaSuccess) return e;
    tick(4, [&] {
      if (p.blocks.size() == 1 && !p.full) {
        // the absorber alone: its block is the trailing m x m triangle solve
        launch_absorber_solve<double>(lay, batch, ws.M64.p, ws.gg_stage.p, ws.status.p, s);
      } else {
        lu_backward_rhs<double>(ws.pc64, lay, batch, ws.M64.p, nullptr, s);
        launch_copy_rhs64(lay, batch, ws.M64.p, ws.X64.p, s);
        launch_extract_blocks(lay, batch, ws.X64.p, p.d_blocks.p, int(p.blocks.size()), p.gg_per, ws.gg_stage.p,
                              ws.status.p, s);
        if (p.full) {
          dim3 grid(unsigned(std::min(256, (p.full_per + 255) / 256)), unsigned(batch));
          count_launch();
          extract_full_kernel<<<grid, 256, 0, s>>>(lay, p.N, p.C, ws.X64.p, p.full_per, ws.full_stage.p, ws.status.p);
        }
      }
      return cudaGetLastError();
    });
  } else if (form == REFEFF_FMS_FORM_BICGSTAB) {
    tick(0, [&] {
      launch_build_system(p.P, batch, ws.k_stage.p, ws.x_stage.p, lay, ws.M64.p, ws.M32.p, ws.status.p, s, bs);
      if (p.model) {
        // learned diagonal: features -> network -> D per state
        const MlpShape& sh = *model_shape(p.model);
        launch_features(batch, p.N, p.L, p.nsp, p.npot, ws.k_stage.p, ws.x_stage.p, p.d_atom_pot.p,
                        p.d_shell_info.p, p.d_shell_pots.p, ws.feat_X.p, s);
        cudaError_t e1 = mlp_forward(sh, model_params(p.model), batch * p.N, ws.feat_X.p, ws.mlp, ws.feat_Y.p, s);
        if (e1 != cudaSuccess) return e1;
        if (model_kind(p.model) == kPrecondBlock)
          launch_scatter_block(batch, p.N, p.L, p.d_atom_lmax.p, ws.feat_Y.p, ws.k_stage.p, p.precond_e_lo,
                               p.precond_e_hi, ws.precond_B.p, s);
        else
          launch_scatter_diag(batch, p.N, p.L, p.nsp, lay.lda, p.d_atom_off.p, p.d_atom_lmax.p, ws.feat_Y.p,
                              ws.k_stage.p, p.precond_e_lo, p.precond_e_hi, ws.precond_D.p, s);
      }
      return cudaGetLastError();
    });
    const bool block = p.model && model_kind(p.model) == kPrecondBlock;
    BlockPrecond blk;
    blk.B = ws.precond_B.p;
    blk.state_atom = p.d_state_atom.p;
    blk.atom_off = p.d_atom_off.p;
    blk.N = p.N;
    blk.C = (p.L + 1) * (p.L + 1);
    e = refine_bicgstab(ws, batch, p.model && !block ? ws.precond_D.p : nullptr, block ? &blk : nullptr,
                        p.refine_iters, p.refine_tol, p.bicg_max_iter, p.bicg_tol, p.bicg_poll, p.ctx->bicg_tensor,
                        s, prof ? &spans : nullptr);
    if (e != cudaSuccess) return e;
    tick(4, [&] {
      count_launch();
      status_not_converged_kernel<<<(batch + 127) / 128, 128, 0, s>>>(batch, ws.converged.p, ws.status.p);
      launch_extract_blocks(lay, batch, ws.X64.p, p.d_blocks.p, int(p.blocks.size()), p.gg_per, ws.gg_stage.p,
                            nullptr, s);
      return cudaGetLastError();
    });
  } else {
    tick(0, [&] {
      launch_build_system(p.P, batch, ws.k_stage.p, ws.x_stage.p, lay, ws.M64.p, ws.M32.p, ws.status.p, s, bs);
      return cudaGetLastError();
    });
    e = tick(1, [&] { return lu_eliminate<float>(ws.pc32, lay, batch, ws.M32.p, lu_work(ws, ws.pc32), s); });
    if (e != cudaSuccess) return e;
    e = refine_fp32(ws, batch, p.refine_iters, p.refine_tol, s, prof ? &spans : nullptr);
    if (e != cudaSuccess) return e;
    tick(4, [&] {
      count_launch();
      status_not_converged_kernel<<<(batch + 127) / 128, 128, 0, s>>>(batch, ws.converged.p, ws.status.p);
      launch_extract_blocks(lay, batch, ws.X64.p, p.d_blocks.p, int(p.blocks.size()), p.gg_per, ws.gg_stage.p,
                            nullptr, s);
      return cudaGetLastError();
    });
  }
  if (prof) {
    cudaStreamSynchronize(s);
    KernelSpans& tc = ws.tc_spans;
    for (auto& sp : tc.spans) spans.push_back({5, sp});
    tc.spans.clear();
    tc.on = false;
    for (auto& sp : spans) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, sp.second.first, sp.second.second);
      p.phase_ms[sp.first] += ms;
      cudaEventDestroy(sp.second.first);
      cudaEventDestroy(sp.second.second);
    }
  }
  return cudaGetLastError();
}

int map_status(int dev) {
  switch (dev) {
    case kDevOk: return REFEFF_FMS_OK;
    case kDevSingular: return REFEFF_FMS_ERR_SINGULAR_MATRIX;
    case kDevNonfinite: return REFEFF_FMS_ERR_NONFINITE_INPUT;
    case kDevZeroRho: return REFEFF_FMS_ERR_ZERO_RHO;
    case kDevNotConverged: return REFEFF_FMS_ERR_NOT_CONVERGED;
    case kDevBreakdown: return REFEFF_FMS_ERR_ITERATIVE_BREAKDOWN;
    default: return REFEFF_FMS_ERR_CUDA;
  }
}

int pick_batch(refeff_fms_plan& p, int E, bool fp32) {
  if (p.max_batch > 0) return std::min(E, p.max_batch);
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const BatchLayout lay = make_layout(p.n, p.m);
  size_t per = bytes_per_system(lay, fp32);
  if (p.full) per += (size_t(lay.lda) * p.m + size_t(p.full_per)) * sizeof(double2);
  per += build_scratch_entries(p.P, 1) * sizeof(double2) + size_t(p.N) * p.N * sizeof(int);
  const size_t budget = size_t(double(free_b) * 0.5);
  int b = int(std::max<size_t>(1, budget / std::max<size_t>(per, 1)));
  b = std::min(b, 256);
  return std::min(E, b);
}

// FP64_LU and FP32_REFINED serve every plan; BICGSTAB the LU-form plans (minv = 0).
bool form_valid(const refeff_fms_plan& p, refeff_fms_form form) {
  if (p.full) return form == REFEFF_FMS_FORM_FP64_LU;  // the full matrix is solved by the LU form only
  return form == REFEFF_FMS_FORM_FP64_LU || form == REFEFF_FMS_FORM_FP32_REFINED ||
         (form == REFEFF_FMS_FORM_BICGSTAB && p.minv == 0);
}

// E - E_ref in eV of a wave number in 1/Angstrom: Re((k a0)^2) / 2 Hartree, the
// definition the learned preconditioner's window uses on the device.
double energy_above_eref_ev(double2 k) {
  constexpr double kBohr = 0.529177249, kHartreeEv = 27.211396;
  return 0.5 * (k.x * k.x - k.y * k.y) * kBohr * kBohr * kHartreeEv;
}

// Results of batch slot i of a workspace -> energy e of the call's outputs
// (gg block, status, full-scattering slice, refinement statistics).
cudaError_t copy_energy_results(refeff_fms_plan& p, Workspace& ws, int i, int e, double2* d_gg, int* d_status,
                                cudaStream_t q) {
  cudaError_t r = cudaMemcpyAsync(d_gg + size_t(e) * p.gg_per, ws.gg_stage.p + size_t(i) * p.gg_per,
                                  size_t(p.gg_per) * sizeof(double2), cudaMemcpyDeviceToDevice, q);
  if (!r) r = cudaMemcpyAsync(d_status + e, ws.status.p + i, sizeof(int), cudaMemcpyDeviceToDevice, q);
  if (!r && p.full)
    r = cudaMemcpyAsync(p.d_full_all.p + size_t(e) * p.full_per, ws.full_stage.p + size_t(i) * p.full_per,
                        size_t(p.full_per) * sizeof(double2), cudaMemcpyDeviceToDevice, q);
  if (!r && p.minv == 0 && p.d_relres_all.p && ws.relres.p) {
    r = cudaMemcpyAsync(p.d_relres_all.p + e, ws.relres.p + i, sizeof(double), cudaMemcpyDeviceToDevice, q);
    if (!r) r = cudaMemcpyAsync(p.d_iters_all.p + e, ws.iters.p + i, sizeof(int), cudaMemcpyDeviceToDevice, q);
  }
  return r;
}

// Solve E energies whose inputs are already on the device (d_k: E*nsp, d_x:
// E*xph); writes d_gg (E*m*m) and d_status (E).  Uses graph replay per batch.
// With two streams (allow_dual, the context's REFEFF_FMS_OPT_DUAL_STREAMS,
// graph replay possible, E >= 8, room for a second workspace) the energies are
// split into batches alternating between two workspaces on two streams (the
// caller's stream and one of the plan's, forked and joined with events), so
// that one batch's latency-bound phases (panels, sweeps) overlap the other's
// arithmetic-bound ones (build, residual, tensor-core updates).
// `batch` > 0 fixes the batch size (one stream); `direct` runs every batch
// un-captured, for a caller that is itself capturing the stream.
int solve_device_energies_enqueue(refeff_fms_plan& p, int E, const double2* d_k, const double2* d_x, refeff_fms_form form,
                          double2* d_gg, int* d_status, cudaStream_t s, bool allow_dual = true, int batch = 0,
                          bool direct = false) {
  refeff_fms_context* ctx = p.ctx;
  const bool fp32 = form != REFEFF_FMS_FORM_FP64_LU;  // the BiCGSTAB form uses the refined form's buffers
  const bool bicg = form == REFEFF_FMS_FORM_BICGSTAB;
  bool dual = allow_dual && ctx->dual_streams && !p.profiling && !bicg && E >= 8 && batch <= 0;
  const int B = batch > 0 ? std::min(batch, E) : pick_batch(p, dual ? (E + 1) / 2 : E, fp32);
  const bool refined = fp32 && p.minv == 0;  // refinement statistics and the FP64 fallback
  const size_t xph = p.xph_per_energy();
  if (p.full) RF_CUDA(ctx, p.d_full_all.alloc(size_t(E) * p.full_per));
  if (refined) {
    RF_CUDA(ctx, p.d_relres_all.alloc(size_t(E)));
    RF_CUDA(ctx, p.d_iters_all.alloc(size_t(E)));
  }
  if (bicg) RF_CUDA(ctx, p.d_bicg_iters_all.alloc(size_t(E)));
  auto prepare = [&](Workspace& ws) -> int {
  int rc = ensure_workspace(ctx, ws, p.n, p.m, B, fp32, &p.tune);
  if (rc) return rc;
  RF_CUDA(ctx, ws.k_stage.alloc(size_t(ws.batch) * p.nsp));
  RF_CUDA(ctx, ws.x_stage.alloc(size_t(ws.batch) * xph));
  RF_CUDA(ctx, ws.gg_stage.alloc(size_t(ws.batch) * p.gg_per));
  if (!fp32 && (p.blocks.size() > 1 || p.full)) RF_CUDA(ctx, ws.X64.alloc(size_t(ws.batch) * ws.lay.lda * p.m));
  RF_CUDA(ctx, ws.hank.alloc(build_scratch_entries(p.P, ws.batch)));
  RF_CUDA(ctx, ws.hflag.alloc(size_t(ws.batch) * p.N * p.N));
  if (p.full) RF_CUDA(ctx, ws.full_stage.alloc(size_t(ws.batch) * p.full_per));
  if (p.minv != 0) {
    RF_CUDA(ctx, ws.t_tab.alloc(size_t(ws.batch) * p.n * 2));
    RF_CUDA(ctx, ws.grow.alloc(size_t(ws.batch) * p.m * p.n));
    RF_CUDA(ctx, ws.iter_scratch.alloc(size_t(ws.batch) * p.m * kIterVectors * p.n));
  }
  if (bicg) {
    const size_t cols = size_t(ws.batch) * p.m;
    RF_CUDA(ctx, ws.bicg_vec.alloc(size_t(kBicgVectors) * cols * ws.lay.lda));
    const int slices = std::max(bicg_slices(p.n, false), bicg_slices(p.n, ctx->bicg_tensor != 0));
    RF_CUDA(ctx, ws.bicg_part.alloc(size_t(slices - 1) * cols * ws.lay.lda));
    RF_CUDA(ctx, ws.bicg_act.alloc(size_t(ws.batch)));
    RF_CUDA(ctx, ws.bicg_err.alloc(1));
    RF_CUDA(ctx, ws.bicg_sc.alloc(cols * kBicgScalars));
    RF_CUDA(ctx, ws.bicg_state.alloc(cols));
    RF_CUDA(ctx, ws.bicg_done.alloc(size_t(ws.batch)));
    RF_CUDA(ctx, ws.bicg_iters.alloc(size_t(ws.batch)));
    RF_CUDA(ctx, ws.bicg_total.alloc(size_t(ws.batch)));
    RF_CUDA(ctx, ws.bicg_active.alloc(1));
    if (p.model) {
      const MlpShape& sh = *model_shape(p.model);
      RF_CUDA(ctx, ws.precond_D.alloc(size_t(ws.batch) * ws.lay.lda));
      if (model_kind(p.model) == kPrecondBlock)
        RF_CUDA(ctx, ws.precond_B.alloc(size_t(ws.batch) * p.N * size_t((p.L + 1) * (p.L + 1)) * (p.L + 1) * (p.L + 1)));
      RF_CUDA(ctx, ws.feat_X.alloc(size_t(ws.batch) * p.N * sh.F));
      RF_CUDA(ctx, ws.feat_Y.alloc(size_t(ws.batch) * p.N * sh.O));
    }
  }
  return REFEFF_FMS_OK;
  };
  int rc = prepare(p.ws);
  if (rc) return rc;
  if (dual && !(p.ws2.batch >= B && p.ws2.lay.n == p.n && p.ws2.lay.m == p.m && (p.ws2.fp32 || !fp32))) {
    // a second workspace only where it fits beside the first with room to spare
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t need = bytes_per_system(make_layout(p.n, p.m), fp32) * size_t(B) +
                        (p.ws.use_tc ? tc_image_bytes(p.n, p.m, B) : 0) +
                        build_scratch_entries(p.P, B) * sizeof(double2);
    if (double(need) > 0.8 * double(free_b)) dual = false;
  }
  if (dual) {
    rc = prepare(p.ws2);
    if (rc) return rc;
    if (!p.s2) {
      RF_CUDA(ctx, cudaStreamCreateWithFlags(&p.s2, cudaStreamNonBlocking));
      RF_CUDA(ctx, cudaEventCreateWithFlags(&p.fork_ev, cudaEventDisableTiming));
      RF_CUDA(ctx, cudaEventCreateWithFlags(&p.join_ev, cudaEventDisableTiming));
    }
    RF_CUDA(ctx, cudaEventRecord(p.fork_ev, s));  // the second stream starts after the caller's earlier work
    RF_CUDA(ctx, cudaStreamWaitEvent(p.s2, p.fork_ev, 0));
  }
  // BiCGSTAB energy window: energies outside it skip the iteration and are
  // solved by the refined LU in the finish step
  bool routed = false;
  if (bicg) {
    p.bicg_lu.assign(size_t(E), 0);
    p.bicg_order.clear();
    RF_CUDA(ctx, cudaMemsetAsync(p.d_bicg_iters_all.p, 0, size_t(E) * sizeof(int), s));
    if (p.bicg_e_lo > -1e299 || p.bicg_e_hi < 1e299) {
      std::vector<double2> hk(size_t(E) * p.nsp);
      RF_CUDA(ctx, cudaMemcpyAsync(hk.data(), d_k, hk.size() * sizeof(double2), cudaMemcpyDeviceToHost, s));
      RF_CUDA(ctx, cudaStreamSynchronize(s));
      for (int e = 0; e < E; ++e) {
        const double ev = energy_above_eref_ev(hk[size_t(e) * p.nsp]);
        if (ev >= p.bicg_e_lo && ev <= p.bicg_e_hi) p.bicg_order.push_back(e);
        else p.bicg_lu[size_t(e)] = 2;
      }
      routed = int(p.bicg_order.size()) != E;
    }
  }
  const int Eit = routed ? int(p.bicg_order.size()) : E;  // energies this loop solves
  auto energy_of = [&](int i) { return routed ? p.bicg_order[size_t(i)] : i; };
  int batch_index = 0;
  for (int e0 = 0; e0 < Eit; e0 += B, ++batch_index) {
    const int nb = std::min(B, Eit - e0);
    const bool second = dual && (batch_index & 1);
    Workspace& ws = second ? p.ws2 : p.ws;
    const cudaStream_t q = second ? p.s2 : s;
    if (routed) {
      for (int i = 0; i < nb; ++i) {
        const int e = energy_of(e0 + i);
        RF_CUDA(ctx, cudaMemcpyAsync(ws.k_stage.p + size_t(i) * p.nsp, d_k + size_t(e) * p.nsp,
                                     p.nsp * sizeof(double2), cudaMemcpyDeviceToDevice, q));
        RF_CUDA(ctx, cudaMemcpyAsync(ws.x_stage.p + size_t(i) * xph, d_x + size_t(e) * xph, xph * sizeof(double2),
                                     cudaMemcpyDeviceToDevice, q));
      }
    } else {
      RF_CUDA(ctx, cudaMemcpyAsync(ws.k_stage.p, d_k + size_t(e0) * p.nsp, size_t(nb) * p.nsp * sizeof(double2),
                                   cudaMemcpyDeviceToDevice, q));
      RF_CUDA(ctx, cudaMemcpyAsync(ws.x_stage.p, d_x + size_t(e0) * xph, size_t(nb) * xph * sizeof(double2),
                                   cudaMemcpyDeviceToDevice, q));
    }
    if (nb == B && !p.profiling && !bicg && !direct) {  // the BiCGSTAB form polls the host: not capturable
      // a graph bakes in its batch size: key by (form, energies in the batch)
      const int key = int(form) * 65536 + nb;
      auto it = ws.graphs.find(key);
      if (it == ws.graphs.end()) {
        // first run un-captured (sets kernel attributes), then capture
        cudaError_t e = run_fms_batch(p, ws, nb, form, q);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "fms batch");
        cudaGraph_t g = nullptr;
        RF_CUDA(ctx, cudaStreamBeginCapture(q, cudaStreamCaptureModeThreadLocal));
        const unsigned long long before = g_launches.load();
        e = run_fms_batch(p, ws, nb, form, q);
        ws.graph_launches[key] = g_launches.load() - before;
        cudaError_t e2 = cudaStreamEndCapture(q, &g);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "fms batch capture");
        if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "end capture");
        cudaGraphExec_t ge = nullptr;
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "graph instantiate");
        ws.graphs[key] = ge;
      } else {
        RF_CUDA(ctx, cudaGraphLaunch(it->second, q));
        g_launches.fetch_add(ws.graph_launches[key], std::memory_order_relaxed);
      }
    } else {
      cudaError_t e = run_fms_batch(p, ws, nb, form, q);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "fms batch");
    }
    if (routed) {  // scatter the batch's results back to its energies
      for (int i = 0; i < nb; ++i) {
        RF_CUDA(ctx, copy_energy_results(p, ws, i, energy_of(e0 + i), d_gg, d_status, q));
        RF_CUDA(ctx, cudaMemcpyAsync(p.d_bicg_iters_all.p + energy_of(e0 + i), ws.bicg_total.p + i, sizeof(int),
                                     cudaMemcpyDeviceToDevice, q));
      }
      continue;
    }
    RF_CUDA(ctx, cudaMemcpyAsync(d_gg + size_t(e0) * p.gg_per, ws.gg_stage.p, size_t(nb) * p.gg_per * sizeof(double2),
                                 cudaMemcpyDeviceToDevice, q));
    RF_CUDA(ctx, cudaMemcpyAsync(d_status + e0, ws.status.p, size_t(nb) * sizeof(int), cudaMemcpyDeviceToDevice, q));
    if (p.full)
      RF_CUDA(ctx, cudaMemcpyAsync(p.d_full_all.p + size_t(e0) * p.full_per, ws.full_stage.p,
                                   size_t(nb) * p.full_per * sizeof(double2), cudaMemcpyDeviceToDevice, q));
    if (refined) {
      RF_CUDA(ctx, cudaMemcpyAsync(p.d_relres_all.p + e0, ws.relres.p, size_t(nb) * sizeof(double),
                                   cudaMemcpyDeviceToDevice, q));
      RF_CUDA(ctx, cudaMemcpyAsync(p.d_iters_all.p + e0, ws.iters.p, size_t(nb) * sizeof(int),
                                   cudaMemcpyDeviceToDevice, q));
    }
    if (bicg)
      RF_CUDA(ctx, cudaMemcpyAsync(p.d_bicg_iters_all.p + e0, ws.bicg_total.p, size_t(nb) * sizeof(int),
                                   cudaMemcpyDeviceToDevice, q));
  }
  if (dual) {
    RF_CUDA(ctx, cudaEventRecord(p.join_ev, p.s2));  // the caller's stream resumes after both
    RF_CUDA(ctx, cudaStreamWaitEvent(s, p.join_ev, 0));
  }
  return REFEFF_FMS_OK;
}

// Completion of solve_device_energies_enqueue: waits for the stream, then
// re-solves with the FP64 LU the energies whose refinement missed.
int solve_device_energies_finish(refeff_fms_plan& p, int E, const double2* d_k, const double2* d_x,
                                 refeff_fms_form form, double2* d_gg, int* d_status, cudaStream_t s) {
  refeff_fms_context* ctx = p.ctx;
  Workspace& ws = p.ws;
  const bool refined = form != REFEFF_FMS_FORM_FP64_LU && p.minv == 0;
  const int B = ws.batch;
  const size_t xph = p.xph_per_energy();
  if (!refined) return REFEFF_FMS_OK;
  // Energies whose refinement missed the tolerance are solved again with the
  // plain FP64 LU (same inputs), so every returned block meets the FP64 bar.
  std::vector<int> st(static_cast<size_t>(E));
  RF_CUDA(ctx, cudaMemcpyAsync(st.data(), d_status, size_t(E) * sizeof(int), cudaMemcpyDeviceToHost, s));
  int tc_timeout = 0, tc_timeout2 = 0;
  if (ws.use_tc) RF_CUDA(ctx, cudaMemcpyAsync(&tc_timeout, ws.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (p.ws2.use_tc && p.ws2.tc_err.p)
    RF_CUDA(ctx, cudaMemcpyAsync(&tc_timeout2, p.ws2.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  RF_CUDA(ctx, cudaStreamSynchronize(s));
  if (tc_timeout || tc_timeout2) {
    // A tensor-core wait gave up: the update of that batch is incomplete, so
    // every FP32 result is redone on the FP64 LU below.
    for (auto& v : st)
      if (v == kDevOk) v = kDevNotConverged;
    RF_CUDA(ctx, cudaMemsetAsync(ws.tc_err.p, 0, sizeof(int), s));
    if (tc_timeout2) RF_CUDA(ctx, cudaMemsetAsync(p.ws2.tc_err.p, 0, sizeof(int), s));
    ctx->last_error = "tensor-core update timed out; energies re-solved with the FP64 LU";
  }
  if (form == REFEFF_FMS_FORM_BICGSTAB) {
    // The BiCGSTAB form's energies that missed the tolerance within the
    // iteration cap, and those outside its window, are solved by the refined
    // LU (FP32 factorisation + FP64 refinement); what that misses goes on to
    // the FP64 LU below.
    std::vector<int> lu;
    for (int e = 0; e < E; ++e) {
      if (p.bicg_lu[size_t(e)] == 2) {
        lu.push_back(e);
      } else if (st[size_t(e)] == kDevNotConverged) {
        p.bicg_lu[size_t(e)] = 1;
        lu.push_back(e);
      }
    }
    for (size_t r0 = 0; r0 < lu.size(); r0 += size_t(B)) {
      const int nb = int(std::min(lu.size() - r0, size_t(B)));
      for (int i = 0; i < nb; ++i) {
        const int e = lu[r0 + size_t(i)];
        RF_CUDA(ctx, cudaMemcpyAsync(ws.k_stage.p + size_t(i) * p.nsp, d_k + size_t(e) * p.nsp,
                                     p.nsp * sizeof(double2), cudaMemcpyDeviceToDevice, s));
        RF_CUDA(ctx, cudaMemcpyAsync(ws.x_stage.p + size_t(i) * xph, d_x + size_t(e) * xph, xph * sizeof(double2),
                                     cudaMemcpyDeviceToDevice, s));
      }
      cudaError_t e = run_fms_batch(p, ws, nb, REFEFF_FMS_FORM_FP32_REFINED, s);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "refined LU batch of the BiCGSTAB form");
      for (int i = 0; i < nb; ++i) RF_CUDA(ctx, copy_energy_results(p, ws, i, lu[r0 + size_t(i)], d_gg, d_status, s));
    }
    if (!lu.empty()) {
      RF_CUDA(ctx, cudaMemcpyAsync(st.data(), d_status, size_t(E) * sizeof(int), cudaMemcpyDeviceToHost, s));
      int lu_timeout = 0;
      if (ws.use_tc) RF_CUDA(ctx, cudaMemcpyAsync(&lu_timeout, ws.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      RF_CUDA(ctx, cudaStreamSynchronize(s));
      if (lu_timeout) {
        for (int e : lu) st[size_t(e)] = kDevNotConverged;
        RF_CUDA(ctx, cudaMemsetAsync(ws.tc_err.p, 0, sizeof(int), s));
        ctx->last_error = "tensor-core update timed out; energies re-solved with the FP64 LU";
      }
    }
  }
  std::vector<int> redo;
  for (int e = 0; e < E; ++e)
    if (st[size_t(e)] == kDevNotConverged) redo.push_back(e);
  p.last_fallback = redo;
  p.last_fallbacks = int(redo.size());
  for (size_t r0 = 0; r0 < redo.size(); r0 += size_t(B)) {
    const int nb = int(std::min(redo.size() - r0, size_t(B)));
    for (int i = 0; i < nb; ++i) {
      const int e = redo[r0 + size_t(i)];
      RF_CUDA(ctx, cudaMemcpyAsync(ws.k_stage.p + size_t(i) * p.nsp, d_k + size_t(e) * p.nsp, p.nsp * sizeof(double2),
                                   cudaMemcpyDeviceToDevice, s));
      RF_CUDA(ctx, cudaMemcpyAsync(ws.x_stage.p + size_t(i) * xph, d_x + size_t(e) * xph, xph * sizeof(double2),
                                   cudaMemcpyDeviceToDevice, s));
    }
    cudaError_t e = run_fms_batch(p, p.ws, nb, REFEFF_FMS_FORM_FP64_LU, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "fp64 fallback batch");
    for (int i = 0; i < nb; ++i) {
      const int en = redo[r0 + size_t(i)];
      RF_CUDA(ctx, cudaMemcpyAsync(d_gg + size_t(en) * p.gg_per, ws.gg_stage.p + size_t(i) * p.gg_per,
                                   size_t(p.gg_per) * sizeof(double2), cudaMemcpyDeviceToDevice, s));
      RF_CUDA(ctx, cudaMemcpyAsync(d_status + en, ws.status.p + i, sizeof(int), cudaMemcpyDeviceToDevice, s));
    }
  }
  return REFEFF_FMS_OK;
}

int solve_device_energies(refeff_fms_plan& p, int E, const double2* d_k, const double2* d_x, refeff_fms_form form,
                          double2* d_gg, int* d_status, cudaStream_t s) {
  const int rc = solve_device_energies_enqueue(p, E, d_k, d_x, form, d_gg, d_status, s);
  if (rc) return rc;
  return solve_device_energies_finish(p, E, d_k, d_x, form, d_gg, d_status, s);
}

}  // namespace

extern "C" int refeff_fms_real_space_spectrum_device(refeff_fms_plan* plan, int n_energies, const void* d_wave_numbers,
                                                     const void* d_phase_shifts, refeff_fms_form form, void* d_gg_out,
                                                     int32_t* d_status, void* stream) {
  if (!plan || n_energies < 0 || (n_energies > 0 && (!d_wave_numbers || !d_phase_shifts || !d_gg_out || !d_status)))
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (!form_valid(*plan, form)) return fail(plan->ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "unknown form for this plan");
  if (n_energies == 0) return REFEFF_FMS_OK;
  RF_CUDA(plan->ctx, cudaSetDevice(plan->ctx->device));
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : plan->ctx->stream;
  return solve_device_energies(*plan, n_energies, static_cast<const double2*>(d_wave_numbers),
                               static_cast<const double2*>(d_phase_shifts), form, static_cast<double2*>(d_gg_out),
                               d_status, s);
}

namespace {

// Host-buffer spectrum in two halves, so that several plans can have their
// device work in flight at once: begin validates, uploads and enqueues on
// stream s; end waits, runs the FP64 fallback, downloads and scatters.
// First half of spectrum_begin: validation, the zeroed host table, the uploads
// of k and the phase shifts, and the device result buffers.
int spectrum_prepare(refeff_fms_plan& p, const refeff_fms_energy_points* points, refeff_fms_form form,
                     refeff_complex128* scattering_out, cudaStream_t s) {
  refeff_fms_context* ctx = p.ctx;
  if (!points || !scattering_out) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  const int E = points->n_energies;
  if (E < 0 || (E > 0 && (!points->wave_numbers || !points->phase_shifts)))
    return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "invalid energy points");
  if (!form_valid(p, form)) return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "unknown form for this plan");
  const size_t C = size_t(p.C), tab = C * C * size_t(p.npot);
  std::memset(scattering_out, 0, size_t(E) * tab * sizeof(refeff_complex128));
  if (E == 0) return REFEFF_FMS_OK;
  RF_CUDA(ctx, cudaSetDevice(ctx->device));
  const size_t xph = p.xph_per_energy();
  RF_CUDA(ctx, p.d_k_all.upload(reinterpret_cast<const double2*>(points->wave_numbers), size_t(E) * p.nsp, s));
  RF_CUDA(ctx, p.d_x_all.upload(reinterpret_cast<const double2*>(points->phase_shifts), size_t(E) * xph, s));
  RF_CUDA(ctx, p.d_gg_all.alloc(size_t(E) * p.gg_per));
  RF_CUDA(ctx, p.d_status_all.alloc(size_t(E)));
  return REFEFF_FMS_OK;
}

int spectrum_begin(refeff_fms_plan& p, const refeff_fms_energy_points* points, refeff_fms_form form,
                   refeff_complex128* scattering_out, cudaStream_t s, bool allow_dual = true, int batch = 0) {
  const int rc = spectrum_prepare(p, points, form, scattering_out, s);
  if (rc || points->n_energies == 0) return rc;
  return solve_device_energies_enqueue(p, points->n_energies, p.d_k_all.p, p.d_x_all.p, form, p.d_gg_all.p,
                                       p.d_status_all.p, s, allow_dual, batch);
}

int spectrum_end(refeff_fms_plan& p, const refeff_fms_energy_points* points, refeff_fms_form form,
                 refeff_complex128* scattering_out, int32_t* status_out, int* failed_out, cudaStream_t s) {
  refeff_fms_context* ctx = p.ctx;
  const int E = points->n_energies;
  *failed_out = 0;
  if (E == 0) return REFEFF_FMS_OK;
  const size_t C = size_t(p.C), tab = C * C * size_t(p.npot);
  int rc = solve_device_energies_finish(p, E, p.d_k_all.p, p.d_x_all.p, form, p.d_gg_all.p, p.d_status_all.p, s);
  if (rc) return rc;
  std::vector<double2> gg(size_t(E) * p.gg_per);
  std::vector<int> st(static_cast<size_t>(E));
  RF_CUDA(ctx, cudaMemcpyAsync(gg.data(), p.d_gg_all.p, gg.size() * sizeof(double2), cudaMemcpyDeviceToHost, s));
  RF_CUDA(ctx, cudaMemcpyAsync(st.data(), p.d_status_all.p, st.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  const bool fp32 = form != REFEFF_FMS_FORM_FP64_LU && p.minv == 0;  // refinement statistics exist
  p.last_relres.assign(fp32 ? size_t(E) : 0, 0.0);
  p.last_iters.assign(fp32 ? size_t(E) : 0, 0);
  p.last_bicg_iters.assign(form == REFEFF_FMS_FORM_BICGSTAB ? size_t(E) : 0, 0);
  if (form == REFEFF_FMS_FORM_BICGSTAB)
    RF_CUDA(ctx, cudaMemcpyAsync(p.last_bicg_iters.data(), p.d_bicg_iters_all.p, size_t(E) * sizeof(int),
                                 cudaMemcpyDeviceToHost, s));
  if (fp32) {
    RF_CUDA(ctx, cudaMemcpyAsync(p.last_relres.data(), p.d_relres_all.p, size_t(E) * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
    RF_CUDA(ctx, cudaMemcpyAsync(p.last_iters.data(), p.d_iters_all.p, size_t(E) * sizeof(int), cudaMemcpyDeviceToHost,
                                 s));
  }
  RF_CUDA(ctx, cudaStreamSynchronize(s));
  int failed = 0, first_bad = -1;
  for (int e = 0; e < E; ++e) {
    const int code = map_status(st[size_t(e)]);
    if (status_out) status_out[e] = code;
    if (code != REFEFF_FMS_OK && failed++ == 0) first_bad = e;
    refeff_complex128* outp = scattering_out + size_t(e) * tab;
    for (size_t q = 0; q < p.blocks.size(); ++q) {
      const SolvedBlock& bl = p.blocks[q];
      for (int c = 0; c < bl.size; ++c)
        for (int r = 0; r < bl.size; ++r) {
          const double2 v = gg[size_t(e) * p.gg_per + size_t(bl.pack) + size_t(r) + size_t(bl.size) * c];
          outp[size_t(r) + C * (size_t(c) + C * size_t(p.block_pot[q]))] = {v.x, v.y};
        }
    }
  }
  *failed_out = failed;
  if (failed)
    return fail(ctx, map_status(st[size_t(first_bad)]),
                "failed to solve FMS energy section " + std::to_string(first_bad + 1));
  return REFEFF_FMS_OK;
}

void fill_report(refeff_fms_report* report, const std::vector<refeff_fms_plan*>& plans, refeff_fms_form form,
                 int failed, std::chrono::steady_clock::time_point t0) {
  if (!report) return;
  report->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  report->energies_failed = failed;
  report->refinement_iterations = 0;
  report->residual_max = 0.0;
  report->fp64_fallbacks = 0;
  for (const refeff_fms_plan* p : plans) {
    for (size_t e = 0; e < p->last_iters.size(); ++e) {
      report->refinement_iterations = std::max(report->refinement_iterations, p->last_iters[e]);
      report->residual_max = std::max(report->residual_max, p->last_relres[e]);
    }
    if (form == REFEFF_FMS_FORM_FP32_REFINED && p->minv == 0) report->fp64_fallbacks += p->last_fallbacks;
  }
}

}  // namespace

extern "C" int refeff_fms_real_space_spectrum(refeff_fms_plan* plan, const refeff_fms_energy_points* points,
                                              refeff_fms_form form, refeff_complex128* scattering_out,
                                              int32_t* status_out, refeff_fms_report* report) {
  if (!plan || !points || !scattering_out) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  refeff_fms_context* ctx = plan->ctx;
  ctx->last_error.clear();
  const auto t0 = std::chrono::steady_clock::now();
  int rc = spectrum_begin(*plan, points, form, scattering_out, ctx->stream);
  if (rc) return rc;
  int failed = 0;
  rc = spectrum_end(*plan, points, form, scattering_out, status_out, &failed, ctx->stream);
  fill_report(report, {plan}, form, failed, t0);
  return rc;
}

extern "C" int refeff_fms_real_space_spectrum_full(refeff_fms_plan* plan, const refeff_fms_energy_points* points,
                                                   refeff_complex128* scattering_out, refeff_complex128* slice_out,
                                                   refeff_complex128* diag_out, int32_t* status_out,
                                                   refeff_fms_report* report) {
  if (!plan || !points || !scattering_out || !slice_out || !diag_out) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  refeff_fms_context* ctx = plan->ctx;
  ctx->last_error.clear();
  if (!plan->full)
    return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "the plan was not created for the full scattering matrix");
  const auto t0 = std::chrono::steady_clock::now();
  const refeff_fms_form form = REFEFF_FMS_FORM_FP64_LU;
  int rc = spectrum_begin(*plan, points, form, scattering_out, ctx->stream);
  if (rc) return rc;
  int failed = 0;
  rc = spectrum_end(*plan, points, form, scattering_out, status_out, &failed, ctx->stream);
  fill_report(report, {plan}, form, failed, t0);
  if (rc && !failed) return rc;
  const int E = points->n_energies;
  if (E > 0) {
    // per energy the device holds [slice b x n | diag N x b x b]: split into the two outputs
    const size_t b = size_t(plan->C), sl = b * size_t(plan->n), dg = size_t(plan->full_per) - sl;
    const size_t pitch = size_t(plan->full_per) * sizeof(double2);
    RF_CUDA(ctx, cudaMemcpy2D(slice_out, sl * sizeof(double2), plan->d_full_all.p, pitch, sl * sizeof(double2),
                              size_t(E), cudaMemcpyDeviceToHost));
    RF_CUDA(ctx, cudaMemcpy2D(diag_out, dg * sizeof(double2), plan->d_full_all.p + sl, pitch, dg * sizeof(double2),
                              size_t(E), cudaMemcpyDeviceToHost));
  }
  return rc;
}

extern "C" int refeff_fms_real_space_spectrum_multi(refeff_fms_context* ctx, int n_plans, refeff_fms_plan* const* plans,
                                                    const refeff_fms_energy_points* points, refeff_fms_form form,
                                                    refeff_complex128* const* scattering_out,
                                                    int32_t* const* status_out, refeff_fms_report* report) {
  if (!ctx || n_plans < 0 || (n_plans > 0 && (!plans || !points || !scattering_out)))
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  ctx->last_error.clear();
  for (int i = 0; i < n_plans; ++i)
    if (!plans[i] || plans[i]->ctx != ctx || !scattering_out[i])
      return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "plan " + std::to_string(i) + " is null or of another context");
  for (int i = 0; i < n_plans; ++i)
    for (int j = 0; j < i; ++j)
      if (plans[i] == plans[j]) return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "a plan appears twice");
  const auto t0 = std::chrono::steady_clock::now();
  RF_CUDA(ctx, cudaSetDevice(ctx->device));
  const int n_streams = std::max(1, std::min(ctx->multi_streams, n_plans));
  while (int(ctx->pool.size()) < n_streams) {
    cudaStream_t q = nullptr;
    RF_CUDA(ctx, cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
    ctx->pool.push_back(q);
  }
  // Packing: plans in decreasing estimated cost (energies x n^3, the LU's
  // work), each onto the stream with the least cost so far (longest
  // processing time first), so that the streams finish together; every plan's
  // work is put in flight before any is completed.
  std::vector<int> order(static_cast<size_t>(n_plans));
  std::vector<double> cost(static_cast<size_t>(n_plans));
  for (int i = 0; i < n_plans; ++i) {
    order[size_t(i)] = i;
    const double n = double(plans[i]->n);
    cost[size_t(i)] = double(std::max(points[i].n_energies, 0)) * n * n * n;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[size_t(a)] > cost[size_t(b)]; });
  std::vector<double> load(static_cast<size_t>(n_streams), 0.0);
  std::vector<int> stream_of(static_cast<size_t>(n_plans), 0);
  for (int i : order) {
    const int q = int(std::min_element(load.begin(), load.end()) - load.begin());
    stream_of[size_t(i)] = q;
    load[size_t(q)] += cost[size_t(i)];
  }
  // Batch sizes are fixed here so that a repeated call has the same launch structure.
  const bool fp32 = form != REFEFF_FMS_FORM_FP64_LU;
  std::vector<int> batch_of(static_cast<size_t>(n_plans), 0);
  bool graphable = ctx->multi_graph && form != REFEFF_FMS_FORM_BICGSTAB;
  std::vector<long long> key{static_cast<long long>(form), static_cast<long long>(n_streams)};
  for (int i : order) {
    const int E = points[i].n_energies;
    if (E > 0) batch_of[size_t(i)] = pick_batch(*plans[i], E, fp32);
    if (plans[i]->profiling) graphable = false;
    key.push_back(static_cast<long long>(reinterpret_cast<intptr_t>(plans[i])));
    key.push_back(E);
    key.push_back(batch_of[size_t(i)]);
  }
  cudaStream_t s0 = ctx->stream;
  int rc = REFEFF_FMS_OK;
  int begun = 0;
  const bool replay = graphable && ctx->mg_exec && ctx->mg_key == key &&
                      ctx->mg_epoch == g_state_epoch.load(std::memory_order_relaxed);
  // capture only a repeat of the last call with nothing moved since (so the capture allocates nothing)
  const bool capture = graphable && !replay && ctx->mg_seen == key &&
                       ctx->mg_seen_epoch == g_state_epoch.load(std::memory_order_relaxed);
  bool on_s0 = false;  // the device work runs on s0 (as the graph) rather than on the pool
  if (replay || capture) {
    // the uploads of every plan on s0, then the device work of all plans as one graph
    for (; begun < n_plans && rc == REFEFF_FMS_OK; ++begun) {
      const int i = order[size_t(begun)];
      rc = spectrum_prepare(*plans[i], &points[i], form, scattering_out[i], s0);
    }
    if (rc == REFEFF_FMS_OK && capture) {
      if (!ctx->fork_ev) RF_CUDA(ctx, cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming));
      while (int(ctx->pool_join.size()) < n_streams) {
        cudaEvent_t ev = nullptr;
        RF_CUDA(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        ctx->pool_join.push_back(ev);
      }
      if (ctx->mg_exec) {
        cudaGraphExecDestroy(ctx->mg_exec);
        ctx->mg_exec = nullptr;
      }
      const unsigned long long epoch = g_state_epoch.load(std::memory_order_relaxed);
      bool ok = cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      const unsigned long long before = g_launches.load();
      if (ok) {
        // fork the pool into the capture, put every plan's batches on its stream, join back
        ok = cudaEventRecord(ctx->fork_ev, s0) == cudaSuccess;
        for (int q = 0; q < n_streams && ok; ++q) ok = cudaStreamWaitEvent(ctx->pool[size_t(q)], ctx->fork_ev, 0) == cudaSuccess;
        for (int j = 0; j < n_plans && ok; ++j) {
          const int i = order[size_t(j)];
          refeff_fms_plan& p = *plans[i];
          if (points[i].n_energies == 0) continue;
          ok = solve_device_energies_enqueue(p, points[i].n_energies, p.d_k_all.p, p.d_x_all.p, form, p.d_gg_all.p,
                                             p.d_status_all.p, ctx->pool[size_t(stream_of[size_t(i)])], false,
                                             batch_of[size_t(i)], true) == REFEFF_FMS_OK;
        }
        for (int q = 0; q < n_streams; ++q) {  // join every forked stream, also after a failure
          cudaEventRecord(ctx->pool_join[size_t(q)], ctx->pool[size_t(q)]);
          cudaStreamWaitEvent(s0, ctx->pool_join[size_t(q)], 0);
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(s0, &g);
        ok = ok && ec == cudaSuccess && g != nullptr;
        cudaGraphExec_t ge = nullptr;
        if (ok) ok = cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
        if (g) cudaGraphDestroy(g);
        // no buffer may have moved while capturing (an allocation inside the capture fails it anyway)
        if (ok && g_state_epoch.load(std::memory_order_relaxed) == epoch) {
          ctx->mg_exec = ge;
          ctx->mg_key = key;
          ctx->mg_epoch = epoch;
          ctx->mg_launches = g_launches.load() - before;
          ++ctx->mg_captures;
        } else if (ge) {
          cudaGraphExecDestroy(ge);
        }
      }
      cudaGetLastError();  // a failed capture leaves no device work and no sticky error
      g_launches.fetch_sub(g_launches.load() - before);  // captured launches count when they run
      ctx->last_error.clear();
    }
    if (rc == REFEFF_FMS_OK && ctx->mg_exec && ctx->mg_key == key) {
      RF_CUDA(ctx, cudaGraphLaunch(ctx->mg_exec, s0));
      g_launches.fetch_add(ctx->mg_launches, std::memory_order_relaxed);
      if (replay) ++ctx->mg_replays;
      on_s0 = true;
    } else if (rc == REFEFF_FMS_OK) {
      // the capture did not take: the same batches one launch sequence per plan, on the pool after the uploads
      RF_CUDA(ctx, cudaEventRecord(ctx->fork_ev, s0));
      for (int q = 0; q < n_streams; ++q) RF_CUDA(ctx, cudaStreamWaitEvent(ctx->pool[size_t(q)], ctx->fork_ev, 0));
      for (int j = 0; j < n_plans && rc == REFEFF_FMS_OK; ++j) {
        const int i = order[size_t(j)];
        refeff_fms_plan& p = *plans[i];
        if (points[i].n_energies == 0) continue;
        rc = solve_device_energies_enqueue(p, points[i].n_energies, p.d_k_all.p, p.d_x_all.p, form, p.d_gg_all.p,
                                           p.d_status_all.p, ctx->pool[size_t(stream_of[size_t(i)])], false,
                                           batch_of[size_t(i)]);
      }
      ctx->mg_seen.clear();
    }
  } else {
    ctx->mg_seen.clear();
    for (; begun < n_plans && rc == REFEFF_FMS_OK; ++begun) {
      const int i = order[size_t(begun)];
      // the many-cluster call already overlaps clusters on its stream pool: one stream per plan
      rc = spectrum_begin(*plans[i], &points[i], form, scattering_out[i], ctx->pool[size_t(stream_of[size_t(i)])],
                          false, batch_of[size_t(i)]);
    }
  }
  int failed = 0, first_rc = rc;
  std::vector<refeff_fms_plan*> done_plans;
  for (int j = 0; j < begun; ++j) {
    const int i = order[size_t(j)];
    cudaStream_t q = on_s0 ? s0 : ctx->pool[size_t(stream_of[size_t(i)])];
    if (!on_s0 && (replay || capture)) RF_CUDA(ctx, cudaStreamSynchronize(s0));  // uploads were on s0
    int f = 0;
    const int r = rc == REFEFF_FMS_OK ? spectrum_end(*plans[i], &points[i], form, scattering_out[i],
                                                     status_out ? status_out[i] : nullptr, &f, q)
                                      : (cudaStreamSynchronize(q), REFEFF_FMS_OK);
    failed += f;
    if (first_rc == REFEFF_FMS_OK) first_rc = r;
    done_plans.push_back(plans[i]);
  }
  if (graphable && !on_s0 && first_rc == REFEFF_FMS_OK) {  // a repeat of this call is captured
    ctx->mg_seen = key;
    ctx->mg_seen_epoch = g_state_epoch.load(std::memory_order_relaxed);
  }
  fill_report(report, done_plans, form, failed, t0);
  return first_rc;
}

extern "C" int refeff_fms_context_graph_stats(const refeff_fms_context* ctx, long long* captures, long long* replays) {
  if (!ctx) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (captures) *captures = ctx->mg_captures;
  if (replays) *replays = ctx->mg_replays;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_refinement_stats(const refeff_fms_plan* plan, int n_energies, double* rel_residual,
                                                int* iterations, int* fp64_fallback) {
  if (!plan || n_energies < 0) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  const int have = int(plan->last_iters.size());
  for (int e = 0; e < n_energies; ++e) {
    if (rel_residual) rel_residual[e] = e < have ? plan->last_relres[size_t(e)] : 0.0;
    if (iterations) iterations[e] = e < have ? plan->last_iters[size_t(e)] : 0;
    if (fp64_fallback) fp64_fallback[e] = 0;
  }
  if (fp64_fallback)
    for (int e : plan->last_fallback)
      if (e < n_energies) fp64_fallback[e] = 1;
  return REFEFF_FMS_OK;
}

// ---------------------------------------------------------------------------
// BiCGSTAB form and its learned preconditioner
// ---------------------------------------------------------------------------
namespace {

int ensure_shell_tables(refeff_fms_plan& p, cudaStream_t s) {
  if (p.d_shell_info.p) return REFEFF_FMS_OK;
  const ShellTables t = shell_tables(p.N, p.npot, p.pos_dev.data(), p.pot_dev.data());
  RF_CUDA(p.ctx, p.d_shell_info.upload(t.info.data(), t.info.size(), s));
  RF_CUDA(p.ctx, p.d_shell_pots.upload(t.pots.data(), t.pots.size(), s));
  RF_CUDA(p.ctx, cudaStreamSynchronize(s));
  return REFEFF_FMS_OK;
}

// RHS columns of M64 <- unit vectors of states [s0, s0 + cnt), zero beyond.
__global__ void unit_rhs_kernel(BatchLayout lay, double2* M, int s0, int cnt) {
  const int b = blockIdx.y;
  double2* Mb = M + size_t(b) * lay.stride + size_t(lay.lda) * lay.n;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < lay.lda * lay.m; idx += gridDim.x * blockDim.x) {
    const int r = idx % lay.lda, c = idx / lay.lda;
    Mb[idx] = make_double2(c < cnt && r == s0 + c ? 1.0 : 0.0, 0.0);
  }
}

__global__ void inverse_diagonal_kernel(BatchLayout lay, const double2* M, int s0, int cnt, double2* out) {
  const int b = blockIdx.x, c = threadIdx.x;
  if (c >= cnt) return;
  out[size_t(b) * cnt + c] = M[size_t(b) * lay.stride + size_t(s0 + c) + size_t(lay.lda) * (lay.n + c)];
}

// out[(b cnt + r) cnt + c] = (A^-1)[s0 + r, s0 + c]: the solved unit columns, row-major per energy
__global__ void inverse_block_kernel(BatchLayout lay, const double2* M, int s0, int cnt, double2* out) {
  const int b = blockIdx.x;
  for (int idx = threadIdx.x; idx < cnt * cnt; idx += blockDim.x) {
    const int r = idx / cnt, c = idx % cnt;
    out[size_t(b) * cnt * cnt + idx] = M[size_t(b) * lay.stride + size_t(s0 + r) + size_t(lay.lda) * (lay.n + c)];
  }
}

}  // namespace

extern "C" int refeff_fms_plan_set_precond_window(refeff_fms_plan* plan, double e_lo_ev, double e_hi_ev) {
  if (!plan || std::isnan(e_lo_ev) || std::isnan(e_hi_ev) || e_lo_ev > e_hi_ev) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  plan->precond_e_lo = e_lo_ev;
  plan->precond_e_hi = e_hi_ev;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_set_bicgstab_window(refeff_fms_plan* plan, double e_lo_ev, double e_hi_ev) {
  if (!plan || std::isnan(e_lo_ev) || std::isnan(e_hi_ev) || e_lo_ev > e_hi_ev) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  plan->bicg_e_lo = e_lo_ev;
  plan->bicg_e_hi = e_hi_ev;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_bicgstab_lu_energies(const refeff_fms_plan* plan, int n_energies, int32_t* flags) {
  if (!plan || n_energies < 0 || (n_energies > 0 && !flags)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  for (int e = 0; e < n_energies; ++e) flags[e] = e < int(plan->bicg_lu.size()) ? plan->bicg_lu[size_t(e)] : 0;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_set_preconditioner(refeff_fms_plan* plan, refeff_fms_precond_model* model) {
  if (!plan) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (model && model_lmax(model) != plan->L)
    return fail(plan->ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "preconditioner model built for another lmax");
  if (model && model_kind(model) == kPrecondBlock && plan->nsp != 1)
    return fail(plan->ctx, REFEFF_FMS_ERR_UNSUPPORTED, "block-diagonal preconditioner needs one spin channel");
  RF_CUDA(plan->ctx, cudaSetDevice(plan->ctx->device));
  if (model) {
    const int rc = ensure_shell_tables(*plan, plan->ctx->stream);
    if (rc) return rc;
  }
  if (model && model_kind(model) == kPrecondBlock && !plan->d_state_atom.p) {
    // state -> device atom, for the per-atom block apply
    std::vector<int> sa(static_cast<size_t>(plan->n));
    for (int d = 0; d < plan->N; ++d)
      for (int st = plan->off_dev[size_t(d)]; st < plan->off_dev[size_t(d) + 1]; ++st) sa[size_t(st)] = d;
    RF_CUDA(plan->ctx, plan->d_state_atom.upload(sa.data(), sa.size(), plan->ctx->stream));
    RF_CUDA(plan->ctx, cudaStreamSynchronize(plan->ctx->stream));
  }
  plan->model = model;
  plan->ws.precond_D.release();  // re-sized on the next BiCGSTAB call
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_set_bicgstab(refeff_fms_plan* plan, int max_iterations, double tolerance,
                                            int poll_interval) {
  if (!plan || max_iterations < 1 || !(tolerance > 0.0) || poll_interval < 1) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  plan->bicg_max_iter = max_iterations;
  plan->bicg_tol = tolerance;
  plan->bicg_poll = poll_interval;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_bicgstab_stats(const refeff_fms_plan* plan, int n_energies, int32_t* iterations) {
  if (!plan || n_energies < 0 || (n_energies > 0 && !iterations)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  for (int e = 0; e < n_energies; ++e)
    iterations[e] = e < int(plan->last_bicg_iters.size()) ? plan->last_bicg_iters[size_t(e)] : 0;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_plan_precond_features(refeff_fms_plan* plan, const refeff_fms_energy_points* points,
                                                float* features_out) {
  if (!plan || !points || points->n_energies < 0 || !features_out) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  refeff_fms_plan& p = *plan;
  const int E = points->n_energies;
  if (E == 0) return REFEFF_FMS_OK;
  RF_CUDA(p.ctx, cudaSetDevice(p.ctx->device));
  cudaStream_t s = p.ctx->stream;
  int rc = ensure_shell_tables(p, s);
  if (rc) return rc;
  const int F = feature_count(p.L);
  DevBuf<double2> dk, dx;
  DevBuf<float> dX;
  RF_CUDA(p.ctx, dk.upload(reinterpret_cast<const double2*>(points->wave_numbers), size_t(E) * p.nsp, s));
  RF_CUDA(p.ctx, dx.upload(reinterpret_cast<const double2*>(points->phase_shifts), size_t(E) * p.xph_per_energy(), s));
  RF_CUDA(p.ctx, dX.alloc(size_t(E) * p.N * F));
  launch_features(E, p.N, p.L, p.nsp, p.npot, dk.p, dx.p, p.d_atom_pot.p, p.d_shell_info.p, p.d_shell_pots.p, dX.p, s);
  RF_CUDA(p.ctx, cudaGetLastError());
  RF_CUDA(p.ctx, cudaMemcpyAsync(features_out, dX.p, size_t(E) * p.N * F * sizeof(float), cudaMemcpyDeviceToHost, s));
  RF_CUDA(p.ctx, cudaStreamSynchronize(s));
  return REFEFF_FMS_OK;
}

namespace {

// Columns s0..s0+cnt of A^-1 for the states of one atom, solved in FP64 per energy batch; the diagonal or the
// whole cnt x cnt block of the atom is copied out.
int inverse_columns(refeff_fms_plan* plan, const refeff_fms_energy_points* points, int atom, bool whole_block,
                    refeff_complex128* out_host, int32_t* status_out) {
  if (!plan || !points || points->n_energies < 0 || !out_host) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  refeff_fms_plan& p = *plan;
  refeff_fms_context* ctx = p.ctx;
  if (atom < 0 || atom >= p.N) return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "atom index outside the cluster");
  const int d = atom == 0 ? p.N - 1 : atom - 1;  // device order: absorber last
  const int s0 = p.off_dev[size_t(d)], cnt = p.off_dev[size_t(d) + 1] - s0;
  if (cnt > p.m) return fail(ctx, REFEFF_FMS_ERR_UNSUPPORTED, "atom has more states than the absorber block");
  const int E = points->n_energies;
  if (E == 0) return REFEFF_FMS_OK;
  RF_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const int B = pick_batch(p, E, false);
  int rc = ensure_workspace(ctx, p.ws, p.n, p.m, B, false, &p.tune);
  if (rc) return rc;
  Workspace& ws = p.ws;
  const BatchLayout& lay = ws.lay;
  const size_t xph = p.xph_per_energy();
  RF_CUDA(ctx, ws.k_stage.alloc(size_t(ws.batch) * p.nsp));
  RF_CUDA(ctx, ws.x_stage.alloc(size_t(ws.batch) * xph));
  const size_t per = whole_block ? size_t(cnt) * cnt : size_t(cnt);
  DevBuf<double2> dout;
  RF_CUDA(ctx, dout.alloc(size_t(ws.batch) * per));
  std::vector<int> st(static_cast<size_t>(ws.batch));
  for (int e0 = 0; e0 < E; e0 += B) {
    const int nb = std::min(B, E - e0);
    RF_CUDA(ctx, cudaMemcpyAsync(ws.k_stage.p, reinterpret_cast<const double2*>(points->wave_numbers) + size_t(e0) * p.nsp,
                                 size_t(nb) * p.nsp * sizeof(double2), cudaMemcpyHostToDevice, s));
    RF_CUDA(ctx, cudaMemcpyAsync(ws.x_stage.p, reinterpret_cast<const double2*>(points->phase_shifts) + size_t(e0) * xph,
                                 size_t(nb) * xph * sizeof(double2), cudaMemcpyHostToDevice, s));
    RF_CUDA(ctx, cudaMemsetAsync(ws.status.p, 0, size_t(nb) * sizeof(int), s));
    RF_CUDA(ctx, cudaMemsetAsync(ws.info.p, 0, size_t(nb) * sizeof(int), s));
    launch_build_system(p.P, nb, ws.k_stage.p, ws.x_stage.p, lay, ws.M64.p, nullptr, ws.status.p, s);
    count_launch();
    unit_rhs_kernel<<<dim3(64, unsigned(nb)), 256, 0, s>>>(lay, ws.M64.p, s0, cnt);
    RF_CUDA(ctx, lu_eliminate<double>(ws.pc64, lay, nb, ws.M64.p, lu_work(ws, ws.pc64), s));
    lu_backward_rhs<double>(ws.pc64, lay, nb, ws.M64.p, nullptr, s);
    count_launch();
    if (whole_block)
      inverse_block_kernel<<<unsigned(nb), 256, 0, s>>>(lay, ws.M64.p, s0, cnt, dout.p);
    else
      inverse_diagonal_kernel<<<unsigned(nb), 64, 0, s>>>(lay, ws.M64.p, s0, cnt, dout.p);
    RF_CUDA(ctx, cudaGetLastError());
    RF_CUDA(ctx, cudaMemcpyAsync(out_host + size_t(e0) * per, dout.p, size_t(nb) * per * sizeof(double2),
                                 cudaMemcpyDeviceToHost, s));
    RF_CUDA(ctx, cudaMemcpyAsync(st.data(), ws.status.p, size_t(nb) * sizeof(int), cudaMemcpyDeviceToHost, s));
    RF_CUDA(ctx, cudaStreamSynchronize(s));
    for (int i = 0; i < nb; ++i)
      if (status_out) status_out[e0 + i] = map_status(st[size_t(i)]);
  }
  return REFEFF_FMS_OK;
}

}  // namespace

extern "C" int refeff_fms_plan_inverse_diagonal(refeff_fms_plan* plan, const refeff_fms_energy_points* points, int atom,
                                                refeff_complex128* diag_out, int32_t* status_out) {
  return inverse_columns(plan, points, atom, false, diag_out, status_out);
}

extern "C" int refeff_fms_plan_inverse_block(refeff_fms_plan* plan, const refeff_fms_energy_points* points, int atom,
                                             refeff_complex128* block_out, int32_t* status_out) {
  return inverse_columns(plan, points, atom, true, block_out, status_out);
}

extern "C" int refeff_fms_gg_section(const refeff_fms_plan* plan, const refeff_complex128* scattering, int nspu,
                                     refeff_complex128* out) {
  if (!plan || !scattering || !out || nspu < plan->nsp) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  const int ang = (plan->abs_lmax + 1) * (plan->abs_lmax + 1);
  const int active = ang * plan->nsp, outc = ang * nspu;
  const size_t C = size_t(plan->C);
  for (int i = 0; i < outc * outc; ++i) out[i] = {0.0, 0.0};
  for (int c = 0; c < active; ++c)
    for (int r = 0; r < active; ++r)
      out[size_t(r) + size_t(outc) * c] = scattering[size_t(r) + C * (size_t(c) + C * size_t(plan->abs_pot))];
  return REFEFF_FMS_OK;
}

// ---------------------------------------------------------------------------
// dense batched solve
// ---------------------------------------------------------------------------
namespace {

// [A | B] already in M64 (every system of the batch): solve and leave X in
// ws.X64 (n x m per system, leading dimension lay.lda), statuses in ws.status
// and first zero pivots in ws.info.  Asynchronous on stream s.
int dense_solve_device(refeff_fms_context* ctx, Workspace& ws, int batch, bool fp32, cudaStream_t s) {
  const BatchLayout& lay = ws.lay;
  RF_CUDA(ctx, cudaMemsetAsync(ws.status.p, 0, size_t(batch) * sizeof(int), s));
  RF_CUDA(ctx, cudaMemsetAsync(ws.info.p, 0, size_t(batch) * sizeof(int), s));
  if (!fp32) {
    cudaError_t e = lu_eliminate<double>(ws.pc64, lay, batch, ws.M64.p, lu_work(ws, ws.pc64), s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "lu_eliminate<double>");
    lu_backward_rhs<double>(ws.pc64, lay, batch, ws.M64.p, nullptr, s);
    RF_CUDA(ctx, ws.X64.alloc(size_t(ws.batch) * lay.lda * lay.m));
    launch_copy_rhs64(lay, batch, ws.M64.p, ws.X64.p, s);
  } else {
    launch_split_system(lay, batch, ws.M64.p, ws.M32.p, s);
    cudaError_t e = lu_eliminate<float>(ws.pc32, lay, batch, ws.M32.p, lu_work(ws, ws.pc32), s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "lu_eliminate<float>");
    // M32's RHS columns hold Y32; refinement uses the hi/lo split system in M64
    e = refine_fp32(ws, batch, ctx->dense_refinement, 1.0e-10, s);  // 0 corrections: the FP32 LU solution
    if (e != cudaSuccess) return cuda_fail(ctx, e, "refine");
    count_launch();
    status_not_converged_kernel<<<(batch + 127) / 128, 128, 0, s>>>(batch, ws.converged.p, ws.status.p);
  }
  RF_CUDA(ctx, cudaGetLastError());
  return REFEFF_FMS_OK;
}

}  // namespace

namespace {

// KKR system of each k-point in place (fms reciprocal solve_k_point,
// crates/refeff-core/src/fms/reciprocal.rs:103-134): with G(k) in the right-hand
// side columns of [A | B], A = I - G(k) T, T given by its non-zero entries per
// column (tcol_ptr / tcol_row / tcol_val, rows ascending as the reference
// subtracts them).
__global__ void kkr_system_kernel(BatchLayout lay, double2* __restrict__ M, const int* __restrict__ tcol_ptr,
                                  const int* __restrict__ tcol_row, const double2* __restrict__ tcol_val) {
  const int b = blockIdx.z, c = blockIdx.y, n = lay.n;
  double2* Mb = M + size_t(b) * lay.stride;
  const double2* G = Mb + size_t(lay.lda) * n;  // G(k) = B
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    double2 a = make_double2(r == c ? 1.0 : 0.0, 0.0);
    for (int q = tcol_ptr[c]; q < tcol_ptr[c + 1]; ++q) a = csub(a, cmul(G[size_t(r) + size_t(lay.lda) * tcol_row[q]], tcol_val[q]));
    Mb[size_t(r) + size_t(lay.lda) * c] = a;
  }
}

// acc[r + n c] += sum over the batch (in k-point order) of w_b X_b[r, c] (FmsReciprocalAccumulator::push, reciprocal.rs:172-200).
__global__ void kkr_accumulate_kernel(BatchLayout lay, int batch, const double2* __restrict__ X, const double* __restrict__ w,
                                      double2* __restrict__ acc) {
  const int n = lay.n;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n * n; idx += gridDim.x * blockDim.x) {
    const int r = idx % n, c = idx / n;
    double2 s = acc[idx];
    for (int b = 0; b < batch; ++b) {
      const double2 x = X[size_t(b) * lay.lda * lay.m + size_t(r) + size_t(lay.lda) * c];
      s.x = fma(w[b], x.x, s.x);
      s.y = fma(w[b], x.y, s.y);
    }
    acc[idx] = s;
  }
}

}  // namespace

extern "C" int refeff_fms_reciprocal_integrate(refeff_fms_context* ctx, int order, int n_kpoints,
                                               const refeff_complex128* structure_factors, const double* weights,
                                               const refeff_complex128* t_matrix, refeff_fms_form form,
                                               refeff_complex128* green_out, int32_t* status_out) {
  if (!ctx || !structure_factors || !weights || !t_matrix || !green_out) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  ctx->last_error.clear();
  if (order <= 0) return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "reciprocal FMS needs a nonempty square matrix");
  if (n_kpoints <= 0) return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "reciprocal FMS requires at least one k-point");
  if (form != REFEFF_FMS_FORM_FP64_LU && form != REFEFF_FMS_FORM_FP32_REFINED)
    return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "unknown form");
  const bool fp32 = form == REFEFF_FMS_FORM_FP32_REFINED;
  if (fp32 && order > 64)
    return fail(ctx, REFEFF_FMS_ERR_UNSUPPORTED, "the refined form solves at most 64 right-hand sides; use the FP64 LU");
  const size_t nn = size_t(order) * order;
  double total = 0.0;
  for (int q = 0; q < n_kpoints; ++q) {
    if (!std::isfinite(weights[q]) || !(weights[q] > 0.0))
      return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "reciprocal FMS k-point weight must be positive and finite");
    total += weights[q];
  }
  if (!std::isfinite(total) || !(total > 0.0))
    return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "reciprocal FMS total k-point weight must be positive and finite");
  for (size_t i = 0; i < nn * size_t(n_kpoints); ++i)
    if (!std::isfinite(structure_factors[i].re) || !std::isfinite(structure_factors[i].im))
      return fail(ctx, REFEFF_FMS_ERR_NONFINITE_INPUT, "non-finite structure factor");
  // the lattice T by columns, non-zero entries only (FmsReciprocalPlan::new, reciprocal.rs:80-97)
  std::vector<int> ptr(static_cast<size_t>(order) + 1, 0), rows;
  std::vector<double2> vals;
  for (int c = 0; c < order; ++c) {
    for (int r = 0; r < order; ++r) {
      const refeff_complex128 v = t_matrix[size_t(r) + size_t(order) * c];
      if (!std::isfinite(v.re) || !std::isfinite(v.im)) return fail(ctx, REFEFF_FMS_ERR_NONFINITE_INPUT, "non-finite T");
      if (v.re != 0.0 || v.im != 0.0) {
        rows.push_back(r);
        vals.push_back(make_double2(v.re, v.im));
      }
    }
    ptr[size_t(c) + 1] = int(rows.size());
  }
  if (rows.empty()) {  // the reference's empty column lists: A = I
    rows.push_back(0);
    vals.push_back(make_double2(0.0, 0.0));
  }
  RF_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  Workspace ws;
  const BatchLayout lay0 = make_layout(order, order);
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const size_t per = bytes_per_system(lay0, fp32) + size_t(lay0.lda) * order * sizeof(double2);
  const int B = int(std::max<size_t>(1, std::min<size_t>(size_t(n_kpoints), std::min<size_t>(256, free_b / 2 / per))));
  int rc = ensure_workspace(ctx, ws, order, order, B, fp32);
  if (rc) return rc;
  const BatchLayout& lay = ws.lay;
  DevBuf<int> d_ptr, d_rows;
  DevBuf<double2> d_vals, d_acc;
  DevBuf<double> d_w;
  RF_CUDA(ctx, d_ptr.upload(ptr.data(), ptr.size(), s));
  RF_CUDA(ctx, d_rows.upload(rows.data(), rows.size(), s));
  RF_CUDA(ctx, d_vals.upload(vals.data(), vals.size(), s));
  RF_CUDA(ctx, d_w.upload(weights, size_t(n_kpoints), s));
  RF_CUDA(ctx, d_acc.alloc(nn));
  RF_CUDA(ctx, cudaMemsetAsync(d_acc.p, 0, nn * sizeof(double2), s));
  std::vector<int> st(static_cast<size_t>(n_kpoints));
  for (int k0 = 0; k0 < n_kpoints; k0 += B) {
    const int nb = std::min(B, n_kpoints - k0);
    RF_CUDA(ctx, cudaMemsetAsync(ws.M64.p, 0, size_t(nb) * lay.stride * sizeof(double2), s));
    for (int b = 0; b < nb; ++b)
      RF_CUDA(ctx, cudaMemcpy2DAsync(ws.M64.p + size_t(b) * lay.stride + size_t(lay.lda) * order,
                                     size_t(lay.lda) * sizeof(double2), structure_factors + size_t(k0 + b) * nn,
                                     size_t(order) * sizeof(double2), size_t(order) * sizeof(double2), size_t(order),
                                     cudaMemcpyHostToDevice, s));
    count_launch();
    kkr_system_kernel<<<dim3(unsigned((order + 127) / 128), unsigned(order), unsigned(nb)), 128, 0, s>>>(
        lay, ws.M64.p, d_ptr.p, d_rows.p, d_vals.p);
    rc = dense_solve_device(ctx, ws, nb, fp32, s);
    if (rc) return rc;
    count_launch();
    kkr_accumulate_kernel<<<unsigned(std::min<size_t>(1024, (nn + 255) / 256)), 256, 0, s>>>(lay, nb, ws.X64.p,
                                                                                            d_w.p + k0, d_acc.p);
    RF_CUDA(ctx, cudaMemcpyAsync(st.data() + k0, ws.status.p, size_t(nb) * sizeof(int), cudaMemcpyDeviceToHost, s));
  }
  std::vector<double2> acc(nn);
  RF_CUDA(ctx, cudaMemcpyAsync(acc.data(), d_acc.p, nn * sizeof(double2), cudaMemcpyDeviceToHost, s));
  int tc_timeout = 0;
  if (ws.use_tc) RF_CUDA(ctx, cudaMemcpyAsync(&tc_timeout, ws.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  RF_CUDA(ctx, cudaStreamSynchronize(s));
  if (tc_timeout) return fail(ctx, REFEFF_FMS_ERR_CUDA, "tensor-core update timed out");
  int first_bad = -1;
  for (int q = 0; q < n_kpoints; ++q) {
    const int code = map_status(st[size_t(q)]);
    if (status_out) status_out[q] = code;
    if (code != REFEFF_FMS_OK && first_bad < 0) first_bad = q;
  }
  if (first_bad >= 0)
    return fail(ctx, map_status(st[size_t(first_bad)]),
                "reciprocal KKR solve failed at k-point " + std::to_string(first_bad + 1));
  // FmsReciprocalAccumulator::finish (reciprocal.rs:203-222)
  for (size_t i = 0; i < nn; ++i) {
    green_out[i] = {acc[i].x / total, acc[i].y / total};
    if (!std::isfinite(green_out[i].re) || !std::isfinite(green_out[i].im))
      return fail(ctx, REFEFF_FMS_ERR_NONFINITE_INPUT, "non-finite integrated Green matrix");
  }
  return REFEFF_FMS_OK;
}

namespace {

// In-place partial-pivot LU solve of the small dense system A X = B (n x n,
// n x m, column-major, FP64); false when a pivot is zero.
bool small_lu_solve(int n, int m, std::vector<std::complex<double>>& A, std::vector<std::complex<double>>& B) {
  using cd = std::complex<double>;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::abs(A[size_t(k) + size_t(n) * k].real()) + std::abs(A[size_t(k) + size_t(n) * k].imag());
    for (int r = k + 1; r < n; ++r) {
      const cd v = A[size_t(r) + size_t(n) * k];
      const double a = std::abs(v.real()) + std::abs(v.imag());
      if (a > best) { best = a; p = r; }
    }
    if (!(best > 0.0)) return false;
    if (p != k) {
      for (int c = 0; c < n; ++c) std::swap(A[size_t(k) + size_t(n) * c], A[size_t(p) + size_t(n) * c]);
      for (int c = 0; c < m; ++c) std::swap(B[size_t(k) + size_t(n) * c], B[size_t(p) + size_t(n) * c]);
    }
    const cd piv = A[size_t(k) + size_t(n) * k];
    for (int r = k + 1; r < n; ++r) {
      const cd l = A[size_t(r) + size_t(n) * k] / piv;
      A[size_t(r) + size_t(n) * k] = l;
      for (int c = k + 1; c < n; ++c) A[size_t(r) + size_t(n) * c] -= l * A[size_t(k) + size_t(n) * c];
      for (int c = 0; c < m; ++c) B[size_t(r) + size_t(n) * c] -= l * B[size_t(k) + size_t(n) * c];
    }
  }
  for (int c = 0; c < m; ++c)
    for (int r = n - 1; r >= 0; --r) {
      cd v = B[size_t(r) + size_t(n) * c];
      for (int q = r + 1; q < n; ++q) v -= A[size_t(r) + size_t(n) * q] * B[size_t(q) + size_t(n) * c];
      B[size_t(r) + size_t(n) * c] = v / A[size_t(r) + size_t(n) * r];
    }
  return true;
}

}  // namespace

extern "C" int refeff_fms_reciprocal_core_hole(int order, const refeff_complex128* green, int absorber_offset, int block,
                                               const refeff_complex128* t_difference, refeff_complex128* out) {
  using cd = std::complex<double>;
  if (order <= 0 || !green || !t_difference || !out || absorber_offset < 0) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (block <= 0 || absorber_offset + block > order) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  const size_t n = size_t(order), b = size_t(block), a = size_t(absorber_offset);
  auto G = [&](size_t r, size_t c) { return cd(green[r + n * c].re, green[r + n * c].im); };
  for (size_t i = 0; i < n * n; ++i)
    if (!std::isfinite(green[i].re) || !std::isfinite(green[i].im)) return REFEFF_FMS_ERR_NONFINITE_INPUT;
  std::vector<cd> C(b * b), dyson(b * b), eff(b * b);
  for (size_t i = 0; i < b * b; ++i) {
    C[i] = cd(t_difference[i].re, t_difference[i].im);
    if (!std::isfinite(C[i].real()) || !std::isfinite(C[i].imag())) return REFEFF_FMS_ERR_NONFINITE_INPUT;
  }
  // dyson = I + C G_aa; effective T = dyson^-1 C (fms_reciprocal_apply_core_hole, reciprocal.rs:268-275)
  for (size_t c = 0; c < b; ++c)
    for (size_t r = 0; r < b; ++r) {
      cd v = r == c ? cd(1.0, 0.0) : cd(0.0, 0.0);
      for (size_t q = 0; q < b; ++q) v += C[r + b * q] * G(a + q, a + c);
      dyson[r + b * c] = v;
    }
  eff = C;
  if (!small_lu_solve(block, block, dyson, eff)) return REFEFF_FMS_ERR_SINGULAR_MATRIX;
  // G - G[:, a] eff G[a, :] (reciprocal.rs:277-301)
  std::vector<cd> left(n * b);
  for (size_t c = 0; c < b; ++c)
    for (size_t r = 0; r < n; ++r) {
      cd v(0.0, 0.0);
      for (size_t q = 0; q < b; ++q) v += G(r, a + q) * eff[q + b * c];
      left[r + n * c] = v;
    }
  for (size_t c = 0; c < n; ++c)
    for (size_t r = 0; r < n; ++r) {
      cd v = G(r, c);
      for (size_t q = 0; q < b; ++q) v -= left[r + n * q] * G(a + q, c);
      if (!std::isfinite(v.real()) || !std::isfinite(v.imag())) return REFEFF_FMS_ERR_NONFINITE_INPUT;
      out[r + n * c] = {v.real(), v.imag()};
    }
  return REFEFF_FMS_OK;
}

extern "C" int refeff_complex_lu_solve_batched(refeff_fms_context* ctx, int n, int m, int batch,
                                               const refeff_complex128* A, const refeff_complex128* B,
                                               refeff_complex128* X, refeff_fms_form form, int32_t* status_out,
                                               int32_t* pivot_out) {
  if (!ctx || n <= 0 || m <= 0 || m > 64 || batch <= 0 || !A || !B || !X) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (form != REFEFF_FMS_FORM_FP64_LU && form != REFEFF_FMS_FORM_FP32_REFINED)
    return fail(ctx, REFEFF_FMS_ERR_INVALID_ARGUMENT, "unknown form");
  ctx->last_error.clear();
  RF_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const bool fp32 = form == REFEFF_FMS_FORM_FP32_REFINED;
  Workspace ws;
  int rc = ensure_workspace(ctx, ws, n, m, batch, fp32);
  if (rc) return rc;
  const BatchLayout& lay = ws.lay;
  RF_CUDA(ctx, cudaMemsetAsync(ws.M64.p, 0, size_t(batch) * lay.stride * sizeof(double2), s));
  for (int b = 0; b < batch; ++b) {
    RF_CUDA(ctx, cudaMemcpy2DAsync(ws.M64.p + size_t(b) * lay.stride, size_t(lay.lda) * sizeof(double2),
                                   A + size_t(b) * n * n, size_t(n) * sizeof(double2), size_t(n) * sizeof(double2), size_t(n),
                                   cudaMemcpyHostToDevice, s));
    RF_CUDA(ctx, cudaMemcpy2DAsync(ws.M64.p + size_t(b) * lay.stride + size_t(lay.lda) * n,
                                   size_t(lay.lda) * sizeof(double2), B + size_t(b) * n * m, size_t(n) * sizeof(double2),
                                   size_t(n) * sizeof(double2), size_t(m), cudaMemcpyHostToDevice, s));
  }
  rc = dense_solve_device(ctx, ws, batch, fp32, s);
  if (rc) return rc;
  for (int b = 0; b < batch; ++b)
    RF_CUDA(ctx, cudaMemcpy2DAsync(X + size_t(b) * n * m, size_t(n) * sizeof(double2), ws.X64.p + size_t(b) * lay.lda * m,
                                   size_t(lay.lda) * sizeof(double2), size_t(n) * sizeof(double2), size_t(m),
                                   cudaMemcpyDeviceToHost, s));
  std::vector<int> st(static_cast<size_t>(batch)), info(static_cast<size_t>(batch));
  RF_CUDA(ctx, cudaMemcpyAsync(st.data(), ws.status.p, st.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  RF_CUDA(ctx, cudaMemcpyAsync(info.data(), ws.info.p, info.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
  int tc_timeout = 0;
  if (ws.use_tc) RF_CUDA(ctx, cudaMemcpyAsync(&tc_timeout, ws.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  RF_CUDA(ctx, cudaStreamSynchronize(s));
  if (tc_timeout) return fail(ctx, REFEFF_FMS_ERR_CUDA, "tensor-core update timed out");
  int first_bad = REFEFF_FMS_OK;
  for (int b = 0; b < batch; ++b) {
    const int code = map_status(st[size_t(b)]);
    if (status_out) status_out[b] = code;
    if (pivot_out) pivot_out[b] = info[size_t(b)];
    if (code != REFEFF_FMS_OK && first_bad == REFEFF_FMS_OK) first_bad = code;
  }
  if (first_bad != REFEFF_FMS_OK) return fail(ctx, first_bad, "batched solve: at least one system failed");
  return REFEFF_FMS_OK;
}
