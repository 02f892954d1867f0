// FMS system assembly on the GPU: pair geometry (once per cluster) and the
// fused G0 / T / (I - G0 T) build (once per energy batch).
//
// Reference arithmetic followed here:
//   getang            crates/refeff-core/src/fms/cluster.rs:201-241
//   rotxan small-d    crates/refeff-core/src/fms/internals/rotation.rs:3-125
//   xclmz polynomials crates/refeff-core/src/fms/polynomial.rs:8-83
//   xgllm             crates/refeff-core/src/fms/xgllm.rs:9-57
//   G0 element        crates/refeff-core/src/fms/pairs.rs:242-323, 413-460
//   prefactor         crates/refeff-core/src/fms/internals/geometry.rs:14-28
//   T table           crates/refeff-core/src/fms/t_matrix.rs:10-190
//   A = I - G0 T      crates/refeff-core/src/fms/internals/linear.rs:102-135
// All of it is evaluated in FP64.  Rotation tables depend only on geometry,
// so they are computed once per plan and stay resident in HBM; the Hankel
// polynomial and the propagator prefactor depend on the energy and are
// recomputed per (pair, energy) inside the build kernel, next to the store.
#include "cplx.cuh"
#include "fms_plan.cuh"

namespace rfx {

__host__ __device__ constexpr int dsmall_per_dir(int L) { return (L + 1) * (2 * L + 1) * (2 * L + 3) / 3; }
__device__ __forceinline__ int lblock_offset(int l) { return l * (2 * l - 1) * (2 * l + 1) / 3; }

// ---------------------------------------------------------------------------
// Pair geometry: one thread per ordered pair (i, j), i != j, device order.
// The small-d recursion keeps two levels in registers/local memory.
// ---------------------------------------------------------------------------
template <int L>
__device__ void rotxan_small_d(double beta, double* out /* dsmall_per_dir(L) */) {
  constexpr int D0 = 2 * L + 3;  // indices 1..2L+1 used
  double bufa[D0 * D0], bufb[D0 * D0];
  double* prev = bufa;
  double* cur = bufb;
  auto at = [](double* b, int n, int m) -> double& { return b[n + D0 * m]; };
  const int ndm = 2 * L + 1;  // lxp1 + mxp1 - 1 with mmax = lmax
  const double xc = cos(beta / 2.0), xs = sin(beta / 2.0), s = sin(beta);
  // level il = 1
  for (int q = 0; q < D0 * D0; ++q) cur[q] = 0.0;
  at(cur, 1, 1) = 1.0;
  out[0] = 1.0;
  if (L >= 1) {
    double* t = prev; prev = cur; cur = t;
    for (int q = 0; q < D0 * D0; ++q) cur[q] = 0.0;
    at(cur, 1, 1) = xc * xc;
    at(cur, 1, 2) = s / sqrt(2.0);
    at(cur, 1, 3) = xs * xs;
    at(cur, 2, 1) = -at(cur, 1, 2);
    at(cur, 2, 2) = cos(beta);
    at(cur, 2, 3) = at(cur, 1, 2);
    at(cur, 3, 1) = at(cur, 1, 3);
    at(cur, 3, 2) = -at(cur, 2, 3);
    at(cur, 3, 3) = at(cur, 1, 1);
    // drix(m2, m1, l=1) = dri0(2, m1+2, m2+2) stored at [(m2+1)*3 + (m1+1)]
    for (int m2 = -1; m2 <= 1; ++m2)
      for (int m1 = -1; m1 <= 1; ++m1) out[1 + (m2 + 1) * 3 + (m1 + 1)] = at(cur, m1 + 2, m2 + 2);
  }
  for (int l = 3; l <= L + 1; ++l) {
    double* t = prev; prev = cur; cur = t;
    for (int q = 0; q < D0 * D0; ++q) cur[q] = 0.0;
    int ln = min(2 * l - 1, ndm), lm = min(2 * l - 3, ndm);
    for (int n = 1; n <= ln; ++n) {
      for (int m = 1; m <= lm; ++m) {
        double t1 = double((2 * l - 1 - n) * (2 * l - 2 - n));
        double tt = double((2 * l - 1 - m) * (2 * l - 2 - m));
        double f1 = sqrt(t1 / tt);
        double f2 = sqrt(double((2 * l - 1 - n) * (n - 1)) / tt);
        double f3 = sqrt(double((n - 2) * (n - 1)) / tt);
        double dlnm = f1 * xc * xc * at(prev, n, m);
        if (n > 1) dlnm -= f2 * s * at(prev, n - 1, m);
        if (n > 2) dlnm += f3 * xs * xs * at(prev, n - 2, m);
        at(cur, n, m) = dlnm;
        if (n > 2 * l - 3) at(cur, m, n) = (((n - m) & 1) == 0 ? 1.0 : -1.0) * dlnm;
      }
      if (n > 2 * l - 3) {
        at(cur, 2 * l - 2, 2 * l - 2) = at(cur, 2, 2);
        at(cur, 2 * l - 1, 2 * l - 2) = -at(cur, 1, 2);
        at(cur, 2 * l - 2, 2 * l - 1) = -at(cur, 2, 1);
        at(cur, 2 * l - 1, 2 * l - 1) = at(cur, 1, 1);
      }
    }
    const int lo = l - 1;  // angular momentum of this level
    const int w = 2 * lo + 1;
    double* o = out + lblock_offset(lo);
    for (int m2 = -lo; m2 <= lo; ++m2)
      for (int m1 = -lo; m1 <= lo; ++m1) o[(m2 + lo) * w + (m1 + lo)] = at(cur, m1 + l, m2 + l);
  }
}

template <int L>
__global__ void plan_geometry_kernel(PlanDev P) {
  const int N = P.N;
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= int64_t(N) * N) return;
  const int j = int(idx % N), i = int(idx / N);  // pair (row atom i, column atom j) stored at j + N*i
  const float* pi = P.pos + 3 * i;
  const float* pj = P.pos + 3 * j;
  double x = double(pi[0]) - double(pj[0]);
  double y = double(pi[1]) - double(pj[1]);
  double z = double(pi[2]) - double(pj[2]);
  double r = sqrt(x * x + y * y + z * z);
  double* dsm = P.pair_dsmall + size_t(idx) * P.ds;
  P.pair_dist[idx] = r;
  const int ne = 4 * L + 1;
  double2* eph = P.pair_eph + size_t(idx) * ne;
  if (i == j) {
    P.pair_phi[idx] = 0.0;
    for (int q = 0; q < P.ds; ++q) dsm[q] = 0.0;
    for (int q = 0; q < ne; ++q) eph[q] = make_double2(0.0, 0.0);
    return;
  }
  // getang with FEFF's single-precision threshold
  const double tiny = double(1.0e-7f);
  const double half_pi = 1.57079632679489661923;
  double phi;
  if (fabs(x) < tiny) phi = fabs(y) < tiny ? 0.0 : (y > tiny ? half_pi : -half_pi);
  else phi = atan2(y, x);
  double theta;
  if (r <= tiny) theta = 0.0;
  else if (z <= -r) theta = 3.14159265358979323846;
  else if (z < r) theta = acos(z / r);
  else theta = 0.0;
  P.pair_phi[idx] = phi;
  // azimuth phases e^{i mm (phi - pi)} of the G0 element, energy independent
  for (int mm = -2 * L; mm <= 2 * L; ++mm) {
    double sn, cs;
    sincos(double(mm) * (phi - 3.14159265358979323846), &sn, &cs);
    eph[mm + 2 * L] = make_double2(cs, sn);
  }
  rotxan_small_d<L>(theta, dsm);                        // forward, beta
  rotxan_small_d<L>(-theta, dsm + dsmall_per_dir(L));   // backward, -beta
}

void launch_plan_geometry(const PlanDev& P, cudaStream_t s) {
  const int64_t pairs = int64_t(P.N) * P.N;
  const int threads = 64;
  const unsigned blocks = unsigned((pairs + threads - 1) / threads);
  switch (P.L) {
    case 0: count_launch(); plan_geometry_kernel<0><<<blocks, threads, 0, s>>>(P); break;
    case 1: count_launch(); plan_geometry_kernel<1><<<blocks, threads, 0, s>>>(P); break;
    case 2: count_launch(); plan_geometry_kernel<2><<<blocks, threads, 0, s>>>(P); break;
    case 3: count_launch(); plan_geometry_kernel<3><<<blocks, threads, 0, s>>>(P); break;
    case 4: count_launch(); plan_geometry_kernel<4><<<blocks, threads, 0, s>>>(P); break;
    case 5: count_launch(); plan_geometry_kernel<5><<<blocks, threads, 0, s>>>(P); break;
    case 6: count_launch(); plan_geometry_kernel<6><<<blocks, threads, 0, s>>>(P); break;
    default: break;  // rejected on the host
  }
}

__global__ void plan_df_tables_kernel(size_t nd, const double* __restrict__ d, float2* __restrict__ ddf, size_t ne,
                                      const double2* __restrict__ e, float4* __restrict__ edf) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nd + ne; i += size_t(gridDim.x) * blockDim.x) {
    if (i < nd) {
      const float h = float(d[i]);
      ddf[i] = make_float2(h, float(d[i] - double(h)));
    } else {
      edf[i - nd] = split_hi_lo(e[i - nd]);
    }
  }
}

void launch_plan_df_tables(const PlanDev& P, cudaStream_t s) {
  const size_t nd = size_t(P.N) * P.N * P.ds, ne = size_t(P.N) * P.N * (4 * P.L + 1);
  count_launch();
  plan_df_tables_kernel<<<unsigned(std::min<size_t>((nd + ne + 255) / 256, 8192)), 256, 0, s>>>(
      nd, P.pair_dsmall, P.pair_dsmall_df, ne, P.pair_eph, P.pair_eph_df);
}

// ---- double-float (FP32 pair) helpers for the refined form's build ----
// A complex double-float is a float4 (re hi, im hi, re lo, im lo), the layout
// of split_hi_lo, so a result is stored as the hi/lo system entry directly.
__device__ __forceinline__ void df_prod(float ah, float al, float bh, float bl, float& ph, float& pl) {
  const float p = __fmul_rn(ah, bh);  // rounded product: must not be fused into the sum below
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  ph = p + e;
  pl = e - (ph - p);
}
__device__ __forceinline__ float4 dfc_mul(float4 a, float4 b) {
  df re{0.f, 0.f}, im{0.f, 0.f};
  df_mac(re, a.x, a.z, b.x, b.z);
  df_mac(re, -a.y, -a.w, b.y, b.w);
  df_mac(im, a.x, a.z, b.y, b.w);
  df_mac(im, a.y, a.w, b.x, b.z);
  return make_float4(re.hi, im.hi, re.lo, im.lo);
}
__device__ __forceinline__ void df_add(float& h, float& l, float bh, float bl) {
  float sh, e;
  df_two_sum(h, bh, sh, e);
  e += l + bl;
  h = sh + e;
  l = e - (h - sh);
}
__device__ __forceinline__ float4 dfc_neg(float4 a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }
__device__ __forceinline__ float4 dfc_sub(float4 a, float4 b) {
  df_add(a.x, a.z, -b.x, -b.z);
  df_add(a.y, a.w, -b.y, -b.w);
  return a;
}

// ---------------------------------------------------------------------------
// Build kernel: CTA = (column atom j, chunk of kBuildRowAtoms row atoms, energy).
// ---------------------------------------------------------------------------
struct BuildSmem {
  // offsets in doubles from the dynamic smem base
  int tcol0, tcol1, colinfo, rowinfo, pref, eph, g, dsm, clm, flag;
  int total_bytes;
};

__host__ __device__ inline BuildSmem build_smem_layout(int L, int nsp, int ds) {
  BuildSmem b{};
  const int L1 = L + 1;
  const int ncol_max = nsp * L1 * L1;
  const int RA = kBuildRowAtoms;
  int o = 0;
  b.tcol0 = o; o += 2 * ncol_max;
  b.tcol1 = o; o += 2 * ncol_max;
  b.colinfo = o; o += 2 * ncol_max;            // int4 per column (as 2 doubles)
  b.rowinfo = o; o += 2 * RA * ncol_max;       // int4 per row
  b.pref = o; o += 2 * RA * nsp;
  b.eph = o; o += 2 * RA * (4 * L + 1);
  b.g = o; o += 2 * RA * nsp * L1 * L1 * L1;
  b.dsm = o; o += RA * ds;
  b.clm = o; o += 2 * RA * nsp * (L + 2) * L1;
  b.flag = o; o += RA;                          // one int per pair (stored in a double slot)
  b.total_bytes = o * int(sizeof(double));
  return b;
}

__device__ __forceinline__ double2 t_phase(double2 d) {
  // (exp(2 i d) - 1) / (2 i), crates/refeff-core/src/fms/internals/t_matrix.rs:38-41
  double2 e = cexp(make_double2(-2.0 * d.y, 2.0 * d.x));
  double2 num = make_double2(e.x - 1.0, e.y);
  return make_double2(num.y / 2.0, -num.x / 2.0);
}

__device__ __forceinline__ double so_coef(const PlanDev& P, const double* tab, int l, int m, int s) {
  return tab[l + (P.L + 1) * ((m + P.L) + (2 * P.L + 1) * (s - 1))];
}

// Compact T of one state (l, m, spin s) of an atom with potential `pot`
// (fms_t_matrix_element, t_matrix.rs:10-143): t0 = T(0, state); t1 = T(1,
// state), the spin-flip coupling to the partner (l, m -+ 1, other spin) when
// nsp = 2.  Returns false when a phase shift it reads is not finite.
__device__ inline bool state_t_matrix(const PlanDev& P, const double2* xe, int pot, int l, int m, int s, double2& t0,
                                      double2& t1) {
  const int nsp = P.nsp, L = P.L, D = 2 * L + 1;
  auto phase = [&](int sp, int ll) { return xe[(sp - 1) + nsp * ((ll + L) + D * pot)]; };
  t1 = make_double2(0.0, 0.0);
  const double2 dm = phase(s, l);
  const bool finite = cfinite(dm) && cfinite(phase(s, -l));
  if (nsp == 1 && P.ispin == 0) {
    t0 = t_phase(dm);
    return finite;
  }
  int mp = 0, sp = 0;
  bool has_partner = false;
  if (nsp == 2) {
    if (s == 1 && m > -l) { mp = m - 1; sp = 2; has_partner = true; }
    if (s == 2 && m < l) { mp = m + 1; sp = 1; has_partner = true; }
  }
  const int cs = nsp == 1 ? (P.ispin > 0 ? 2 : 1) : s;
  const double mi = so_coef(P, P.t3m, l, m, cs), pl = so_coef(P, P.t3p, l, m, cs);
  const double2 a = t_phase(dm), b = t_phase(phase(s, -l));
  t0 = make_double2(a.x * (mi * mi) + b.x * (pl * pl), a.y * (mi * mi) + b.y * (pl * pl));
  if (has_partner) {
    const double mf = so_coef(P, P.t3m, l, m, s), ms = so_coef(P, P.t3m, l, mp, sp);
    const double pf = so_coef(P, P.t3p, l, m, s), ps = so_coef(P, P.t3p, l, mp, sp);
    const double2 a2 = t_phase(phase(sp, l)), b2 = t_phase(phase(sp, -l));
    const double2 mph = make_double2((a.x + a2.x) * 0.5, (a.y + a2.y) * 0.5);
    const double2 pph = make_double2((b.x + b2.x) * 0.5, (b.y + b2.y) * 0.5);
    t1 = make_double2(mph.x * mf * ms + pph.x * pf * ps, mph.y * mf * ms + pph.y * pf * ps);
  }
  return finite;
}

// Per-state T table for the iterative forms: t[e][2 * state + band] in
// device state order (band 0 = T(0, state), band 1 = T(1, state)).
__global__ void t_table_kernel(PlanDev P, const double2* __restrict__ xph, double2* __restrict__ t,
                               int* __restrict__ status) {
  const int a = blockIdx.x, e = blockIdx.y, nsp = P.nsp;
  const int D = 2 * P.L + 1;
  const double2* xe = xph + size_t(e) * size_t(nsp) * D * P.npot;
  const int off = P.atom_off[a], cnt = P.atom_off[a + 1] - off, pot = P.atom_pot[a];
  for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
    const int s = q % nsp + 1, lm = q / nsp;
    int l = 0;
    while ((l + 1) * (l + 1) <= lm) ++l;
    double2 t0, t1;
    if (!state_t_matrix(P, xe, pot, l, lm - l * l - l, s, t0, t1)) atomicMax(status + e, int(kDevNonfinite));
    t[(size_t(e) * P.n + off + q) * 2] = t0;
    t[(size_t(e) * P.n + off + q) * 2 + 1] = t1;
  }
}

void launch_t_table(const PlanDev& P, int E, const double2* xphase, double2* t, int* status, cudaStream_t s) {
  count_launch();
  t_table_kernel<<<dim3(unsigned(P.N), unsigned(E)), 64, 0, s>>>(P, xphase, t, status);
}

// Per ordered pair (i, j) and wave number k: whether the pair scatters (i != j,
// within rdirec), the pair prefactor e^{i rho}/rho e^{-msd k^2} and the Hankel
// polynomial table xclmz(rho), clm(il, im) at c[il + (L+2) im] (pairs.rs:9-51,
// polynomial.rs:8-83), in FP64; the refined form (kMode 1) stores them as
// double-float pairs in the same 16 bytes.
template <int kMode>
__device__ __forceinline__ void pair_tables(const PlanDev& P, double2 k, int i, int j, double2* c, double2* pref,
                                            int& ok, int* status_e) {
  const int L = P.L, L1 = L + 1, rows = L + 2, N = P.N;
  const size_t pij = size_t(j) + size_t(N) * i;
  const double dist = P.pair_dist[pij];
  ok = (i != j) && (dist * dist <= P.rdirec2);
  if (!cfinite(k)) { atomicMax(status_e, int(kDevNonfinite)); ok = 0; }
  if (!ok) return;
  const double2 rho = make_double2(k.x * dist, k.y * dist);
  if (rho.x == 0.0 && rho.y == 0.0) { atomicMax(status_e, int(kDevZeroRho)); ok = 0; return; }
  const double msd = P.sigsqr[size_t(j) + size_t(N) * i];
  // e^{i rho} / rho * e^{-msd k^2}
  const double2 ph = cdiv(cexp(make_double2(-rho.y, rho.x)), rho);
  if (msd != 0.0) {
    const double2 k2 = cmul(k, k);
    const double2 damp = cexp(make_double2(-msd * k2.x, -msd * k2.y));
    *pref = cmul(ph, damp);
  } else {
    *pref = ph;  // e^{0} = 1 exactly: the same value without the FP64 exponential
  }
  // xclmz recursion
  const double2 z = cdiv(make_double2(0.0, -1.0), rho);
  const double2 one = make_double2(1.0, 0.0);
  for (int q = 0; q < rows * L1; ++q) c[q] = make_double2(0.0, 0.0);
  c[0] = one;
  if (L >= 1) c[1] = csub(one, z);
  for (int il = 2; il <= L; ++il) {
    const double2 f = cscale(z, double(2 * il - 1));
    c[il] = csub(c[il - 2], cmul(f, c[il - 1]));
  }
  double2 cmm = one;
  for (int im = 2; im <= L1; ++im) {
    const int mmm = im - 1;
    cmm = cmul(cneg(cmm), cscale(z, double(2 * mmm - 1)));
    c[(im - 1) + rows * (im - 1)] = cmm;
    const double2 oz = csub(one, cscale(z, double(im)));
    c[im + rows * (im - 1)] = cmul(cscale(cmm, double(2 * im - 1)), oz);
    for (int il = im + 1; il <= L; ++il) {
      const double2 f = cscale(z, double(2 * il - 1));
      c[il + rows * (im - 1)] =
          csub(c[(il - 2) + rows * (im - 1)], cmul(f, cadd(c[(il - 1) + rows * (im - 1)], c[(il - 1) + rows * (im - 2)])));
    }
  }
  if constexpr (kMode == 1) {
    // the refined form works on double-float copies (same 16 bytes per entry)
    for (int q = 0; q < rows * L1; ++q) reinterpret_cast<float4*>(c)[q] = split_hi_lo(c[q]);
    *reinterpret_cast<float4*>(pref) = split_hi_lo(*pref);
  }
}

// The pair tables of every (energy, ordered pair, spin) of a batch, one thread
// each: hank[((e N + j) N + i) nsp + s] holds (L+2)(L+1) Hankel entries and the
// prefactor, hflag[(e N + j) N + i] whether the pair scatters.  In the build
// CTAs this FP64 work ran on one thread per pair while the others waited at a
// barrier; here it fills the GPU and the build starts from finished tables.
template <int kMode>
__global__ void __launch_bounds__(256) pair_hankel_kernel(PlanDev P, int E, const double2* __restrict__ kE,
                                                          double2* __restrict__ hank, int* __restrict__ hflag,
                                                          int* __restrict__ status) {
  const int N = P.N, nsp = P.nsp, per = (P.L + 2) * (P.L + 1) + 1;
  const long long total = (long long)E * N * N * nsp;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int s = int(t % nsp);
    long long q = t / nsp;
    const int i = int(q % N);
    q /= N;
    const int j = int(q % N);
    const int e = int(q / N);
    double2* c = hank + size_t(t) * per;
    int ok = 0;
    pair_tables<kMode>(P, kE[size_t(e) * nsp + s], i, j, c, c + (per - 1), ok, status + e);
    if (s == 0) hflag[(size_t(e) * N + j) * N + i] = ok;
  }
}

// kMode 0: FP64 system [A | B]; 1: the same as hi/lo float pairs plus the FP32
// copy; 2: the plain free propagator G0 (FP64, n x n, for the iterative forms).
template <int kMode>
__global__ void __launch_bounds__(256) build_system_kernel(PlanDev P, const double2* __restrict__ kE,
                                                           const double2* __restrict__ xph, BatchLayout lay,
                                                           double2* __restrict__ M64, float2* __restrict__ M32,
                                                           int* __restrict__ status, const double2* __restrict__ hank,
                                                           const int* __restrict__ hflag) {
  extern __shared__ double sm[];
  const int L = P.L, L1 = L + 1, nsp = P.nsp, N = P.N;
  const int j = blockIdx.x;
  const int i0 = blockIdx.y * kBuildRowAtoms;
  const int e = blockIdx.z;
  const int i1 = min(i0 + kBuildRowAtoms, N);
  const int RA = i1 - i0;
  const int cj0 = P.atom_off[j], ncol = P.atom_off[j + 1] - cj0;
  const int r0 = P.atom_off[i0], nrow = P.atom_off[i1] - r0;
  const BuildSmem lay_s = build_smem_layout(L, nsp, P.ds);
  double2* tcol0 = reinterpret_cast<double2*>(sm + lay_s.tcol0);
  double2* tcol1 = reinterpret_cast<double2*>(sm + lay_s.tcol1);
  int4* colinfo = reinterpret_cast<int4*>(sm + lay_s.colinfo);
  int4* rowinfo = reinterpret_cast<int4*>(sm + lay_s.rowinfo);
  double2* pref = reinterpret_cast<double2*>(sm + lay_s.pref);
  double2* eph = reinterpret_cast<double2*>(sm + lay_s.eph);
  double2* gtab = reinterpret_cast<double2*>(sm + lay_s.g);
  double* dsm = sm + lay_s.dsm;
  double2* clm = reinterpret_cast<double2*>(sm + lay_s.clm);
  int* flag = reinterpret_cast<int*>(sm + lay_s.flag);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int D = 2 * L + 1;
  const double2* xe = kMode == 2 ? nullptr : xph + size_t(e) * size_t(nsp) * D * P.npot;
  const double2* ke = kE + size_t(e) * nsp;
  const int potj = P.atom_pot[j];

  // ---- columns of atom j: state decode and compact T (t_matrix.rs:149-190) ----
  for (int q = tid; q < ncol; q += nthr) {
    const int s = q % nsp + 1, lm = q / nsp;
    int l = 0;
    while ((l + 1) * (l + 1) <= lm) ++l;
    const int m = lm - l * l - l;
    int partner = -1;
    if (nsp == 2) {
      if (s == 1 && m > -l) partner = q - 1;
      if (s == 2 && m < l) partner = q + 1;
    }
    colinfo[q] = make_int4(l, m, s, partner);
    double2 t0 = make_double2(0.0, 0.0), t1 = t0;
    if (kMode != 2 && !state_t_matrix(P, xe, potj, l, m, s, t0, t1)) atomicMax(status + e, int(kDevNonfinite));
    if constexpr (kMode == 1) {
      reinterpret_cast<float4*>(tcol0)[q] = split_hi_lo(t0);
      reinterpret_cast<float4*>(tcol1)[q] = split_hi_lo(t1);
    } else {
      tcol0[q] = t0;
      tcol1[q] = t1;
    }
  }
  // ---- rows of the chunk ----
  // Rows are visited grouped by (l, spin), then atom and m, so that the lanes
  // of a warp share l1 and the spin: the mu loop below has one trip count per
  // warp and no lane idles on a spin mismatch.
  // rowinfo[v] = (atom << 2 | spin, l, m, row offset in the chunk).
  for (int v = tid; v < nrow; v += nthr) {
    int l = 0, w = v, cnt = 0;
    for (;; ++l) {
      cnt = 0;
      for (int p = 0; p < RA; ++p) cnt += P.atom_lmax[i0 + p] >= l;
      const int group = cnt * (2 * l + 1) * nsp;
      if (w < group) break;
      w -= group;
    }
    const int per_spin = cnt * (2 * l + 1);
    const int sp = w / per_spin + 1;
    w %= per_spin;
    int k = w / (2 * l + 1), p = 0;
    for (;; ++p)
      if (P.atom_lmax[i0 + p] >= l && k-- == 0) break;
    const int m = w % (2 * l + 1) - l;
    const int rr = P.atom_off[i0 + p] - r0 + (l * l + (m + l)) * nsp + (sp - 1);
    rowinfo[v] = make_int4((p << 2) | sp, l, m, rr);
  }
  // ---- per pair: small-d tables (resident, from the plan) ----
  for (int t = tid; t < RA * P.ds; t += nthr) {
    const int p = t / P.ds, q = t % P.ds;
    const size_t src = (size_t(j) + size_t(N) * (i0 + p)) * P.ds + q;
    if constexpr (kMode == 1) reinterpret_cast<float2*>(dsm)[t] = P.pair_dsmall_df[src];
    else dsm[t] = P.pair_dsmall[src];
  }
  // ---- per pair: azimuth phases e^{i m (phi - pi)}, m in [-2L, 2L] (resident, from the plan) ----
  for (int t = tid; t < RA * (4 * L + 1); t += nthr) {
    const int p = t / (4 * L + 1), q = t % (4 * L + 1);
    const size_t src = (size_t(j) + size_t(N) * (i0 + p)) * (4 * L + 1) + q;
    if constexpr (kMode == 1) reinterpret_cast<float4*>(eph)[t] = P.pair_eph_df[src];
    else eph[t] = P.pair_eph[src];
  }
  // ---- per (pair, spin): rho, prefactor, Hankel polynomial table ----
  const int rows = L + 2;
  if (hank) {
    // computed for the whole batch by pair_hankel_kernel: copy this CTA's 16 pairs
    const int per = rows * L1 + 1;
    const size_t t0 = (size_t(e) * N + j) * N + i0;
    for (int idx = tid; idx < RA * nsp * per; idx += nthr) {
      const int tl = idx / per, q = idx - tl * per;
      const double2 v = hank[(t0 * nsp + tl) * per + q];
      if (q < rows * L1) clm[size_t(tl) * rows * L1 + q] = v;
      else pref[tl] = v;
    }
    for (int p = tid; p < RA; p += nthr) flag[p] = hflag[t0 + p];
  } else {
    for (int t = tid; t < RA * nsp; t += nthr) {
      const int p = t / nsp, sp = t % nsp;
      int ok = 0;
      pair_tables<kMode>(P, ke[sp], i0 + p, j, clm + size_t(t) * rows * L1, pref + t, ok, status + e);
      if (sp == 0) flag[p] = ok;
    }
  }
  __shared__ int gdec[(kMaxL + 1) * (kMaxL + 1) * (kMaxL + 1)];
  for (int q = tid; q < L1 * L1 * L1; q += nthr) gdec[q] = (q % L1) | (((q / L1) % L1) << 8) | ((q / (L1 * L1)) << 16);
  __syncthreads();
  // ---- z-axis propagator g(l1, l2, mu) per (pair, spin) (xgllm) ----
  // entry t = rem + gsz ps of the table, rem = l1 + L1 (l2 + L1 mu); (ps, rem) follow t without a
  // division, (l1, l2, mu) come from the decode table
  const int gsz = L1 * L1 * L1;
  auto advance_g = [&](int& ps, int& rem) {
    rem += nthr;
    while (rem >= gsz) {
      rem -= gsz;
      ++ps;
    }
  };
  for (int t = tid, ps = tid / gsz, rem = tid % gsz; t < RA * nsp * gsz; t += nthr, advance_g(ps, rem)) {
    const int p = nsp == 2 ? ps >> 1 : ps;
    const int dec = gdec[rem];
    const int l1 = dec & 0xFF, l2 = (dec >> 8) & 0xFF, mu = dec >> 16;
    if constexpr (kMode == 1) {
      // g in double-float: gamtl = c(l1, nu) (2 l1 + 1) / xnlm, gam = c(l2, mu + nu) (-1)^mu xnlm, summed,
      // times the pair prefactor
      float4 gdf = make_float4(0.f, 0.f, 0.f, 0.f);
      if (flag[p] && mu <= l1 && mu <= l2) {
        const float4* c = reinterpret_cast<const float4*>(clm) + size_t(ps) * rows * L1;
        const float2 w1 = P.xnlm_w_df[mu + L1 * l1];
        float2 n2 = P.xnlm_df[mu + L1 * l2];
        if (mu & 1) n2 = make_float2(-n2.x, -n2.y);
        df gr{0.f, 0.f}, gi{0.f, 0.f};
        const int numax = min(l1, l2 - mu);
        for (int nu = 0; nu <= numax; ++nu) {
          const float4 c1 = c[l1 + rows * nu], c2 = c[l2 + rows * (mu + nu)];
          float arh, arl, aih, ail, brh, brl, bih, bil;
          df_prod(c1.x, c1.z, w1.x, w1.y, arh, arl);
          df_prod(c1.y, c1.w, w1.x, w1.y, aih, ail);
          df_prod(c2.x, c2.z, n2.x, n2.y, brh, brl);
          df_prod(c2.y, c2.w, n2.x, n2.y, bih, bil);
          df_mac(gr, arh, arl, brh, brl);
          df_mac(gr, -aih, -ail, bih, bil);
          df_mac(gi, arh, arl, bih, bil);
          df_mac(gi, aih, ail, brh, brl);
        }
        gdf = dfc_mul(reinterpret_cast<const float4*>(pref)[ps], make_float4(gr.hi, gi.hi, gr.lo, gi.lo));
      }
      reinterpret_cast<float4*>(gtab)[t] = gdf;
      continue;
    }
    double2 g = make_double2(0.0, 0.0);
    if (flag[p] && mu <= l1 && mu <= l2) {
      const double2* c = clm + size_t(ps) * rows * L1;
      const double wn1 = P.xnlm_w[mu + L1 * l1], n2 = P.xnlm[mu + L1 * l2];
      const double sgn = (mu & 1) ? -1.0 : 1.0;
      const int numax = min(l1, l2 - mu);
      for (int nu = 0; nu <= numax; ++nu) {
        const double2 cl1 = c[l1 + rows * nu];
        const double2 cl2 = c[l2 + rows * (mu + nu)];
        const double2 gamtl = make_double2(cl1.x * wn1, cl1.y * wn1);  // (2 l1 + 1) c / xnlm
        const double2 gam = make_double2(cl2.x * (sgn * n2), cl2.y * (sgn * n2));
        g = cadd(g, cmul(gamtl, gam));
      }
      g = cmul(pref[ps], g);  // the pair prefactor e^{i rho}/rho e^{-msd k^2}, folded in once per table entry
    }
    gtab[t] = g;
  }
  __syncthreads();

  // ---- elements: rows fastest (coalesced column-major stores) ----
  const int dpd = P.ds / 2;
  const int bcol_j = P.bcol ? P.bcol[j] : (j == N - 1 ? 0 : -1);
  const bool absorber_col = bcol_j >= 0;  // the columns of a representative also form B
  const size_t base = size_t(e) * lay.stride;
  auto g0 = [&](int p, int l1, int m1, int s1, int l2, int m2, int s2) -> double2 {
    if (s1 != s2 || !flag[p]) return make_double2(0.0, 0.0);
    const double* tf = dsm + size_t(p) * P.ds + lblock_offset(l2);          // forward (beta), l2 block
    const double* tb = dsm + size_t(p) * P.ds + dpd + lblock_offset(l1);    // backward (-beta), l1 block
    const double2* gg = gtab + size_t(p * nsp + (s1 - 1)) * gsz;
    const int w1 = 2 * l1 + 1, w2 = 2 * l2 + 1, mn = min(l1, l2);
    double sx = 0.0, sy = 0.0;
    for (int mu = -mn; mu <= mn; ++mu) {
      const int amu = mu < 0 ? -mu : mu;
      const double dd = tb[(mu + l1) * w1 + (m1 + l1)] * tf[(m2 + l2) * w2 + (mu + l2)];
      const double2 gv = gg[l1 + L1 * (l2 + L1 * amu)];
      sx = fma(dd, gv.x, sx);
      sy = fma(dd, gv.y, sy);
    }
    const double2 ph = eph[p * (4 * L + 1) + (m2 - m1 + 2 * L)];
    return cmul(ph, make_double2(sx, sy));
  };
  // the same element in double-float on the FP32 pipes (refined form): GB300
  // runs FP32 about 64 times faster than FP64, and the system is stored as hi/lo
  // float pairs anyway
  const float2* dsm2 = reinterpret_cast<const float2*>(dsm);
  const float4* gtab4 = reinterpret_cast<const float4*>(gtab);
  const float4* eph4 = reinterpret_cast<const float4*>(eph);
  auto g0df = [&](int p, int l1, int m1, int s1, int l2, int m2, int s2) -> float4 {
    if (s1 != s2 || !flag[p]) return make_float4(0.f, 0.f, 0.f, 0.f);
    const float2* tf = dsm2 + size_t(p) * P.ds + lblock_offset(l2);
    const float2* tb = dsm2 + size_t(p) * P.ds + dpd + lblock_offset(l1);
    const float4* gg = gtab4 + size_t(p * nsp + (s1 - 1)) * gsz;
    const int w1 = 2 * l1 + 1, w2 = 2 * l2 + 1, mn = min(l1, l2);
    df sx{0.f, 0.f}, sy{0.f, 0.f};
    for (int mu = -mn; mu <= mn; ++mu) {
      const int amu = mu < 0 ? -mu : mu;
      const float2 b = tb[(mu + l1) * w1 + (m1 + l1)], f = tf[(m2 + l2) * w2 + (mu + l2)];
      float dh, dl;
      df_prod(b.x, b.y, f.x, f.y, dh, dl);
      const float4 gv = gg[l1 + L1 * (l2 + L1 * amu)];
      df_mac(sx, dh, dl, gv.x, gv.z);
      df_mac(sy, dh, dl, gv.y, gv.w);
    }
    return dfc_mul(eph4[p * (4 * L + 1) + (m2 - m1 + 2 * L)], make_float4(sx.hi, sy.hi, sx.lo, sy.lo));
  };
  const int total = nrow * ncol;
  // element idx is (row v, column cc) with idx = v + nrow cc; (v, cc) follow idx without a division
  auto advance = [&](int& v, int& cc) {
    v += nthr;
    while (v >= nrow) {
      v -= nrow;
      ++cc;
    }
  };
  for (int idx = tid, v = tid % nrow, cc = tid / nrow; idx < total; idx += nthr, advance(v, cc)) {
    const int4 ri = rowinfo[v];
    const int4 ci = colinfo[cc];
    const int rp = ri.x >> 2, rs = ri.x & 3;
    const int r = r0 + ri.w, c = cj0 + cc;
    if constexpr (kMode == 1) {
      float4 a = make_float4(0.f, 0.f, 0.f, 0.f), gcol = a;
      if (i0 + rp != j) {
        const float4* t0 = reinterpret_cast<const float4*>(tcol0);
        const float4* t1 = reinterpret_cast<const float4*>(tcol1);
        gcol = g0df(rp, ri.y, ri.z, rs, ci.x, ci.y, ci.z);
        a = dfc_neg(dfc_mul(gcol, t0[cc]));
        if (ci.w >= 0) {
          const int4 pi = colinfo[ci.w];
          a = dfc_sub(a, dfc_mul(g0df(rp, ri.y, ri.z, rs, pi.x, pi.y, pi.z), t1[cc]));
        }
      }
      if (r == c) df_add(a.x, a.z, 1.f, 0.f);
      const size_t ai = base + size_t(r) + size_t(lay.lda) * c;
      reinterpret_cast<float4*>(M64)[ai] = a;
      M32[ai] = make_float2(a.x, a.y);
      if (absorber_col) {
        const size_t bi = base + size_t(r) + size_t(lay.lda) * (size_t(lay.n) + bcol_j + cc);
        reinterpret_cast<float4*>(M64)[bi] = gcol;
        M32[bi] = make_float2(gcol.x, gcol.y);
      }
      continue;
    }
    double2 a = make_double2(0.0, 0.0), gcol = make_double2(0.0, 0.0);
    if (i0 + rp != j) {
      gcol = g0(rp, ri.y, ri.z, rs, ci.x, ci.y, ci.z);
      a = cneg(cmul(gcol, tcol0[cc]));
      if (kMode != 2 && ci.w >= 0) {
        const int4 pi = colinfo[ci.w];
        const double2 gp = g0(rp, ri.y, ri.z, rs, pi.x, pi.y, pi.z);
        a = csub(a, cmul(gp, tcol1[cc]));
      }
    }
    const size_t ai = base + size_t(r) + size_t(lay.lda) * c;
    if (kMode == 2) {
      M64[ai] = gcol;
      continue;
    }
    if (r == c) a.x += 1.0;
    if (kMode == 1) {
      // FP32 form: the FP64 system is kept as an exact-to-2^-48 hi/lo float pair
      // (same 16 bytes per entry) for the refinement residual; hi is the LU copy.
      const float4 sa = split_hi_lo(a);
      reinterpret_cast<float4*>(M64)[ai] = sa;
      M32[ai] = make_float2(sa.x, sa.y);
    } else {
      M64[ai] = a;
    }
    if (absorber_col) {
      const size_t bi = base + size_t(r) + size_t(lay.lda) * (size_t(lay.n) + bcol_j + cc);
      if (kMode == 1) {
        const float4 sb = split_hi_lo(gcol);
        reinterpret_cast<float4*>(M64)[bi] = sb;
        M32[bi] = make_float2(sb.x, sb.y);
      } else {
        M64[bi] = gcol;
      }
    }
  }
}

template <int kMode>
static void launch_build_mode(const PlanDev& P, int E, const double2* k, const double2* xphase, const BatchLayout& lay,
                              double2* M64, float2* M32, int* status, const BuildScratch* scratch, cudaStream_t s) {
  const BuildSmem b = build_smem_layout(P.L, P.nsp, P.ds);
  dim3 grid(unsigned(P.N), unsigned((P.N + kBuildRowAtoms - 1) / kBuildRowAtoms), unsigned(E));
  ensure_smem_limit(reinterpret_cast<const void*>(build_system_kernel<kMode>), size_t(b.total_bytes));
  double2* hank = scratch ? scratch->hank : nullptr;
  int* hflag = scratch ? scratch->hflag : nullptr;
  if (hank && hflag) {
    const long long work = (long long)E * P.N * P.N * P.nsp;
    count_launch();
    pair_hankel_kernel<kMode><<<unsigned(std::min<long long>(4096, (work + 255) / 256)), 256, 0, s>>>(P, E, k, hank,
                                                                                                     hflag, status);
  } else {
    hank = nullptr;
    hflag = nullptr;
  }
  count_launch();
  build_system_kernel<kMode><<<grid, 256, b.total_bytes, s>>>(P, k, xphase, lay, M64, M32, status, hank, hflag);
}

size_t build_scratch_entries(const PlanDev& P, int E) {
  return size_t(E) * P.N * P.N * P.nsp * size_t((P.L + 2) * (P.L + 1) + 1);
}

void launch_build_system(const PlanDev& P, int E, const double2* k, const double2* xphase, const BatchLayout& lay,
                         double2* M64, float2* M32, int* status, cudaStream_t s, const BuildScratch* scratch) {
  if (M32) launch_build_mode<1>(P, E, k, xphase, lay, M64, M32, status, scratch, s);
  else launch_build_mode<0>(P, E, k, xphase, lay, M64, nullptr, status, scratch, s);
}

void launch_build_g0(const PlanDev& P, int E, const double2* k, const BatchLayout& lay, double2* G0, int* status,
                     cudaStream_t s, const BuildScratch* scratch) {
  launch_build_mode<2>(P, E, k, nullptr, lay, G0, nullptr, status, scratch, s);
}

}  // namespace rfx
