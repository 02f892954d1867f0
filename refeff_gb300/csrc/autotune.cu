// Autotuner of the batched form: for a set of clusters solved together by
// refeff_fms_real_space_spectrum_multi, it picks per size bucket the FP32
// elimination's inner panel width (16 or 32 columns, or single-level panels)
// and whether 64-column blocks are paired, then the number of streams the
// clusters are packed onto, by timing the candidates on a sample of each
// cluster's energies.  Choices are cached in a JSON file keyed by the device,
// the form and the clusters' sizes, so a later run of the same workload applies
// them without measuring.
//
// It is written on the public C ABI only (plan queries, plan tuning, context
// options and the many-cluster call), and replaces the fixed rayon split of
// fms_real_space_spectrum (crates/refeff-core/src/fms/driver.rs:231-239),
// which has no tunable parameters of its own.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/refeff_fms.h"

namespace {

struct Bucket {
  int n_lo = 0, n_hi = 0;  // inclusive state-count range
  int inner = 0, paired = -1;
  std::vector<int> plans;
};

struct Entry {
  int streams = 4;
  std::vector<Bucket> buckets;
  double seconds_default = 0.0, seconds_tuned = 0.0;
};

// C = nsp (L+1)^2 channels: nsp = 2 exactly when C / 2 is a square (C cannot
// be both a square and twice one).
void split_channels(int C, int& nsp, int& L) {
  auto isq = [](int v) {
    const int r = int(std::lround(std::sqrt(double(v))));
    return r * r == v ? r : -1;
  };
  const int half = C % 2 == 0 ? isq(C / 2) : -1;
  nsp = half > 0 ? 2 : 1;
  L = (half > 0 ? half : isq(C)) - 1;
}

// Buckets of neighbouring sizes: n rounded up to a multiple of 256.
int bucket_of(int n) { return (n + 255) / 256; }

std::string device_name(int dev) {
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
  std::string s = prop.name;
  for (auto& c : s)
    if (c == '"' || c == '\\') c = '_';
  return s;
}

std::string workload_key(int dev, refeff_fms_form form, const std::vector<std::pair<int, int>>& nm) {
  std::vector<std::pair<int, int>> sorted = nm;
  std::sort(sorted.begin(), sorted.end());
  std::ostringstream k;
  k << device_name(dev) << "|form" << int(form) << "|";
  for (size_t i = 0; i < sorted.size(); ++i) k << (i ? "," : "") << sorted[i].first << "x" << sorted[i].second;
  return k.str();
}

// The cache file: one entry per line,
//   "<key>": {"streams": S, "seconds_default": a, "seconds_tuned": b, "buckets": [[lo, hi, inner, paired], ...]}
// inside a JSON object {"refeff_fms_autotune": 1, "entries": {...}}.
std::map<std::string, std::string> read_cache(const std::string& path) {
  std::map<std::string, std::string> out;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    const size_t a = line.find('"');
    const size_t b = a == std::string::npos ? a : line.find("\": {", a + 1);
    if (a == std::string::npos || b == std::string::npos || line.find("\"streams\"") == std::string::npos) continue;
    std::string body = line.substr(b + 3);
    while (!body.empty() && (body.back() == ',' || body.back() == ' ' || body.back() == '\r')) body.pop_back();
    out[line.substr(a + 1, b - a - 1)] = body;
  }
  return out;
}

bool write_cache(const std::string& path, const std::map<std::string, std::string>& entries) {
  std::ofstream f(path, std::ios::trunc);
  if (!f) return false;
  f << "{\"refeff_fms_autotune\": 1, \"entries\": {\n";
  size_t i = 0;
  for (const auto& kv : entries) f << "\"" << kv.first << "\": " << kv.second << (++i < entries.size() ? ",\n" : "\n");
  f << "}}\n";
  return bool(f);
}

std::string entry_json(const Entry& e) {
  std::ostringstream o;
  o.precision(9);
  o << "{\"streams\": " << e.streams << ", \"seconds_default\": " << e.seconds_default
    << ", \"seconds_tuned\": " << e.seconds_tuned << ", \"buckets\": [";
  for (size_t i = 0; i < e.buckets.size(); ++i)
    o << (i ? ", " : "") << "[" << e.buckets[i].n_lo << ", " << e.buckets[i].n_hi << ", " << e.buckets[i].inner << ", "
      << e.buckets[i].paired << "]";
  o << "]}";
  return o.str();
}

bool parse_entry(const std::string& body, Entry& e) {
  auto num_after = [&](const char* tag, double& v) {
    const size_t p = body.find(tag);
    if (p == std::string::npos) return false;
    v = std::strtod(body.c_str() + p + std::strlen(tag), nullptr);
    return true;
  };
  double s = 0;
  if (!num_after("\"streams\": ", s)) return false;
  e.streams = int(s);
  num_after("\"seconds_default\": ", e.seconds_default);
  num_after("\"seconds_tuned\": ", e.seconds_tuned);
  const size_t p = body.find("\"buckets\": [");
  if (p == std::string::npos) return false;
  const char* c = body.c_str() + p + std::strlen("\"buckets\": [");
  e.buckets.clear();
  while (*c) {
    while (*c == ' ' || *c == ',') ++c;
    if (*c != '[') break;
    ++c;
    Bucket b;
    char* end = nullptr;
    b.n_lo = int(std::strtol(c, &end, 10));
    c = end + 1;
    b.n_hi = int(std::strtol(c, &end, 10));
    c = end + 1;
    b.inner = int(std::strtol(c, &end, 10));
    c = end + 1;
    b.paired = int(std::strtol(c, &end, 10));
    c = end;
    while (*c && *c != ']') ++c;
    if (*c == ']') ++c;
    e.buckets.push_back(b);
  }
  return true;
}

}  // namespace

extern "C" int refeff_fms_autotune_multi(refeff_fms_context* ctx, int n_plans, refeff_fms_plan* const* plans,
                                         const refeff_fms_energy_points* points, refeff_fms_form form,
                                         int sample_energies, const char* cache_path, refeff_fms_tuning* out) {
  if (!ctx || n_plans <= 0 || !plans || !points || sample_energies < 0) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return REFEFF_FMS_ERR_CUDA;
  std::vector<std::pair<int, int>> nm(static_cast<size_t>(n_plans));
  std::vector<int> nsp(static_cast<size_t>(n_plans)), xph(static_cast<size_t>(n_plans));
  for (int i = 0; i < n_plans; ++i) {
    int n = 0, C = 0, m = 0, npot = 0;
    int rc = refeff_fms_plan_query(plans[i], &n, &C, &m, &npot);
    if (rc) return rc;
    nm[size_t(i)] = {n, m};
    int ns = 1, L = 0;
    split_channels(C, ns, L);
    nsp[size_t(i)] = ns;                      // wave numbers per energy
    xph[size_t(i)] = ns * (2 * L + 1) * npot;  // phase shifts per energy
  }
  const std::string key = workload_key(dev, form, nm);
  std::map<std::string, std::string> cache;
  if (cache_path && *cache_path) cache = read_cache(cache_path);

  // the buckets and their plans
  std::map<int, Bucket> by;
  for (int i = 0; i < n_plans; ++i) {
    Bucket& b = by[bucket_of(nm[size_t(i)].first)];
    if (b.plans.empty()) b.n_lo = b.n_hi = nm[size_t(i)].first;
    b.n_lo = std::min(b.n_lo, nm[size_t(i)].first);
    b.n_hi = std::max(b.n_hi, nm[size_t(i)].first);
    b.plans.push_back(i);
  }
  auto apply = [&](const Entry& e) -> int {
    int rc = refeff_fms_context_set_option(ctx, REFEFF_FMS_OPT_MULTI_STREAMS, e.streams);
    if (rc) return rc;
    for (int i = 0; i < n_plans; ++i) {
      const int n = nm[size_t(i)].first;
      int inner = 0, paired = -1;
      for (const Bucket& b : e.buckets)
        if (n >= b.n_lo && n <= b.n_hi) { inner = b.inner; paired = b.paired; }
      rc = refeff_fms_plan_set_tuning(plans[i], inner, paired);
      if (rc) return rc;
    }
    return REFEFF_FMS_OK;
  };
  auto report = [&](const Entry& e, int from_cache) {
    if (!out) return;
    out->streams = e.streams;
    out->buckets = int(e.buckets.size());
    out->seconds_default = e.seconds_default;
    out->seconds_tuned = e.seconds_tuned;
    out->from_cache = from_cache;
  };
  auto hit = cache.find(key);
  Entry cached;
  if (hit != cache.end() && parse_entry(hit->second, cached)) {
    const int rc = apply(cached);
    if (rc == REFEFF_FMS_OK) report(cached, 1);
    return rc;
  }

  // the sample: up to sample_energies evenly spaced energies of every plan (all when 0)
  std::vector<std::vector<std::complex<double>>> ks(static_cast<size_t>(n_plans)), xs(static_cast<size_t>(n_plans));
  std::vector<refeff_fms_energy_points> sp(static_cast<size_t>(n_plans));
  std::vector<std::vector<std::complex<double>>> outs(static_cast<size_t>(n_plans));
  std::vector<std::vector<int32_t>> sts(static_cast<size_t>(n_plans));
  for (int i = 0; i < n_plans; ++i) {
    const int E = points[i].n_energies;
    const int S = sample_energies > 0 ? std::min(E, sample_energies) : E;
    int n = 0, C = 0, m = 0, npot = 0;
    refeff_fms_plan_query(plans[i], &n, &C, &m, &npot);
    const auto* kin = reinterpret_cast<const std::complex<double>*>(points[i].wave_numbers);
    const auto* xin = reinterpret_cast<const std::complex<double>*>(points[i].phase_shifts);
    for (int q = 0; q < S; ++q) {
      const int e = S > 1 ? int((long long)q * (E - 1) / (S - 1)) : 0;
      ks[size_t(i)].insert(ks[size_t(i)].end(), kin + size_t(e) * nsp[size_t(i)], kin + size_t(e + 1) * nsp[size_t(i)]);
      xs[size_t(i)].insert(xs[size_t(i)].end(), xin + size_t(e) * xph[size_t(i)], xin + size_t(e + 1) * xph[size_t(i)]);
    }
    sp[size_t(i)].n_energies = S;
    sp[size_t(i)].wave_numbers = reinterpret_cast<const refeff_complex128*>(ks[size_t(i)].data());
    sp[size_t(i)].phase_shifts = reinterpret_cast<const refeff_complex128*>(xs[size_t(i)].data());
    outs[size_t(i)].resize(size_t(S) * size_t(C) * size_t(C) * size_t(npot));
    sts[size_t(i)].resize(size_t(S));
  }
  // time of the many-cluster call over a subset of the plans: one warm call
  // (graph capture for the batch shape), then the best of two (the first
  // repeat captures the call as one graph, the second replays it)
  auto timed = [&](const std::vector<int>& subset, double& seconds) -> int {
    std::vector<refeff_fms_plan*> pl;
    std::vector<refeff_fms_energy_points> pt;
    std::vector<refeff_complex128*> o;
    std::vector<int32_t*> st;
    for (int i : subset) {
      pl.push_back(plans[i]);
      pt.push_back(sp[size_t(i)]);
      o.push_back(reinterpret_cast<refeff_complex128*>(outs[size_t(i)].data()));
      st.push_back(sts[size_t(i)].data());
    }
    seconds = 1e300;
    for (int rep = 0; rep < 3; ++rep) {
      const auto t0 = std::chrono::steady_clock::now();
      const int rc = refeff_fms_real_space_spectrum_multi(ctx, int(pl.size()), pl.data(), pt.data(), form, o.data(),
                                                          st.data(), nullptr);
      if (rc) return rc;
      const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (rep > 0) seconds = std::min(seconds, dt);
    }
    return REFEFF_FMS_OK;
  };
  std::vector<int> all(static_cast<size_t>(n_plans));
  for (int i = 0; i < n_plans; ++i) all[size_t(i)] = i;

  Entry e;
  e.streams = 4;
  for (auto& kv : by) e.buckets.push_back(kv.second);
  int rc = apply(e);  // the defaults
  if (rc) return rc;
  rc = timed(all, e.seconds_default);
  if (rc) return rc;
  const bool fp32 = form == REFEFF_FMS_FORM_FP32_REFINED;
  if (fp32) {
    for (Bucket& b : e.buckets) {
      struct Cand {
        int inner, paired;
      };
      std::vector<Cand> cands = {{0, -1}, {16, 1}, {16, 0}, {32, 1}, {32, 0}, {1, 0}};
      double best = 1e300;
      Cand pick = {0, -1};
      for (const Cand& c : cands) {
        if (c.inner >= 16 && b.n_hi < 128) continue;
        for (int i : b.plans) refeff_fms_plan_set_tuning(plans[i], c.inner, c.paired);
        double t = 0;
        rc = timed(b.plans, t);
        if (rc) return rc;
        if (t < best * 0.98) {  // a candidate must win by 2% to displace the incumbent
          best = t;
          pick = c;
        }
      }
      b.inner = pick.inner;
      b.paired = pick.paired;
      for (int i : b.plans) refeff_fms_plan_set_tuning(plans[i], b.inner, b.paired);
    }
  }
  double best = 1e300;
  int best_streams = 4;
  for (int streams : {4, 2, 8, 16}) {
    if (streams > 2 * n_plans && streams != 4) continue;
    e.streams = streams;
    rc = apply(e);
    if (rc) return rc;
    double t = 0;
    rc = timed(all, t);
    if (rc) return rc;
    if (t < best * 0.98) {
      best = t;
      best_streams = streams;
    }
  }
  e.streams = best_streams;
  e.seconds_tuned = best;
  rc = apply(e);
  if (rc) return rc;
  if (cache_path && *cache_path) {
    cache[key] = entry_json(e);
    if (!write_cache(cache_path, cache)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  report(e, 0);
  return REFEFF_FMS_OK;
}
