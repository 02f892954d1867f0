// FEFF file seam of the FMS stage: the handoff readers (fms.inp, global.inp,
// geom.dat, .dimensions.dat, phase.bin with its PAD encoding) and the
// byte-compatible gg.bin / gg.dat / log3.dat writers, plus the module-level
// entry refeff_fms_run_dir that turns a work directory's handoffs into gg
// sections on the GPU.
//
// Reference behaviour followed:
//   fms.inp reader          crates/refeff-io/src/fms_input.rs:287-430
//   global.inp control line crates/refeff-io/src/global_input.rs:314-330
//   geom.dat reader         crates/refeff-io/src/structure_output.rs:470-570
//   .dimensions.dat         crates/refeff-io/src/structure_output.rs:428-441
//   phase.bin reader        crates/refeff-io/src/phase_bin/parse.rs:18-410
//   PAD decode              crates/refeff-io/src/pad.rs:102-127
//   E20.10 writer           crates/refeff-io/src/format.rs:164-209
//   gg.dat / gg.bin text    crates/refeff-io/src/gg_dat.rs:155-233
//   stage flow              crates/refeff-engine/src/fms.rs:1102-1127, 3549-3695, 4218-4322, 4972-5054
//   log3.dat                crates/refeff-engine/src/fms.rs:5995-6058
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/refeff_fms.h"
#include "host_internal.h"

namespace {

// ---------------------------------------------------------------------------
// number formatting
// ---------------------------------------------------------------------------

// Integer power by repeated squaring, the algorithm the reference's `powi`
// lowers to (compiler-rt __powidf2): multiply for each set bit, square, and
// take the reciprocal for negative exponents.
double powi_squaring(double a, int b) {
  const bool recip = b < 0;
  double r = 1.0;
  while (true) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? 1.0 / r : r;
}

// Fortran E<width>.<precision> with a zero-scaled mantissa (0.d...E+ee), as
// written by the reference for gg.dat (format.rs:174-209): signed zero kept,
// exponent at least two digits, left-padded to the field width.
void append_fortran_exp(std::string& out, double value, int width, int precision) {
  const int exponent = value == 0.0 ? 0 : int(std::floor(std::log10(std::fabs(value)))) + 1;
  const double mantissa = value == 0.0 ? value : value / powi_squaring(10.0, exponent);
  char mant[64];
  std::snprintf(mant, sizeof mant, "%.*f", precision, mantissa);
  const int ae = exponent < 0 ? -exponent : exponent;
  char digits[16];
  std::snprintf(digits, sizeof digits, "%d", ae);
  const int ndig = int(std::strlen(digits));
  const int ewidth = ndig > 2 ? ndig : 2;
  const int field = int(std::strlen(mant)) + 2 + ewidth;
  for (int i = field; i < width; ++i) out.push_back(' ');
  out += mant;
  out.push_back('E');
  out.push_back(exponent < 0 ? '-' : '+');
  for (int i = ndig; i < ewidth; ++i) out.push_back('0');
  out += digits;
}

std::string section_prefix(int number, int rows, int cols) {
  char buf[512];
  std::snprintf(buf, sizeof buf,
                "#SN#   Section: %4d\n#DF# This section written in txt.\n#H#\n"
                "#DT# 2D complex array with sizes %4d%4d\n"
                "#H# File is organized as follows:  Array(1,i)     Array(1,i+1)    Array(1,i+2)  . . .\n"
                "#H#                                Array(2,i)\n"
                "#H#                                     .\n#H#                                     .\n"
                "#H#                                     .\n",
                number, rows, cols);
  return buf;
}

// gg_dat_bytes (gg_dat.rs:174-202): per section the canonical prefix, then one
// line per row, each value as E20.10(re) ' ' E20.10(im).
std::string gg_dat_text(int n_sections, int dim, const refeff_complex128* values) {
  std::string out;
  out.reserve(size_t(n_sections) * (600 + size_t(dim) * dim * 42));
  for (int s = 0; s < n_sections; ++s) {
    out += section_prefix(s + 1, dim, dim);
    const refeff_complex128* sec = values + size_t(s) * dim * dim;
    for (int r = 0; r < dim; ++r) {
      for (int c = 0; c < dim; ++c) {
        const refeff_complex128 v = sec[size_t(r) + size_t(dim) * c];
        append_fortran_exp(out, v.re, 20, 10);
        out.push_back(' ');
        append_fortran_exp(out, v.im, 20, 10);
      }
      out.push_back('\n');
    }
  }
  return out;
}

// gg_slice.bin / gg_diag.bin (crates/refeff-io/src/rhorrp_gg_bin.rs:138-160,
// 228-252): Fortran sequential unformatted records, each a 4-byte
// little-endian length, the payload and the length again; a header record of
// 32-bit dimensions, then one record of default-kind complex values (two
// little-endian f32 each) in FEFF's column-major order.  The values are the
// reference's Complex32 data: each part narrowed to f32, and a part that is
// not finite after narrowing is an error (validate_complex_values, :562-572).
void put_u32_le(std::string& out, uint32_t v) {
  for (int i = 0; i < 4; ++i) out.push_back(char((v >> (8 * i)) & 0xffu));
}

void put_record(std::string& out, const std::string& payload) {
  put_u32_le(out, uint32_t(payload.size()));
  out += payload;
  put_u32_le(out, uint32_t(payload.size()));
}

// header dims, then count complex values (already in file order); false on a non-finite value
bool rhorrp_bin(const std::vector<int>& dims, size_t count, const refeff_complex128* values, std::string& out) {
  std::string header, payload;
  for (int d : dims) put_u32_le(header, uint32_t(d));
  payload.reserve(count * 8);
  for (size_t i = 0; i < count; ++i) {
    const float part[2] = {float(values[i].re), float(values[i].im)};
    for (float f : part) {
      if (!std::isfinite(f)) return false;
      uint32_t bits;
      std::memcpy(&bits, &f, sizeof bits);
      put_u32_le(payload, bits);
    }
  }
  out.clear();
  put_record(out, header);
  put_record(out, payload);
  return true;
}

bool write_file_atomic(const std::string& path, const std::string& bytes) {
  const std::string tmp = path + ".tmp";
  {
    std::ofstream f(tmp, std::ios::binary | std::ios::trunc);
    if (!f) return false;
    f.write(bytes.data(), std::streamsize(bytes.size()));
    if (!f) return false;
  }
  return std::rename(tmp.c_str(), path.c_str()) == 0;
}

bool read_file(const std::string& path, std::string& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

std::vector<std::string> split_lines(const std::string& text) {
  std::vector<std::string> lines;
  size_t a = 0;
  while (a <= text.size()) {
    size_t b = text.find('\n', a);
    if (b == std::string::npos) b = text.size();
    std::string line = text.substr(a, b - a);
    if (!line.empty() && line.back() == '\r') line.pop_back();
    lines.push_back(line);
    if (b == text.size()) break;
    a = b + 1;
  }
  if (!lines.empty() && lines.back().empty()) lines.pop_back();
  return lines;
}

std::vector<std::string> fields(const std::string& line) {
  std::vector<std::string> out;
  std::istringstream ss(line);
  std::string t;
  while (ss >> t) out.push_back(t);
  return out;
}

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t");
  return s.substr(a, b - a + 1);
}

bool parse_double(const std::string& t, double& v) {
  std::string u = t;
  for (char& c : u)
    if (c == 'D' || c == 'd') c = 'E';
  char* end = nullptr;
  v = std::strtod(u.c_str(), &end);
  return end && *end == '\0' && !u.empty();
}

bool parse_int(const std::string& t, long long& v) {
  char* end = nullptr;
  v = std::strtoll(t.c_str(), &end, 10);
  return end && *end == '\0' && !t.empty();
}

// ---------------------------------------------------------------------------
// PAD decoding (pad.rs:102-127)
// ---------------------------------------------------------------------------
constexpr int kPadOff = 37, kPadBase = 90, kPadHalf = 45;

bool pad_decode(const char* s, int npack, double& out) {
  const int iexp = int(static_cast<unsigned char>(s[0])) - kPadOff - kPadHalf;
  const int second = int(static_cast<unsigned char>(s[1])) - kPadOff;
  const int isgn = (second % 2) * 2 - 1;
  const int itmp = second / 2;
  const double base = double(kPadBase);
  double sum = double(itmp) / powi_squaring(base, 2);
  for (int i = npack - 1; i >= 2; --i)
    sum += double(int(static_cast<unsigned char>(s[i])) - kPadOff) / powi_squaring(base, i + 1);
  out = 2.0 * double(isgn) * double(kPadBase) * sum * powi_squaring(10.0, iexp);
  return true;
}

struct PadCursor {
  const std::vector<std::string>& lines;
  size_t pos = 0;
  std::string error;
  bool complex_block(int npack, size_t expected, std::vector<refeff_complex128>& out) {
    out.clear();
    while (out.size() < expected) {
      if (pos >= lines.size()) { error = "phase.bin ended inside a PAD block"; return false; }
      const std::string t = trim(lines[pos++]);
      if (t.empty() || t[0] != '$') { error = "expected a '$' PAD line"; return false; }
      const std::string payload = t.substr(1);
      const size_t unit = size_t(2 * npack);
      if (payload.empty() || payload.size() % unit) { error = "bad PAD payload length"; return false; }
      for (size_t k = 0; k + unit <= payload.size(); k += unit) {
        refeff_complex128 v;
        pad_decode(payload.c_str() + k, npack, v.re);
        pad_decode(payload.c_str() + k + npack, npack, v.im);
        if (out.size() < expected) out.push_back(v);
      }
    }
    return true;
  }
  bool real_block(int npack, size_t expected, std::vector<double>& out) {
    out.clear();
    while (out.size() < expected) {
      if (pos >= lines.size()) { error = "phase.bin ended inside a PAD block"; return false; }
      const std::string t = trim(lines[pos++]);
      if (t.empty() || t[0] != '!') { error = "expected a '!' PAD line"; return false; }
      const std::string payload = t.substr(1);
      if (payload.empty() || payload.size() % size_t(npack)) { error = "bad PAD payload length"; return false; }
      for (size_t k = 0; k + size_t(npack) <= payload.size(); k += size_t(npack)) {
        double v;
        pad_decode(payload.c_str() + k, npack, v);
        if (out.size() < expected) out.push_back(v);
      }
    }
    return true;
  }
};

struct PhaseBin {
  int nsp = 0, ne = 0, npot = 0, npad = 0;
  int ne1 = 0, ne3 = 0, ihole = 0, ntrans = 8, nq = 1;
  std::vector<refeff_complex128> rkk;   // q = 0 transition moments (energy, transition, spin), energy fastest
  std::vector<refeff_complex128> em;    // ne
  std::vector<refeff_complex128> eref;  // ne x nsp, energy fastest
  std::vector<int> lmax;                // per potential
  std::vector<int> iz;                  // atomic number per potential (potential header)
  double rnrmav = 0.0;                  // average Norman radius, Bohr (scalar block, parse.rs:50)
  // phase shifts per potential: (energy, l_slot, spin) with l_slot = l + lmax(pot)
  std::vector<std::vector<refeff_complex128>> ph;
};

int read_phase_bin(const std::string& path, PhaseBin& pb, std::string& err) {
  std::string text;
  if (!read_file(path, text)) { err = "cannot read " + path; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  const std::vector<std::string> lines = split_lines(text);
  if (lines.empty()) { err = "empty phase.bin"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  const std::vector<std::string> h = fields(lines[0]);
  if (h.size() != 8 && h.size() != 10 && h.size() != 11) { err = "phase.bin header needs 8, 10 or 11 integers"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  long long v[11] = {0};
  for (size_t i = 0; i < h.size(); ++i)
    if (!parse_int(h[i], v[i])) { err = "bad phase.bin header field " + h[i]; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  pb.nsp = int(v[0]);
  pb.ne = int(v[1]);
  pb.ne1 = int(v[2]);
  pb.ne3 = int(v[3]);
  pb.npot = int(v[4]) + 1;
  pb.ihole = int(v[5]);
  pb.npad = int(v[7]);
  if (h.size() >= 10) pb.ntrans = int(v[9]);  // indmax (parse.rs:31-46)
  if (h.size() == 11) pb.nq = int(v[10]);
  if (pb.ntrans < 0 || pb.nq < 1) { err = "phase.bin transition counts out of range"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  if (pb.nsp < 1 || pb.nsp > 2 || pb.ne < 0 || pb.npot < 1 || pb.npad <= 2) { err = "phase.bin header out of range"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  PadCursor cur{lines, 1, ""};
  std::vector<double> dum;
  if (!cur.real_block(pb.npad, 3, dum) || !cur.complex_block(pb.npad, size_t(pb.ne), pb.em) ||
      !cur.complex_block(pb.npad, size_t(pb.ne) * pb.nsp, pb.eref)) {
    err = cur.error;
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  pb.rnrmav = dum[0];
  pb.lmax.resize(size_t(pb.npot));
  pb.iz.resize(size_t(pb.npot));
  pb.ph.resize(size_t(pb.npot));
  for (int p = 0; p < pb.npot; ++p) {
    if (cur.pos >= lines.size()) { err = "phase.bin ended before potential " + std::to_string(p); return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
    const std::vector<std::string> ph = fields(lines[cur.pos++]);
    long long lm = 0, iz = 0;
    if (ph.size() < 2 || !parse_int(ph[0], lm) || !parse_int(ph[1], iz) || lm < 0) { err = "bad potential header"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
    pb.lmax[size_t(p)] = int(lm);
    pb.iz[size_t(p)] = int(iz);
    const int lc = 2 * int(lm) + 1;
    auto& tab = pb.ph[size_t(p)];
    tab.assign(size_t(pb.ne) * lc * pb.nsp, {0.0, 0.0});
    for (int s = 0; s < pb.nsp; ++s) {
      std::vector<refeff_complex128> blk;
      if (!cur.complex_block(pb.npad, size_t(pb.ne) * lc, blk)) { err = cur.error; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
      // parse.rs:143-158: energy outer, l slot inner
      size_t idx = 0;
      for (int e = 0; e < pb.ne; ++e)
        for (int l = 0; l < lc; ++l) tab[size_t(e) + size_t(pb.ne) * (size_t(l) + size_t(lc) * s)] = blk[idx++];
    }
  }
  // transition moments, one block per q (parse.rs:88-100, 156-180): spin outer,
  // transition, energy inner -- the order of the (energy, transition, spin)
  // column-major table kept here for q = 0
  for (int q = 0; q < pb.nq; ++q) {
    std::vector<refeff_complex128> blk;
    if (!cur.complex_block(pb.npad, size_t(pb.ne) * pb.ntrans * pb.nsp, blk)) { err = cur.error; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
    if (q == 0) pb.rkk = std::move(blk);
  }
  return REFEFF_FMS_OK;
}

refeff_complex128 csqrt_polar(double re, double im) {
  // num-complex sqrt (the wave number is formed in f64 before narrowing)
  if (im == 0.0) {
    if (!std::signbit(re)) return {std::sqrt(re), im};
    const double r = std::sqrt(-re);
    return {0.0, std::signbit(im) ? -r : r};
  }
  if (re == 0.0) {
    const double x = std::sqrt(std::fabs(im) / 2.0);
    return {x, im > 0 ? x : -x};
  }
  const double r = std::hypot(re, im), th = std::atan2(im, re);
  const double sr = std::sqrt(r), h = th / 2.0;
  return {sr * std::cos(h), sr * std::sin(h)};
}

double narrow(double v) { return double(float(v)); }

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" int refeff_fms_write_gg_dat(const char* path, int n_sections, int dim, const refeff_complex128* values) {
  if (!path || n_sections < 0 || dim < 0 || (n_sections > 0 && dim > 0 && !values)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  return write_file_atomic(path, gg_dat_text(n_sections, dim, values)) ? REFEFF_FMS_OK : REFEFF_FMS_ERR_INVALID_ARGUMENT;
}

extern "C" int refeff_fms_write_gg_slice_bin(const char* path, int ne, int rows, int cols,
                                             const refeff_complex128* values) {
  if (!path || ne <= 0 || rows <= 0 || cols <= 0 || !values) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  std::string out;
  if (!rhorrp_bin({rows, cols, ne}, size_t(ne) * rows * cols, values, out)) return REFEFF_FMS_ERR_NONFINITE_INPUT;
  return write_file_atomic(path, out) ? REFEFF_FMS_OK : REFEFF_FMS_ERR_INVALID_ARGUMENT;
}

extern "C" int refeff_fms_write_gg_diag_bin(const char* path, int ne, int n_atoms, int dim,
                                            const refeff_complex128* values) {
  if (!path || ne <= 0 || n_atoms <= 0 || dim <= 0 || !values) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  std::string out;
  if (!rhorrp_bin({dim, dim, n_atoms, ne}, size_t(ne) * n_atoms * dim * dim, values, out))
    return REFEFF_FMS_ERR_NONFINITE_INPUT;
  return write_file_atomic(path, out) ? REFEFF_FMS_OK : REFEFF_FMS_ERR_INVALID_ARGUMENT;
}

extern "C" int refeff_fms_phase_bin_dims(const char* path, int* nsp, int* ne, int* npot, int* lmax_max) {
  if (!path) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  PhaseBin pb;
  std::string err;
  const int rc = read_phase_bin(path, pb, err);
  if (rc) return rc;
  int lm = 0;
  for (int v : pb.lmax) lm = v > lm ? v : lm;
  if (nsp) *nsp = pb.nsp;
  if (ne) *ne = pb.ne;
  if (npot) *npot = pb.npot;
  if (lmax_max) *lmax_max = lm;
  return REFEFF_FMS_OK;
}

extern "C" int refeff_fms_phase_bin_read(const char* path, refeff_complex128* energy_grid,
                                         refeff_complex128* reference_energy, int* potential_lmax,
                                         refeff_complex128* phase_shifts) {
  if (!path) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  PhaseBin pb;
  std::string err;
  const int rc = read_phase_bin(path, pb, err);
  if (rc) return rc;
  int lm = 0;
  for (int v : pb.lmax) lm = v > lm ? v : lm;
  const int lc = 2 * lm + 1;
  if (energy_grid) std::memcpy(energy_grid, pb.em.data(), pb.em.size() * sizeof(refeff_complex128));
  if (reference_energy) std::memcpy(reference_energy, pb.eref.data(), pb.eref.size() * sizeof(refeff_complex128));
  for (int p = 0; p < pb.npot; ++p) {
    if (potential_lmax) potential_lmax[p] = pb.lmax[size_t(p)];
    if (!phase_shifts) continue;
    const int plc = 2 * pb.lmax[size_t(p)] + 1;
    for (int s = 0; s < pb.nsp; ++s)
      for (int l = 0; l < lc; ++l)
        for (int e = 0; e < pb.ne; ++e) {
          const int sl = l - lm + pb.lmax[size_t(p)];  // signed l aligned at 0
          refeff_complex128 v{0.0, 0.0};
          if (sl >= 0 && sl < plc) v = pb.ph[size_t(p)][size_t(e) + size_t(pb.ne) * (size_t(sl) + size_t(plc) * s)];
          phase_shifts[size_t(e) + size_t(pb.ne) * (size_t(l) + size_t(lc) * (size_t(s) + size_t(pb.nsp) * p))] = v;
        }
  }
  return REFEFF_FMS_OK;
}

namespace {

struct FmsInp {
  int mfms = 0, idwopt = 0, minv = 0;
  double rfms2 = 0, rdirec = 0, toler1 = 0, toler2 = 0, tk = 0, thetad = 0, sig2g = 0;
  std::vector<int> lmaxph;
  int do_fms = 0;
  bool save_gg_slice = false;
};

int parse_fms_inp(const std::string& path, FmsInp& f, std::string& err) {
  std::string text;
  if (!read_file(path, text)) { err = "cannot read " + path; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  const auto L = split_lines(text);
  size_t i = 0;
  auto expect = [&](const char* hdr) {
    if (i >= L.size() || trim(L[i]) != hdr) { err = std::string("fms.inp: expected header ") + hdr; return false; }
    ++i;
    return true;
  };
  auto nums = [&](size_t count, std::vector<double>& out) {
    if (i >= L.size()) { err = "fms.inp ended early"; return false; }
    const auto fs = fields(L[i++]);
    if (fs.size() < count) { err = "fms.inp: short value line"; return false; }
    out.resize(count);
    for (size_t k = 0; k < count; ++k)
      if (!parse_double(fs[k], out[k])) { err = "fms.inp: bad number " + fs[k]; return false; }
    return true;
  };
  std::vector<double> v;
  if (!expect("mfms, idwopt, minv") || !nums(3, v)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  f.mfms = int(v[0]); f.idwopt = int(v[1]); f.minv = int(v[2]);
  if (!expect("rfms2, rdirec, toler1, toler2") || !nums(4, v)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  f.rfms2 = v[0]; f.rdirec = v[1]; f.toler1 = v[2]; f.toler2 = v[3];
  if (!expect("tk, thetad, sig2g") || !nums(3, v)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  f.tk = v[0]; f.thetad = v[1]; f.sig2g = v[2];
  if (!expect("lmaxph(0:nph)") || i >= L.size()) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  for (const auto& t : fields(L[i++])) {
    long long x;
    if (!parse_int(t, x)) { err = "fms.inp: bad lmaxph " + t; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
    f.lmaxph.push_back(int(x));
  }
  if (!expect("the number of decomposi") || !nums(1, v)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (i < L.size() && trim(L[i]) == "save_gg_slice") {
    ++i;
    if (i >= L.size()) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    const std::string b = trim(L[i++]);
    f.save_gg_slice = !b.empty() && (b[0] == 'T' || b[0] == 't' || b == ".true." || b == ".TRUE.");
    if (!expect("do_fms") || !nums(1, v)) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    f.do_fms = int(v[0]);
  } else {
    f.do_fms = f.mfms;
  }
  return REFEFF_FMS_OK;
}

int parse_global_ispin(const std::string& path, int& ispin, std::string& err) {
  std::string text;
  if (!read_file(path, text)) { err = "cannot read " + path; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  const auto L = split_lines(text);
  for (size_t i = 0; i + 1 < L.size(); ++i)
    if (trim(L[i]) == "ipol, ispin, le2, elpty, angks, l2lp, do_nrixs, ldecmx, lj") {
      const auto fs = fields(L[i + 1]);
      double x;
      if (fs.size() >= 2 && parse_double(fs[1], x)) { ispin = int(x); return REFEFF_FMS_OK; }
    }
  err = "global.inp: control line not found";
  return REFEFF_FMS_ERR_INVALID_ARGUMENT;
}

struct GeomRow {
  double x, y, z;
  int iph;
};

int parse_geom_text(const std::string& text, int& nph, std::vector<GeomRow>& rows, std::string& err) {
  const auto L = split_lines(text);
  size_t i = 0;
  while (i < L.size() && trim(L[i]).empty()) ++i;
  if (i >= L.size()) { err = "empty geom.dat"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  const auto h = fields(L[i++]);
  long long nat = 0, np = 0;
  if (h.size() < 5 || h[0] != "nat," || h[1] != "nph" || h[2] != "=" || !parse_int(h[3], nat) || !parse_int(h[4], np)) {
    err = "geom.dat: expected 'nat, nph =' header";
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  nph = int(np);
  size_t models = 0;
  while (models < size_t(np + 1) && i < L.size()) {
    if (trim(L[i]).empty()) { ++i; continue; }
    models += fields(L[i++]).size();
  }
  i += 2;  // column header + separator
  rows.clear();
  while (rows.size() < size_t(nat) && i < L.size()) {
    if (trim(L[i]).empty()) { ++i; continue; }
    const auto fs = fields(L[i++]);
    GeomRow r;
    long long iph;
    if (fs.size() < 6 || !parse_double(fs[1], r.x) || !parse_double(fs[2], r.y) || !parse_double(fs[3], r.z) ||
        !parse_int(fs[4], iph)) {
      err = "geom.dat: bad atom row";
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    }
    r.iph = int(iph);
    rows.push_back(r);
  }
  if (rows.size() != size_t(nat)) { err = "geom.dat: fewer rows than nat"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  return REFEFF_FMS_OK;
}

void set_error(refeff_fms_context* ctx, const std::string& msg) { rfx::set_last_error(ctx, msg); }

}  // namespace

extern "C" int refeff_fms_run_dir(refeff_fms_context* ctx, const char* work_dir, refeff_fms_form form,
                                  refeff_fms_report* report) {
  if (!ctx || !work_dir) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  const std::string dir = std::string(work_dir) + "/";
  std::string err;
  FmsInp fi;
  int rc = parse_fms_inp(dir + "fms.inp", fi, err);
  if (rc) { set_error(ctx, err); return rc; }
  if (fi.mfms == 0) return REFEFF_FMS_OK;  // fms_enabled (fms.rs:633-635): the stage is off
  PhaseBin pb;
  rc = read_phase_bin(dir + "phase.bin", pb, err);
  if (rc) { set_error(ctx, err); return rc; }
  int ispin = 0;
  rc = parse_global_ispin(dir + "global.inp", ispin, err);
  if (rc) { set_error(ctx, err); return rc; }
  int nph = 0;
  std::vector<GeomRow> geom;
  std::string gtext;
  if (!read_file(dir + "geom.dat", gtext)) {
    // no geom.dat: FEFF's rdinp writes it from feff.inp before this stage runs;
    // build the same text (same 5-decimal rounding) from feff.inp here
    std::string ferr;
    rc = rfx::geom_dat_from_feff_inp(dir + "feff.inp", gtext, ferr);
    if (rc) { set_error(ctx, "no geom.dat, and feff.inp: " + ferr); return rc; }
  }
  rc = parse_geom_text(gtext, nph, geom, err);
  if (rc) { set_error(ctx, err); return rc; }
  const int max_potential = pb.npot - 1;
  if (nph != max_potential) {
    set_error(ctx, "geom.dat nph does not match phase.bin maximum potential");
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  if (int(fi.lmaxph.size()) <= max_potential) {
    set_error(ctx, "fms.inp has too few lmaxph values");
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  // global_fms_lmax (fms.rs:4218-4239) and the phase-bin lmax check (4241-4258)
  int L = 0;
  for (int p = 0; p <= max_potential; ++p) {
    if (fi.lmaxph[size_t(p)] < 0 || fi.lmaxph[size_t(p)] > pb.lmax[size_t(p)]) {
      set_error(ctx, "lmaxph outside the phase.bin lmax");
      return REFEFF_FMS_ERR_INVALID_ANGULAR_LIMIT;
    }
    L = std::max(L, fi.lmaxph[size_t(p)]);
  }
  if (fi.idwopt >= 0 && fi.idwopt != 0 && fi.idwopt != 3) {
    set_error(ctx, "only idwopt < 0 (uniform sig2g), 0 (correlated Debye) and 3 (classical Debye) are supported");
    return REFEFF_FMS_ERR_UNSUPPORTED;
  }
  // effective radii (fms.rs:4260-4284)
  const float rfms2 = fi.rfms2 >= 0.0 ? float(fi.rfms2) : 0.0f;
  const float rdirec = fi.rdirec >= 0.0 ? float(fi.rdirec) : 0.0f;
  // cluster (fms_atoms_from_geom, fms.rs:4286-4322)
  std::vector<float> pos(geom.size() * 3), opos(geom.size() * 3);
  std::vector<int> pots(geom.size()), opots(geom.size());
  for (size_t i = 0; i < geom.size(); ++i) {
    pos[3 * i] = float(geom[i].x);
    pos[3 * i + 1] = float(geom[i].y);
    pos[3 * i + 2] = float(geom[i].z);
    pots[i] = geom[i].iph;
  }
  int natoms = 0;
  rc = refeff_fms_yprep_cluster(0, max_potential, int(geom.size()), pots.data(), pos.data(), rfms2, int(geom.size()),
                                opos.data(), opots.data(), &natoms);
  if (rc) { set_error(ctx, "cluster preparation failed"); return rc; }
  // plan
  refeff_fms_plan_input in{};
  in.n_atoms = natoms;
  in.positions_xyz = opos.data();
  in.potentials = opots.data();
  in.spin_channels = pb.nsp;
  in.spin_selector = ispin;
  // gg holds the absorber block only, which does not depend on lfms; the
  // all-potential range still requires a representative of every potential
  // (driver.rs:36-60, fms.rs:4314-4320).
  if (fi.do_fms != 0) {
    std::vector<int> seen(size_t(max_potential) + 1, 0);
    for (int a = 0; a < natoms; ++a) seen[size_t(opots[size_t(a)])] = 1;
    for (int p = 0; p <= max_potential; ++p)
      if (!seen[size_t(p)] || natoms <= max_potential) {
        set_error(ctx, "FMS cluster lacks a representative of potential " + std::to_string(p));
        return REFEFF_FMS_ERR_MISSING_REPRESENTATIVE;
      }
  }
  in.lfms = 0;
  in.minv = fi.minv;
  in.max_potential = max_potential;
  in.global_lmax = L;
  in.raw_potential_lmax = fi.lmaxph.data();
  in.direct_cutoff = rdirec;
  // pair sigma^2 (fms_mean_square_displacements_with_metadata, fms.rs:4345-4433):
  // the Debye models take phase.bin's rnrmav and per-potential atomic numbers
  std::vector<float> msd;
  in.mean_square_displacements = nullptr;
  if (fi.idwopt == 0 || fi.idwopt == 3) {
    msd.resize(size_t(natoms) * size_t(natoms));
    rc = refeff_fms_debye_sigma2_table(ctx, fi.idwopt, natoms, opos.data(), opots.data(), pb.npot, pb.iz.data(),
                                       fi.tk, fi.thetad, pb.rnrmav, float(fi.sig2g), msd.data(), nullptr);
    if (rc) return rc;
    in.mean_square_displacements = msd.data();
  }
  in.sig2g = float(fi.sig2g);
  in.convergence_tolerance = float(fi.toler1);
  in.zero_tolerance = float(fi.toler2);
  // save_gg_slice asks for the full scattering matrix, which forces the LU form
  // (full_scattering_matrix_requested, fms.rs:3610; driver.rs:72-96)
  refeff_fms_plan* plan = nullptr;
  rc = fi.save_gg_slice ? refeff_fms_real_space_plan_create_full(ctx, &in, &plan)
                        : refeff_fms_real_space_plan_create(ctx, &in, &plan);
  if (rc) return rc;
  int n = 0, C = 0, m = 0, npot = 0;
  refeff_fms_plan_query(plan, &n, &C, &m, &npot);
  // per energy: wave numbers (fms.rs:4972-4985) and xphase (fms.rs:5002-5054), narrowed to f32
  const int E = pb.ne, nsp = pb.nsp, D = 2 * L + 1;
  std::vector<refeff_complex128> k(size_t(E) * nsp), xph(size_t(E) * nsp * D * npot, {0.0, 0.0});
  const double bohr = 0.529177249;
  for (int e = 0; e < E; ++e) {
    for (int s = 0; s < nsp; ++s) {
      const refeff_complex128 em = pb.em[size_t(e)], er = pb.eref[size_t(e) + size_t(E) * s];
      const refeff_complex128 w = csqrt_polar(2.0 * (em.re - er.re), 2.0 * (em.im - er.im));
      k[size_t(e) * nsp + s] = {narrow(w.re / bohr), narrow(w.im / bohr)};
    }
    refeff_complex128* xe = xph.data() + size_t(e) * nsp * D * npot;
    for (int p = 0; p < npot; ++p) {
      const int eff = std::min(fi.lmaxph[size_t(p)], L), plm = pb.lmax[size_t(p)], plc = 2 * plm + 1;
      for (int s = 0; s < nsp; ++s)
        for (int l = -eff; l <= eff; ++l) {
          const refeff_complex128 v = pb.ph[size_t(p)][size_t(e) + size_t(E) * (size_t(l + plm) + size_t(plc) * s)];
          xe[size_t(s) + size_t(nsp) * (size_t(l + L) + size_t(D) * p)] = {narrow(v.re), narrow(v.im)};
        }
    }
  }
  std::vector<refeff_complex128> scat(size_t(E) * C * C * npot);
  std::vector<int32_t> status(static_cast<size_t>(E));
  refeff_fms_energy_points pts{E, k.data(), xph.data()};
  std::vector<refeff_complex128> slice, diag;
  if (fi.save_gg_slice) {
    slice.resize(size_t(E) * C * n);
    diag.resize(size_t(E) * natoms * C * C);
    rc = refeff_fms_real_space_spectrum_full(plan, &pts, scat.data(), slice.data(), diag.data(), status.data(), report);
  } else {
    rc = refeff_fms_real_space_spectrum(plan, &pts, form, scat.data(), status.data(), report);
  }
  if (rc) {
    refeff_fms_real_space_plan_destroy(plan);
    return rc;
  }
  // gg sections widened to .dimensions.dat nspu (fms.rs:1975-2047)
  int nspu = nsp;
  {
    std::string dtext;
    if (read_file(dir + ".dimensions.dat", dtext)) {
      const auto L2 = split_lines(dtext);
      for (const auto& line : L2) {
        const auto fs = fields(line);
        long long v4;
        if (fs.size() >= 4 && parse_int(fs[3], v4)) { nspu = int(v4); break; }
      }
      if (nspu < nsp) {
        refeff_fms_real_space_plan_destroy(plan);
        set_error(ctx, ".dimensions.dat nspu is smaller than the active spin count");
        return REFEFF_FMS_ERR_INVALID_ARGUMENT;
      }
    }
  }
  const int ang = m / nsp, dim = ang * nspu;
  std::vector<refeff_complex128> sections(size_t(E) * dim * dim);
  for (int e = 0; e < E; ++e)
    refeff_fms_gg_section(plan, scat.data() + size_t(e) * C * C * npot, nspu, sections.data() + size_t(e) * dim * dim);
  refeff_fms_real_space_plan_destroy(plan);
  const std::string gg = gg_dat_text(E, dim, sections.data());
  if (!write_file_atomic(dir + "gg.bin", gg) || !write_file_atomic(dir + "gg.dat", gg)) {
    set_error(ctx, "cannot write gg.bin / gg.dat");
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  // gg_slice.bin and gg_diag.bin (generate_gg_outputs_from_source_handoffs, fms.rs:1102-1127)
  if (fi.save_gg_slice) {
    std::string bytes;
    if (!rhorrp_bin({C, n, E}, slice.size(), slice.data(), bytes)) {
      set_error(ctx, "gg_slice value is not finite");
      return REFEFF_FMS_ERR_NONFINITE_INPUT;
    }
    if (!write_file_atomic(dir + "gg_slice.bin", bytes)) {
      set_error(ctx, "cannot write gg_slice.bin");
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    }
    if (!rhorrp_bin({C, C, natoms, E}, diag.size(), diag.data(), bytes)) {
      set_error(ctx, "gg_diag value is not finite");
      return REFEFF_FMS_ERR_NONFINITE_INPUT;
    }
    if (!write_file_atomic(dir + "gg_diag.bin", bytes)) {
      set_error(ctx, "cannot write gg_diag.bin");
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    }
  }
  // log3.dat (fms.rs:5995-6058)
  std::string log = "FMS calculation of full Green's function ...\nFEFF-serial using 1 thread.\n";
  char buf[128];
  std::snprintf(buf, sizeof buf, "Using %5d energy points.\n", E);
  log += buf;
  if (fi.idwopt == 0) log += "Applying Debye-Waller factors using a Correlated Debye model.\n";
  if (fi.idwopt == 3) log += "Applying Debye-Waller factors using the Classical Debye model.\n";
  log += "xprep done\n";
  if (fi.do_fms != 0 && natoms > 1) {
    std::snprintf(buf, sizeof buf, "FMS for a cluster of %4d atoms\n", natoms);
    log += buf;
    int next = 1;
    for (int e = 1; e <= E; ++e) {
      if (e < next) continue;
      std::snprintf(buf, sizeof buf, "Energy point %4d/%4d\n", e, E);
      log += buf;
      next = next == 1 ? 10 : next + 10;
    }
  }
  log += "Done with module: FMS.\n";
  if (!write_file_atomic(dir + "log3.dat", log)) {
    set_error(ctx, "cannot write log3.dat");
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  return REFEFF_FMS_OK;
}

// ===========================================================================
// MKGTR stage: gg.bin + phase.bin + global.inp -> fms.bin, gtr.dat, log3.dat
// ===========================================================================
namespace {

// PAD encoding of one value in `npack` characters (pad.rs:33-93): base-90
// digits offset by 37, a decimal exponent byte and a sign folded into the
// second byte, round-half-up in the last digit.
std::string pad_encode(double value, int npack) {
  const double huge = powi_squaring(10.0, 38), tiny = 1.0 / huge;
  std::string out(size_t(npack), ' ');
  const double xsave = value < -huge ? -huge : (value > huge ? huge : value);
  const int isgn = xsave > 0.0 ? 1 : 0;
  double xwork = std::fabs(xsave);
  int iexp = 0;
  if (xwork < huge && xwork > tiny) iexp = 1 + int(std::log(xwork) / 2.3025850929940455);
  else if (xwork >= huge) { iexp = 38; xwork = 1.0; }
  else if (xwork <= tiny) xwork = 0.0;
  xwork /= powi_squaring(10.0, iexp);
  do {
    if (xwork >= 1.0) { xwork *= 0.1; ++iexp; }
    else if (xwork <= 0.099999999994) { xwork *= 10.0; --iexp; }
  } while (xwork >= 1.0);
  int itmp = int(double(kPadHalf) * xwork);
  out[0] = char(iexp + kPadOff + kPadHalf);
  out[1] = char(2 * itmp + isgn + kPadOff);
  xwork = xwork * double(kPadHalf) - double(itmp);
  for (int i = 2; i < npack; ++i) {
    itmp = int(double(kPadBase) * xwork + 1.0e-9);
    out[size_t(i)] = char(itmp + kPadOff);
    xwork = xwork * double(kPadBase) - double(itmp);
  }
  if (xwork >= 0.5) {
    const int up = itmp + kPadOff + 1;
    if (up <= 126) out[size_t(npack) - 1] = char(up);
    else if (static_cast<unsigned char>(out[size_t(npack) - 2]) < 126) {
      out[size_t(npack) - 2] = char(static_cast<unsigned char>(out[size_t(npack) - 2]) + 1);
      out[size_t(npack) - 1] = char(37);
    }
  }
  return out;
}

// '$' lines of complex PAD pairs, flushed once the payload reaches 82 - 2 npack + 1 (pad.rs:142-161).
std::string pad_complex_lines(const refeff_complex128* v, size_t n, int npack) {
  std::string out, payload;
  const size_t maxp = size_t(82 - 2 * npack + 1);
  for (size_t i = 0; i < n; ++i) {
    payload += pad_encode(v[i].re, npack);
    payload += pad_encode(v[i].im, npack);
    if (payload.size() >= maxp || i + 1 == n) {
      out += '$';
      out += payload;
      out += '\n';
      payload.clear();
    }
  }
  return out;
}

struct GlobalInp {
  int ipol = 0, ispin = 0, le2 = 0, do_nrixs = 0;
  double elpty = 0.0, angks = 0.0;
  double ptz[3][6] = {};
};

// global.inp control line and polarization tensor (global_input.rs:314-345).
int parse_global_inp(const std::string& path, GlobalInp& g, std::string& err) {
  std::string text;
  if (!read_file(path, text)) { err = "cannot read " + path; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  const auto L = split_lines(text);
  bool ctl = false, pol = false;
  for (size_t i = 0; i + 1 < L.size(); ++i) {
    const std::string h = trim(L[i]);
    if (!ctl && h == "ipol, ispin, le2, elpty, angks, l2lp, do_nrixs, ldecmx, lj") {
      const auto fs = fields(L[i + 1]);
      double x[7];
      if (fs.size() < 7) { err = "global.inp: short control line"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
      for (int k = 0; k < 7; ++k)
        if (!parse_double(fs[size_t(k)], x[k])) { err = "global.inp: bad control value"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
      g.ipol = int(x[0]); g.ispin = int(x[1]); g.le2 = int(x[2]); g.elpty = x[3]; g.angks = x[4]; g.do_nrixs = int(x[6]);
      ctl = true;
    } else if (!pol && h == "polarization tensor") {
      if (i + 3 >= L.size()) { err = "global.inp: polarization tensor truncated"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
      for (int r = 0; r < 3; ++r) {
        const auto fs = fields(L[i + 1 + size_t(r)]);
        if (fs.size() < 6) { err = "global.inp: short polarization row"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
        for (int c = 0; c < 6; ++c)
          if (!parse_double(fs[size_t(c)], g.ptz[r][c])) { err = "global.inp: bad polarization value"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
      }
      pol = true;
    }
  }
  if (!ctl || !pol) { err = "global.inp: control line or polarization tensor missing"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  return REFEFF_FMS_OK;
}

// gg.bin / gg.dat sections (gg_dat.rs:92-150): '#' header lines, '#DT#' sizes,
// then rows of (re, im) pairs.
int parse_gg_sections(const std::string& path, int& dim, std::vector<refeff_complex128>& vals, int& count,
                      std::string& err) {
  std::string text;
  if (!read_file(path, text)) { err = "cannot read " + path; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  const auto L = split_lines(text);
  dim = -1;
  count = 0;
  vals.clear();
  int rows = 0, cols = 0, got = 0;
  bool open = false;
  for (const auto& line : L) {
    const std::string t = trim(line);
    if (t.empty()) continue;
    if (t[0] == '#') {
      if (t.compare(0, 4, "#SN#") == 0) {
        if (open && got != rows) { err = "gg section ended early"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
        open = true; rows = cols = got = 0;
        ++count;
      } else if (t.compare(0, 4, "#DT#") == 0) {
        const auto fs = fields(t);
        long long r = 0, c = 0;
        if (fs.size() < 2 || !parse_int(fs[fs.size() - 2], r) || !parse_int(fs[fs.size() - 1], c) || r <= 0 || r != c) {
          err = "gg sections must be nonempty square matrices";
          return REFEFF_FMS_ERR_INVALID_ARGUMENT;
        }
        rows = int(r); cols = int(c);
        if (dim < 0) dim = rows;
        if (dim != rows) { err = "gg section shapes differ"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
        vals.resize(size_t(count) * dim * dim);
      }
      continue;
    }
    if (!open || rows == 0 || got >= rows) { err = "gg data row outside a section"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
    const auto fs = fields(t);
    if (fs.size() != size_t(2 * cols)) { err = "gg row has the wrong number of values"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
    refeff_complex128* sec = vals.data() + size_t(count - 1) * dim * dim;
    for (int c = 0; c < cols; ++c) {
      refeff_complex128 v;
      if (!parse_double(fs[size_t(2 * c)], v.re) || !parse_double(fs[size_t(2 * c + 1)], v.im)) {
        err = "bad gg value";
        return REFEFF_FMS_ERR_INVALID_ARGUMENT;
      }
      sec[size_t(got) + size_t(dim) * c] = v;
    }
    ++got;
  }
  if (count == 0 || dim <= 0 || got != rows) { err = "gg file holds no complete section"; return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  return REFEFF_FMS_OK;
}

// core_hole_quantum_numbers (crates/refeff-core/src/core_hole.rs:66-83): FEFF hole index -> kappa.
bool core_hole_kappa(int ihole, int& kappa) {
  switch (ihole) {
    case 1: case 2: case 5: case 10: case 17: case 24: case 29: kappa = -1; return true;
    case 3: case 6: case 11: case 18: case 25: case 30: kappa = 1; return true;
    case 4: case 7: case 12: case 19: case 26: kappa = -2; return true;
    case 8: case 13: case 20: case 27: kappa = 2; return true;
    case 9: case 14: case 21: case 28: kappa = -3; return true;
    case 15: case 22: kappa = 3; return true;
    case 16: case 23: kappa = -4; return true;
    default: return false;
  }
}

bool file_exists(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  return bool(f);
}

}  // namespace

extern "C" int refeff_fms_write_fms_bin(const char* path, double cluster_radius, int ne, int ne1, int ne3, int nph,
                                        int pad_width, int n_spectra, const refeff_complex128* traces) {
  if (!path || ne < 0 || ne1 < 0 || ne3 < 0 || nph < 0 || pad_width <= 2 || pad_width > 40 || n_spectra < 0 ||
      (n_spectra > 0 && ne > 0 && !traces))
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  // fms_bin_string (fms_bin.rs:77-98): title, six counts in I7 (nip declared 0), one PAD block per spectrum
  char buf[256];
  std::snprintf(buf, sizeof buf, "FMS rfms=%7.4f\n", cluster_radius);
  std::string out = buf;
  const long long counts[6] = {ne, ne1, ne3, nph, pad_width, 0};
  for (long long c : counts) {
    std::snprintf(buf, sizeof buf, " %7lld", c);
    out += buf;
  }
  out += '\n';
  for (int sp = 0; sp < n_spectra; ++sp) {
    std::vector<refeff_complex128> row(static_cast<size_t>(ne));
    for (int e = 0; e < ne; ++e) row[size_t(e)] = traces[size_t(sp) + size_t(n_spectra) * e];
    out += pad_complex_lines(row.data(), row.size(), pad_width);
  }
  return write_file_atomic(path, out) ? REFEFF_FMS_OK : REFEFF_FMS_ERR_INVALID_ARGUMENT;
}

extern "C" int refeff_fms_write_gtr_dat(const char* path, int ne, const refeff_complex128* energy,
                                        const refeff_complex128* trace) {
  if (!path || ne < 0 || (ne > 0 && (!energy || !trace))) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  // gtr_dat_string (gtr_dat.rs:60-71): four F13.6 fields per energy
  std::string out;
  char buf[128];
  for (int e = 0; e < ne; ++e) {
    std::snprintf(buf, sizeof buf, "%13.6f%13.6f%13.6f%13.6f\n", energy[e].re, energy[e].im, trace[e].re, trace[e].im);
    out += buf;
  }
  return write_file_atomic(path, out) ? REFEFF_FMS_OK : REFEFF_FMS_ERR_INVALID_ARGUMENT;
}

extern "C" int refeff_fms_run_mkgtr_dir(refeff_fms_context* ctx, const char* work_dir, int* written) {
  if (!ctx || !work_dir) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  if (written) *written = 0;
  const std::string dir = std::string(work_dir) + "/";
  std::string err;
  FmsInp fi;
  int rc = parse_fms_inp(dir + "fms.inp", fi, err);
  if (rc) { set_error(ctx, err); return rc; }
  if (fi.mfms == 0) return REFEFF_FMS_OK;  // fms_enabled (fms.rs:633-635)
  const std::string gg_path = file_exists(dir + "gg.bin") ? dir + "gg.bin" : dir + "gg.dat";
  if (!file_exists(gg_path)) { set_error(ctx, "MKGTR requires gg.bin or gg.dat from the FMS stage"); return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
  if (!file_exists(dir + "phase.bin") || !file_exists(dir + "global.inp")) return REFEFF_FMS_OK;
  GlobalInp gi;
  rc = parse_global_inp(dir + "global.inp", gi, err);
  if (rc) { set_error(ctx, err); return rc; }
  if (gi.do_nrixs == 1) { set_error(ctx, "NRIXS (JAS) MKGTR projections are not supported"); return REFEFF_FMS_ERR_UNSUPPORTED; }
  if (file_exists(dir + "eels.inp")) { set_error(ctx, "EELS MKGTR projections are not supported"); return REFEFF_FMS_ERR_UNSUPPORTED; }
  int produced = 0;
  if (!file_exists(dir + "fms.bin") || !file_exists(dir + "gtr.dat")) {
    PhaseBin pb;
    rc = read_phase_bin(dir + "phase.bin", pb, err);
    if (rc) { set_error(ctx, err); return rc; }
    int dim = 0, count = 0;
    std::vector<refeff_complex128> gg;
    rc = parse_gg_sections(gg_path, dim, gg, count, err);
    if (rc) { set_error(ctx, err); return rc; }
    if (count != pb.ne) { set_error(ctx, "gg section count does not match the phase.bin energy count"); return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
    // green_functions_from_gg (fms.rs:5883-5918): the cached values narrowed to complex64
    for (auto& v : gg) {
      const float re = float(v.re), im = float(v.im);
      if (!std::isfinite(v.re) || !std::isfinite(v.im) || !std::isfinite(re) || !std::isfinite(im)) {
        set_error(ctx, "non-finite gg value");
        return REFEFF_FMS_ERR_NONFINITE_INPUT;
      }
      v = {double(re), double(im)};
    }
    if (fi.lmaxph.empty() || fi.lmaxph[0] < 0) { set_error(ctx, "fms.inp lmaxph(0) must be nonnegative"); return REFEFF_FMS_ERR_INVALID_ANGULAR_LIMIT; }
    const int lmax = fi.lmaxph[0];
    const int active = (gi.ispin == 1 || gi.ispin == -1) ? pb.nsp : 1;  // active_spin_channels (fms.rs:5860-5869)
    int kappa = 0;
    if (!core_hole_kappa(pb.ihole, kappa)) { set_error(ctx, "phase.bin ihole has no core-hole kappa"); return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
    if (pb.ntrans < 8) { set_error(ctx, "phase.bin carries fewer than 8 transition moments"); return REFEFF_FMS_ERR_INVALID_ARGUMENT; }
    refeff_complex128 ptz[9];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) ptz[3 * r + c] = {gi.ptz[r][2 * c], gi.ptz[r][2 * c + 1]};
    const int nm = 2 * lmax + 1;
    std::vector<refeff_complex128> bmat(size_t(nm) * 2 * 8 * nm * 2 * 8);
    int32_t lind[8], kiind[8];
    rc = rfx::mkgtr_transition_matrix(lmax, kappa, gi.ipol, ptz, gi.le2, 0, gi.ispin, pb.nsp, gi.angks, bmat.data(),
                                      lind, kiind);
    if (rc) { set_error(ctx, "transition matrix"); return rc; }
    // rkk (energy, transition, spin) with the first 8 transitions
    std::vector<refeff_complex128> rkk(size_t(pb.ne) * 8 * pb.nsp);
    for (int sp = 0; sp < pb.nsp; ++sp)
      for (int k = 0; k < 8; ++k)
        for (int e = 0; e < pb.ne; ++e)
          rkk[size_t(e) + size_t(pb.ne) * (size_t(k) + 8 * size_t(sp))] =
              pb.rkk[size_t(e) + size_t(pb.ne) * (size_t(k) + size_t(pb.ntrans) * sp)];
    std::vector<refeff_complex128> traces(size_t(pb.ne));
    rc = refeff_fms_mkgtr_trace(ctx, pb.ne, dim, active, lmax, 1, lind, bmat.data(), gg.data(), rkk.data(), pb.nsp,
                                traces.data());
    if (rc) return rc;
    if (refeff_fms_write_fms_bin((dir + "fms.bin").c_str(), fi.rfms2, pb.ne, pb.ne1, pb.ne3, pb.npot - 1, pb.npad, 1,
                                 traces.data()) != REFEFF_FMS_OK ||
        refeff_fms_write_gtr_dat((dir + "gtr.dat").c_str(), pb.ne, pb.em.data(), traces.data()) != REFEFF_FMS_OK) {
      set_error(ctx, "cannot write fms.bin / gtr.dat");
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    }
    produced = 2;
  }
  // ensure_mkgtr_module_log (fms.rs:5941-5963)
  std::string log;
  if (!read_file(dir + "log3.dat", log))
    log = "FMS calculation of full Green's function ...\nFEFF-serial using 1 thread.\nDone with module: FMS.\n";
  if (log.find("Done with module: MKGTR.") == std::string::npos) {
    log += "\nMKGTR: Tracing over Green's function ...\nDone with module: MKGTR.\n";
    if (!write_file_atomic(dir + "log3.dat", log)) {
      set_error(ctx, "cannot write log3.dat");
      return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    }
  }
  if (written) *written = produced;
  return REFEFF_FMS_OK;
}
