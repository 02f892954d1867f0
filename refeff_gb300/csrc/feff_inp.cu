// The cluster from feff.inp: the ATOMS table read through FEFF's line rules,
// turned into the absorber-centred geometry rows that FEFF's rdinp writes to
// geom.dat and the FMS stage reads back.
//
// Reference interfaces replaced here:
//   FEFF input lines (comments, inline comments, BWORDS fields, cards, block
//     sections, INCLUDE / LOAD, END)      crates/refeff-io/src/input.rs:64-372
//   parse_atoms / parse_potentials       crates/refeff-io/src/model.rs:626-676
//   RMULTIPLIER scaling of the atoms     crates/refeff-io/src/model.rs:148, 198-207
//   geometry_rows, the strict selection sort on the fused distance, and
//   geometry_model_atoms                 crates/refeff-io/src/rdinp/geometry.rs:18-119
//   write_geom_dat                       crates/refeff-io/src/rdinp/structure.rs:57-81
//
// Inputs that build the cluster another way (LATTICE / CIF expansion,
// OVERLAP shells, the NRIXS frame rotation) are reported as unsupported.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/refeff_fms.h"

namespace {

struct Line {
  bool card = false;
  std::string keyword;              // card: canonical upper-case keyword
  std::string section;              // data row: its block card
  std::vector<std::string> fields;  // card: arguments; data row: all fields
  int line = 0;
  std::string path;
};

struct InpError {
  int code;
  std::string msg;
};

std::string upper(std::string s) {
  for (auto& c : s) c = char(std::toupper(static_cast<unsigned char>(c)));
  return s;
}

std::string lower(std::string s) {
  for (auto& c : s) c = char(std::tolower(static_cast<unsigned char>(c)));
  return s;
}

bool is_block_card(const std::string& k) {
  static const char* blocks[] = {"ATOMS", "POTENTIALS", "OVERLAP", "LATTICE", "EGRID", "DENSITY", "CONFIG",
                                 "STRETCHES", "ANGLES", "ELNES", "EXELFS", "NRIXS", "MDFF"};
  for (const char* b : blocks)
    if (k == b) return true;
  return false;
}

std::string canonical_keyword(const std::string& k) {
  const std::string t = k.substr(0, 4);
  static const char* map[][2] = {{"ATOM", "ATOMS"}, {"CONF", "CONFIG"},   {"DENS", "DENSITY"}, {"ELNE", "ELNES"},
                                 {"EXEL", "EXELFS"}, {"EGRI", "EGRID"},    {"LATT", "LATTICE"}, {"MDFF", "MDFF"},
                                 {"NRIX", "NRIXS"},  {"OVER", "OVERLAP"},  {"POTE", "POTENTIALS"},
                                 {"TITL", "TITLE"}};
  for (auto& m : map)
    if (t == m[0]) return m[1];
  return k;
}

// Inline comment markers ! # % end the line outside [ ] { } " " ' ' ( ).
std::string strip_inline_comment(const std::string& s) {
  const char open[] = {'[', '{', '"', '\'', '('};
  const char close[] = {']', '}', '"', '\'', ')'};
  int prot = -1;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (prot >= 0) {
      if (c == close[prot]) prot = -1;
      continue;
    }
    bool opened = false;
    for (int q = 0; q < 5; ++q)
      if (c == open[q]) { prot = q; opened = true; break; }
    if (opened) continue;
    if (c == '!' || c == '#' || c == '%') return s.substr(0, i);
  }
  return s;
}

// BWORDS: blanks separate words; a comma ends a word, and a comma with no word
// since the last separator stands for an empty field.
std::vector<std::string> bwords(const std::string& s) {
  std::vector<std::string> w;
  long start = -1;
  bool comma = true;
  for (size_t i = 0; i < s.size(); ++i) {
    const char c = s[i];
    if (c == ' ' || c == '\t') {
      if (start >= 0) {
        w.push_back(s.substr(size_t(start), i - size_t(start)));
        start = -1;
        comma = false;
      }
    } else if (c == ',') {
      if (start >= 0) {
        w.push_back(s.substr(size_t(start), i - size_t(start)));
        start = -1;
      } else if (comma) {
        w.emplace_back();
      }
      comma = true;
    } else if (start < 0) {
      start = long(i);
    }
  }
  if (start >= 0) {
    std::string last = s.substr(size_t(start));
    while (!last.empty() && std::isspace(static_cast<unsigned char>(last.back()))) last.pop_back();
    w.push_back(last);
  }
  return w;
}

std::string strip_delimiters(const std::string& v) {
  const char pairs[][2] = {{'"', '"'}, {'\'', '\''}, {'{', '}'}, {'(', ')'}, {'<', '>'}, {'[', ']'}};
  for (auto& p : pairs)
    if (v.size() >= 2 && v.front() == p[0] && v.back() == p[1]) return v.substr(1, v.size() - 2);
  return v;
}

std::string dir_of(const std::string& path) {
  const size_t k = path.find_last_of('/');
  return k == std::string::npos ? std::string(".") : path.substr(0, k);
}

// One file's logical lines (input.rs parse_logical_lines); `stop` is set at END.
void logical_lines(const std::string& path, const std::string& text, std::vector<Line>& out, bool& stop) {
  std::string active;
  std::istringstream in(text);
  std::string raw;
  int no = 0;
  while (std::getline(in, raw)) {
    ++no;
    if (!raw.empty() && raw.back() == '\r') raw.pop_back();
    for (auto& c : raw)
      if (c == '\t') c = ' ';
    size_t a = 0;
    while (a < raw.size() && std::isspace(static_cast<unsigned char>(raw[a]))) ++a;
    const std::string trimmed = raw.substr(a);
    if (trimmed.empty()) continue;
    const char c0 = trimmed[0];
    if (c0 == ';' || c0 == '*' || c0 == '%' || c0 == '#') continue;
    std::string un = strip_inline_comment(trimmed);
    size_t b = 0, e = un.size();
    while (b < e && std::isspace(static_cast<unsigned char>(un[b]))) ++b;
    while (e > b && std::isspace(static_cast<unsigned char>(un[e - 1]))) --e;
    un = un.substr(b, e - b);
    if (un.empty()) continue;
    const std::vector<std::string> tok = bwords(un);
    if (tok.empty()) continue;
    const std::string first = tok[0];
    const std::string lf = lower(first);
    const bool egrid_payload =
        active == "EGRID" && (lf == "e_grid" || lf == "k_grid" || lf == "exp_grid" || lf == "user_grid");
    const bool density_payload = active == "DENSITY" && (lf == "line" || lf == "plane" || lf == "volume");
    const bool is_card = !egrid_payload && !density_payload && !first.empty() &&
                         std::isalpha(static_cast<unsigned char>(first[0]));
    Line L;
    L.line = no;
    L.path = path;
    if (is_card) {
      L.card = true;
      L.keyword = canonical_keyword(upper(first));
      L.fields.assign(tok.begin() + 1, tok.end());
      if (L.keyword == "END") {
        out.push_back(L);
        stop = true;
        return;
      }
      if (is_block_card(L.keyword)) active = L.keyword;
      else if (L.keyword != "TITLE") active.clear();
    } else if (!active.empty()) {
      L.section = active;
      L.fields = tok;
    } else {
      throw InpError{REFEFF_FMS_ERR_INVALID_ARGUMENT,
                     path + ":" + std::to_string(no) + ": data row found outside a block card"};
    }
    out.push_back(L);
  }
}

// Reader::read_file: INCLUDE / LOAD expanded relative to the including file,
// at most 10 levels, no file included inside itself.
void read_file(const std::string& path, int depth, std::set<std::string>& open_files, std::vector<Line>& out,
               bool& stop) {
  if (depth >= 10) throw InpError{REFEFF_FMS_ERR_INVALID_ARGUMENT, path + ": include depth exceeded"};
  char* rp = realpath(path.c_str(), nullptr);
  const std::string canon = rp ? std::string(rp) : path;
  std::free(rp);
  if (!open_files.insert(canon).second) throw InpError{REFEFF_FMS_ERR_INVALID_ARGUMENT, canon + ": recursive include"};
  std::ifstream f(path, std::ios::binary);
  if (!f) throw InpError{REFEFF_FMS_ERR_INVALID_ARGUMENT, "cannot read " + path};
  std::stringstream ss;
  ss << f.rdbuf();
  std::vector<Line> lines;
  bool local_stop = false;
  logical_lines(path, ss.str(), lines, local_stop);
  for (auto& L : lines) {
    if (L.card && (L.keyword == "INCLUDE" || L.keyword == "LOAD")) {
      if (L.fields.empty())
        throw InpError{REFEFF_FMS_ERR_INVALID_ARGUMENT, path + ": " + L.keyword + " requires a file name"};
      read_file(dir_of(path) + "/" + strip_delimiters(L.fields[0]), depth + 1, open_files, out, stop);
      continue;
    }
    out.push_back(L);
  }
  open_files.erase(canon);
  if (local_stop) stop = true;
}

// parse_f64 (model/parse.rs): Fortran D exponents accepted; the whole field must parse.
bool parse_f64(const std::string& v, double& out) {
  std::string s = v;
  for (auto& c : s)
    if (c == 'D' || c == 'd') c = 'E';
  if (s.empty()) return false;
  if (s == "inf" || s == "+inf" || s == "-inf" || s == "infinity" || s == "NaN" || s == "nan") {
    out = std::strtod(s.c_str(), nullptr);
    return true;
  }
  for (char c : s)
    if (!(std::isdigit(static_cast<unsigned char>(c)) || c == '.' || c == 'e' || c == 'E' || c == '+' || c == '-'))
      return false;
  char* end = nullptr;
  out = std::strtod(s.c_str(), &end);
  return end && *end == '\0';
}

bool parse_i32(const std::string& v, int& out) {
  if (v.empty()) return false;
  size_t i = (v[0] == '+' || v[0] == '-') ? 1 : 0;
  if (i == v.size()) return false;
  for (size_t j = i; j < v.size(); ++j)
    if (!std::isdigit(static_cast<unsigned char>(v[j]))) return false;
  const long long x = std::strtoll(v.c_str(), nullptr, 10);
  if (x < -2147483648LL || x > 2147483647LL) return false;
  out = int(x);
  return true;
}

std::vector<std::string> before_star(const std::vector<std::string>& f) {
  std::vector<std::string> out;
  for (const auto& x : f) {
    if (x == "*") break;
    out.push_back(x);
  }
  return out;
}

// card_by_feff_name for the cards read here (model/cards.rs:68-93).
bool card_named(const Line& L, const char* canonical) {
  if (!L.card) return false;
  if (L.keyword == canonical) return true;
  const std::string t = L.keyword.substr(0, 4);
  const std::string c = canonical;
  if (c == "RMULT") return t == "RMUL";
  if (c == "CIF") return t == "CIF";
  return false;
}

struct Row {
  double x, y, z;
  int ipot;
  double d2;
};

struct Geometry {
  std::vector<Row> rows;
  std::vector<int> model_atoms;  // iatph, one-based rows; [0] = 1
};

Geometry geometry_from_feff_inp(const std::string& path) {
  std::vector<Line> lines;
  std::set<std::string> open_files;
  bool stop = false;
  read_file(path, 0, open_files, lines, stop);
  double rmult = 1.0;
  bool have_rmult = false;
  struct Atom {
    double x, y, z;
    int ipot;
  };
  std::vector<Atom> atoms;
  std::vector<int> pot_ids;
  for (const auto& L : lines) {
    if (L.card) {
      if (L.keyword == "LATTICE" || card_named(L, "CIF") || L.keyword == "OVERLAP" || L.keyword == "NRIXS")
        throw InpError{REFEFF_FMS_ERR_UNSUPPORTED,
                       L.keyword + ": only clusters given row by row in ATOMS are read here"};
      if (!have_rmult && card_named(L, "RMULT")) {
        if (L.fields.empty() || !parse_f64(L.fields[0], rmult))
          throw InpError{REFEFF_FMS_ERR_INVALID_ARGUMENT, path + ": RMULTIPLIER requires a numeric value"};
        have_rmult = true;
      }
      continue;
    }
    const auto f = before_star(L.fields);
    const std::string where = L.path + ":" + std::to_string(L.line);
    if (L.section == "ATOMS") {
      Atom a;
      if (f.size() < 4) throw InpError{REFEFF_FMS_ERR_INVALID_ARGUMENT, where + ": ATOMS rows require x y z ipot"};
      if (!parse_f64(f[0], a.x) || !parse_f64(f[1], a.y) || !parse_f64(f[2], a.z) || !parse_i32(f[3], a.ipot))
        throw InpError{REFEFF_FMS_ERR_INVALID_ARGUMENT, where + ": bad ATOMS row"};
      atoms.push_back(a);
    } else if (L.section == "POTENTIALS") {
      int ip = 0, z = 0;
      if (f.size() < 2 || !parse_i32(f[1], z) || !parse_i32(f[0], ip))
        throw InpError{REFEFF_FMS_ERR_INVALID_ARGUMENT, where + ": POTENTIALS rows require ipot and Z"};
      pot_ids.push_back(ip);
    }
  }
  if (atoms.empty()) throw InpError{REFEFF_FMS_ERR_EMPTY_CLUSTER, path + ": ATOMS is empty"};
  for (auto& a : atoms) {
    a.x *= rmult;
    a.y *= rmult;
    a.z *= rmult;
  }
  // geometry_rows: the absorber is the first atom of potential 0 (else the first atom), at the origin
  size_t abs_i = 0;
  for (size_t i = 0; i < atoms.size(); ++i)
    if (atoms[i].ipot == 0) { abs_i = i; break; }
  Geometry g;
  g.rows.push_back({0.0, 0.0, 0.0, 0, 0.0});
  const Atom& c = atoms[abs_i];
  for (size_t i = 0; i < atoms.size(); ++i) {
    if (i == abs_i) continue;
    const double x = atoms[i].x - c.x, y = atoms[i].y - c.y, z = atoms[i].z - c.z;
    // the fused distance of FEFF's optimised ffsort: z*z + (x*x + y*y) with two fused multiply-adds
    const double d2 = std::fma(z, z, std::fma(x, x, y * y));
    if (d2 > 0.0) g.rows.push_back({x, y, z, atoms[i].ipot, d2});
  }
  // strict less-than selection sort (ties keep FEFF's swap order, not a stable order)
  for (size_t i = 0; i + 1 < g.rows.size(); ++i) {
    size_t mi = i;
    double md = g.rows[i].d2;
    for (size_t j = i + 1; j < g.rows.size(); ++j)
      if (g.rows[j].d2 < md) { md = g.rows[j].d2; mi = j; }
    if (mi != i) std::swap(g.rows[i], g.rows[mi]);
  }
  // geometry_model_atoms
  int maxp = -1;
  for (int p : pot_ids) maxp = std::max(maxp, std::max(p, 0));
  if (pot_ids.empty())
    for (const auto& r : g.rows) maxp = std::max(maxp, std::max(r.ipot, 0));
  if (maxp < 0) maxp = 0;
  g.model_atoms.assign(size_t(maxp) + 1, 0);
  g.model_atoms[0] = 1;
  for (int iph = 1; iph <= maxp; ++iph)
    for (size_t r = 0; r < g.rows.size(); ++r)
      if (g.rows[r].ipot == iph) { g.model_atoms[size_t(iph)] = int(r) + 1; break; }
  while (g.model_atoms.size() > 1 && g.model_atoms.back() == 0) g.model_atoms.pop_back();
  return g;
}

std::string geom_dat_text(const Geometry& g) {
  std::string out;
  char buf[128];
  std::snprintf(buf, sizeof buf, "nat, nph = %5zu%5zu\n", g.rows.size(), g.model_atoms.size() - 1);
  out += buf;
  for (int m : g.model_atoms) {
    std::snprintf(buf, sizeof buf, "%5d", m);
    out += buf;
  }
  out += "\n iat     x       y        z       iph  \n ";
  out += std::string(71, '-');
  out += "\n";
  for (size_t i = 0; i < g.rows.size(); ++i) {
    const Row& r = g.rows[i];
    std::snprintf(buf, sizeof buf, "%4zu%13.5f%13.5f%13.5f%4d%4d\n", i + 1, r.x, r.y, r.z, r.ipot, 1);
    out += buf;
  }
  return out;
}

thread_local std::string g_last_inp_error;

}  // namespace

namespace rfx {
// geom.dat text for the cluster of a feff.inp (used by the work-directory seam
// when a work directory holds feff.inp but no geom.dat).
int geom_dat_from_feff_inp(const std::string& path, std::string& text, std::string& err) {
  try {
    text = geom_dat_text(geometry_from_feff_inp(path));
    return REFEFF_FMS_OK;
  } catch (const InpError& e) {
    err = e.msg;
    return e.code;
  }
}
}  // namespace rfx

extern "C" int refeff_fms_geometry_from_feff_inp(const char* feff_inp_path, int row_capacity, double* xyz_out,
                                                 int32_t* ipot_out, int32_t* n_rows, int model_capacity,
                                                 int32_t* model_atoms_out, int32_t* n_model) {
  if (!feff_inp_path || !n_rows || !n_model || row_capacity < 0 || model_capacity < 0)
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  try {
    const Geometry g = geometry_from_feff_inp(feff_inp_path);
    *n_rows = int32_t(g.rows.size());
    *n_model = int32_t(g.model_atoms.size());
    if (int(g.rows.size()) > row_capacity || int(g.model_atoms.size()) > model_capacity)
      return row_capacity == 0 && model_capacity == 0 ? REFEFF_FMS_OK : REFEFF_FMS_ERR_INVALID_ARGUMENT;
    if (!xyz_out || !ipot_out || !model_atoms_out) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < g.rows.size(); ++i) {
      xyz_out[3 * i] = g.rows[i].x;
      xyz_out[3 * i + 1] = g.rows[i].y;
      xyz_out[3 * i + 2] = g.rows[i].z;
      ipot_out[i] = g.rows[i].ipot;
    }
    for (size_t i = 0; i < g.model_atoms.size(); ++i) model_atoms_out[i] = g.model_atoms[i];
    g_last_inp_error.clear();
    return REFEFF_FMS_OK;
  } catch (const InpError& e) {
    g_last_inp_error = e.msg;
    return e.code;
  }
}

extern "C" int refeff_fms_write_geom_dat(const char* feff_inp_path, const char* geom_dat_path) {
  if (!feff_inp_path || !geom_dat_path) return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  std::string text, err;
  const int rc = rfx::geom_dat_from_feff_inp(feff_inp_path, text, err);
  if (rc) {
    g_last_inp_error = err;
    return rc;
  }
  std::ofstream f(geom_dat_path, std::ios::binary);
  if (!f) {
    g_last_inp_error = std::string("cannot write ") + geom_dat_path;
    return REFEFF_FMS_ERR_INVALID_ARGUMENT;
  }
  f << text;
  g_last_inp_error.clear();
  return f ? REFEFF_FMS_OK : REFEFF_FMS_ERR_INVALID_ARGUMENT;
}

extern "C" const char* refeff_fms_feff_inp_last_error(void) { return g_last_inp_error.c_str(); }
