// inca_gpu: command-line driver with the reference program's interface (src/inca_main.f90),
// running the intracule path through libinca_gpu.so.
//
//   inca_gpu input.inp
//
// Reads the same namelist input (&files, &intracule_job, &cube_job; read_all_input,
// src/mod_input_reader.f90:29-180), the .fchk and .bas files (filefchk / filebas,
// src/mod_read_files.f90:432-726), sets up the integration centres (setup_grids,
// src/mod_input_reader.f90:185-221) and writes the .out report, the .rad table, the vector
// .cube and the _smearing.dat file in the reference's layout (src/mod_intracule.f90:410-568).
//
// Two optional keys extend &intracule_job (a reference input never needs them):
//   precision = 'fp64' | 'mixed'   (default 'mixed')
//   tolerance = 1d-10              (relative tolerance of the mixed form)
// Errors print a message and exit with status 1, as the reference's stop 1.
#include <algorithm>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "inca_gpu.h"

namespace {

[[noreturn]] void die(const std::string& msg) {
  std::printf(" ERROR: %s\n", msg.c_str());
  std::exit(1);
}

std::string lower(std::string s) {
  for (char& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  return s;
}

// ------------------------------------------------------------------ namelist input
struct Value {
  std::vector<std::string> items;  // raw tokens (strings unquoted)
};
using Group = std::map<std::string, std::map<int, std::string>>;  // key -> index(1-based) -> token

// Tokenise a namelist group body: key[(idx)] = v1, v2, ... separated by commas/whitespace.
Group parse_group(const std::string& text, const std::string& name, bool* found) {
  Group g;
  *found = false;
  std::string low = lower(text);
  size_t pos = 0;
  while (true) {
    pos = low.find("&" + name, pos);
    if (pos == std::string::npos) return g;
    const size_t after = pos + 1 + name.size();
    if (after < low.size() && (std::isalnum(static_cast<unsigned char>(low[after])) || low[after] == '_')) {
      pos = after;
      continue;
    }
    pos = after;
    break;
  }
  *found = true;
  // body up to the terminating '/' outside quotes
  std::string body;
  char q = 0;
  for (size_t i = pos; i < text.size(); ++i) {
    const char ch = text[i];
    if (q) {
      if (ch == q) q = 0;
      body += ch;
      continue;
    }
    if (ch == '\'' || ch == '"') {
      q = ch;
      body += ch;
      continue;
    }
    if (ch == '/') break;
    if (ch == '!') {  // comment to end of line
      while (i < text.size() && text[i] != '\n') ++i;
      body += ' ';
      continue;
    }
    body += ch;
  }
  // split into tokens: identifiers with optional (i), '=', values
  std::vector<std::string> tok;
  std::string cur;
  q = 0;
  auto flush = [&]() {
    if (!cur.empty()) tok.push_back(cur);
    cur.clear();
  };
  for (size_t i = 0; i < body.size(); ++i) {
    const char ch = body[i];
    if (q) {
      cur += ch;
      if (ch == q) {
        q = 0;
        flush();
      }
      continue;
    }
    if (ch == '\'' || ch == '"') {
      flush();
      q = ch;
      cur += ch;
      continue;
    }
    if (ch == '=') {
      flush();
      tok.push_back("=");
      continue;
    }
    if (ch == ',' || std::isspace(static_cast<unsigned char>(ch))) {
      flush();
      continue;
    }
    cur += ch;
  }
  flush();
  std::string key;
  int idx = 1;
  for (size_t i = 0; i < tok.size(); ++i) {
    if (i + 1 < tok.size() && tok[i + 1] == "=") {
      std::string k = lower(tok[i]);
      idx = 1;
      const size_t par = k.find('(');
      if (par != std::string::npos) {
        idx = std::atoi(k.c_str() + par + 1);
        k = k.substr(0, par);
      }
      key = k;
      ++i;  // skip '='
      continue;
    }
    if (key.empty()) die("Syntax error in &" + name + " block of the input file.");
    std::string v = tok[i];
    if (!v.empty() && (v[0] == '\'' || v[0] == '"')) v = v.substr(1, v.size() - 2);
    g[key][idx++] = v;
  }
  return g;
}

double to_double(const std::string& s) {
  std::string t = s;
  for (char& ch : t)
    if (ch == 'd' || ch == 'D') ch = 'e';
  char* end = nullptr;
  const double v = std::strtod(t.c_str(), &end);
  if (end == t.c_str()) die("bad real value '" + s + "' in the input file");
  return v;
}

bool to_bool(const std::string& s) {
  std::string t = lower(s);
  if (!t.empty() && t[0] == '.') t = t.substr(1);
  if (t.empty()) die("bad logical value in the input file");
  if (t[0] == 't') return true;
  if (t[0] == 'f') return false;
  die("bad logical value '" + s + "' in the input file");
}

struct Input {
  // &files
  std::string fchk, bas, wfx, log, dm2, outname, cubename, radname;
  // &intracule_job
  std::string calc_type;
  bool radial_integral = false, radial_plot = false, cubeintra = false;
  bool zero = false, two_points = false, c1calc = false;
  double thresh = 1e-8;
  bool nosym = false, nohydro = true, multicenter = true, manual_grid = false, betaone = false;
  int nrad = 50, nang = 590, nblock = 1;
  double p1[3] = {0, 0, 0}, p2[3] = {0, 0, 0};
  int nquad_in = 1;
  std::vector<double> cent_in = std::vector<double>(150, 0.0);
  std::vector<int> nradc_in = std::vector<int>(50, 50), nangc_in = std::vector<int>(50, 590);
  std::vector<double> sfalpha_in = std::vector<double>(50, 1.0), Ps_in = std::vector<double>(50, 1.0);
  std::vector<double> scan_start = std::vector<double>(20, 0.0), scan_end = std::vector<double>(20, 0.0),
                      scan_step = std::vector<double>(20, 0.0);
  std::vector<int> scan_nang = std::vector<int>(20, 590);
  double center_i[3] = {0, 0, 0}, step_i[3] = {0, 0, 0};
  int np_i[3] = {0, 0, 0};
  std::string precision = "mixed";
  double tolerance = 1e-10;
};

Input read_all_input(const std::string& path) {
  std::ifstream f(path);
  if (!f) die("Could not open input file: " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string text = ss.str();
  Input in;
  bool found;
  const Group files = parse_group(text, "files", &found);
  for (const auto& kv : files) {
    const std::string& k = kv.first;
    const std::string v = kv.second.count(1) ? kv.second.at(1) : "";
    if (k == "wfxfilename") in.wfx = v;
    else if (k == "fchkfilename") in.fchk = v;
    else if (k == "basfilename") in.bas = v;
    else if (k == "logfilename") in.log = v;
    else if (k == "dm2name") in.dm2 = v;
    else if (k == "outname") in.outname = v;
    else if (k == "cubeintraname") in.cubename = v;
    else if (k == "r_plot_name") in.radname = v;
    else die("Syntax error in &files block of the input file.");
  }
  const Group job = parse_group(text, "intracule_job", &found);
  auto first = [](const std::map<int, std::string>& m) { return m.begin()->second; };
  for (const auto& kv : job) {
    const std::string& k = kv.first;
    const auto& m = kv.second;
    if (k == "calc_type") in.calc_type = lower(first(m));
    else if (k == "c1calc") in.c1calc = to_bool(first(m));
    else if (k == "intracule_at_zero") in.zero = to_bool(first(m));
    else if (k == "intracule_two_points") in.two_points = to_bool(first(m));
    else if (k == "thresh") in.thresh = to_double(first(m));
    else if (k == "nosym") in.nosym = to_bool(first(m));
    else if (k == "nohydro") in.nohydro = to_bool(first(m));
    else if (k == "x_point1") in.p1[0] = to_double(first(m));
    else if (k == "y_point1") in.p1[1] = to_double(first(m));
    else if (k == "z_point1") in.p1[2] = to_double(first(m));
    else if (k == "x_point2") in.p2[0] = to_double(first(m));
    else if (k == "y_point2") in.p2[1] = to_double(first(m));
    else if (k == "z_point2") in.p2[2] = to_double(first(m));
    else if (k == "multicenter") in.multicenter = to_bool(first(m));
    else if (k == "manual_grid") in.manual_grid = to_bool(first(m));
    else if (k == "nrad") in.nrad = std::atoi(first(m).c_str());
    else if (k == "nang") in.nang = std::atoi(first(m).c_str());
    else if (k == "nquad_in") in.nquad_in = std::atoi(first(m).c_str());
    else if (k == "nblock") in.nblock = std::atoi(first(m).c_str());
    else if (k == "precision") in.precision = lower(first(m));
    else if (k == "tolerance") in.tolerance = to_double(first(m));
    else if (k == "cent_in") {
      for (const auto& e : m)
        if (e.first >= 1 && e.first <= 150) in.cent_in[e.first - 1] = to_double(e.second);
    } else if (k == "nradc_in" || k == "nangc_in" || k == "scan_nang") {
      auto& arr = k == "nradc_in" ? in.nradc_in : (k == "nangc_in" ? in.nangc_in : in.scan_nang);
      for (const auto& e : m)
        if (e.first >= 1 && e.first <= static_cast<int>(arr.size())) arr[e.first - 1] = std::atoi(e.second.c_str());
    } else if (k == "sfalpha_in" || k == "ps_in" || k == "scan_start" || k == "scan_end" || k == "scan_step") {
      auto& arr = k == "sfalpha_in" ? in.sfalpha_in
                  : k == "ps_in"    ? in.Ps_in
                  : k == "scan_start" ? in.scan_start
                  : k == "scan_end" ? in.scan_end
                                    : in.scan_step;
      for (const auto& e : m)
        if (e.first >= 1 && e.first <= static_cast<int>(arr.size())) arr[e.first - 1] = to_double(e.second);
    } else if (k == "center_i" || k == "step_i") {
      double* arr = k == "center_i" ? in.center_i : in.step_i;
      for (const auto& e : m)
        if (e.first >= 1 && e.first <= 3) arr[e.first - 1] = to_double(e.second);
    } else if (k == "np_i") {
      for (const auto& e : m)
        if (e.first >= 1 && e.first <= 3) in.np_i[e.first - 1] = std::atoi(e.second.c_str());
    } else {
      die("Syntax error in &intracule_job block of the input file.");
    }
  }
  const Group cube = parse_group(text, "cube_job", &found);
  for (const auto& kv : cube) {
    static const char* known[] = {"cube", "denscube", "primcube", "aocube", "mocube", "gradient", "laplacian",
                                  "npr", "cao", "mo", "center", "step", "np"};
    if (std::find_if(std::begin(known), std::end(known), [&](const char* s) { return kv.first == s; }) ==
        std::end(known))
      die("Syntax error in &cube_job block of the input file.");
    if (kv.first == "cube" && to_bool(kv.second.begin()->second))
      std::printf(" NOTE: one-electron cube files (&cube_job) are not part of this program.\n");
  }
  if (in.calc_type == "radial_integral") in.radial_integral = true;
  else if (in.calc_type == "radial_plot") in.radial_plot = true;
  else if (in.calc_type == "cubeintra") in.cubeintra = true;
  else if (!in.calc_type.empty()) {
    std::printf(" ERROR: Unknown calc_type '%s'.\n Valid values: radial_integral, radial_plot, cubeintra.\n",
                in.calc_type.c_str());
    std::exit(1);
  }
  if (in.wfx.empty() && in.fchk.empty()) die("No wavefunction file specified. Please provide a .wfx or .fchk file.");
  if (in.precision != "fp64" && in.precision != "mixed") die("precision must be 'fp64' or 'mixed'");
  auto stem = [&]() {
    const size_t dot = path.rfind('.');
    return dot == std::string::npos ? path : path.substr(0, dot);
  };
  if (in.outname.empty()) in.outname = stem() + ".out";
  if (in.radname.empty()) in.radname = stem() + ".rad";
  if (in.cubename.empty()) in.cubename = stem() + "_vector.cube";
  return in;
}

// ------------------------------------------------------------------ .fchk / .bas
struct Molecule {
  int natoms = 0, nelec = 0;
  std::vector<int> an;
  std::vector<double> cartes;  // natoms x 3 (row-major)
  int nprim = 0;
  std::vector<double> alpha, x, y, z;
  std::vector<int> tmn;  // nprim x 3 row-major
};

std::vector<std::string> read_lines(const std::string& path) {
  std::ifstream f(path);
  if (!f) die("Could not open file: " + path);
  std::vector<std::string> lines;
  std::string l;
  while (std::getline(f, l)) lines.push_back(l);
  return lines;
}

template <typename T>
std::vector<T> fchk_array(const std::vector<std::string>& L, const std::string& key, size_t n) {
  for (size_t i = 0; i < L.size(); ++i)
    if (L[i].find(key) != std::string::npos) {
      std::vector<T> out;
      for (size_t j = i + 1; j < L.size() && out.size() < n; ++j) {
        std::istringstream is(L[j]);
        std::string tk;
        while (is >> tk && out.size() < n) out.push_back(static_cast<T>(to_double(tk)));
      }
      if (out.size() < n) die("Section not found -> " + key);
      return out;
    }
  die("Section not found -> " + key);
}

long fchk_scalar(const std::vector<std::string>& L, const std::string& key) {
  for (const auto& l : L)
    if (l.find(key) != std::string::npos) {
      std::istringstream is(l);
      std::string tk, last;
      while (is >> tk) last = tk;
      return std::atol(last.c_str());
    }
  die("Section not found -> " + key);
}

// filefchk (src/mod_read_files.f90:432-691): geometry, electrons and the primitive list in
// shell order (Cartesian components; SP shells: s block then px, py, pz blocks).
void read_fchk(const std::string& path, Molecule& m) {
  const auto L = read_lines(path);
  m.natoms = static_cast<int>(fchk_scalar(L, "Number of atoms"));
  m.nelec = static_cast<int>(fchk_scalar(L, "Number of alpha electrons") + fchk_scalar(L, "Number of beta electrons"));
  m.an = fchk_array<int>(L, "Atomic numbers", m.natoms);
  m.cartes = fchk_array<double>(L, "Current cartesian coordinates", 3 * m.natoms);
  const long ncshl = fchk_scalar(L, "Number of contracted shells");
  const long npshl = fchk_scalar(L, "Number of primitive shells");
  const auto types = fchk_array<int>(L, "Shell types", ncshl);
  const auto pps = fchk_array<int>(L, "Number of primitives per shell", ncshl);
  const auto s2a = fchk_array<int>(L, "Shell to atom map", ncshl);
  const auto pexp = fchk_array<double>(L, "Primitive exponents", npshl);
  static const int comp[5][15][3] = {
      {{0, 0, 0}},
      {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
      {{2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}},
      {{3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1}, {0, 2, 1}, {1, 2, 0}, {1, 0, 2}, {0, 1, 2}, {1, 1, 1}},
      {{4, 0, 0}, {0, 4, 0}, {0, 0, 4}, {3, 1, 0}, {3, 0, 1}, {1, 3, 0}, {0, 3, 1}, {1, 0, 3}, {0, 1, 3},
       {2, 2, 0}, {2, 0, 2}, {0, 2, 2}, {2, 1, 1}, {1, 2, 1}, {1, 1, 2}}};
  static const int ncomp[5] = {1, 3, 6, 10, 15};
  m.alpha.clear(); m.tmn.clear(); m.x.clear(); m.y.clear(); m.z.clear();
  int l = 0;
  auto add = [&](int atom, double a, const int t[3]) {
    m.alpha.push_back(a);
    for (int d = 0; d < 3; ++d) m.tmn.push_back(t[d]);
    m.x.push_back(m.cartes[3 * (atom - 1)]);
    m.y.push_back(m.cartes[3 * (atom - 1) + 1]);
    m.z.push_back(m.cartes[3 * (atom - 1) + 2]);
  };
  for (long s = 0; s < ncshl; ++s) {
    const int t = types[s];
    if (t == -1) {  // SP: all s primitives, then px, py, pz blocks
      for (int blk = 0; blk < 4; ++blk)
        for (int k = 0; k < pps[s]; ++k) add(s2a[s], pexp[l + k], blk == 0 ? comp[0][0] : comp[1][blk - 1]);
      l += pps[s];
    } else {
      const int a = std::abs(t);
      if (a > 4) die("Shell type not implemented: " + std::to_string(t));
      if (t == 1) {  // p: per primitive, x, y, z
        for (int k = 0; k < pps[s]; ++k)
          for (int c = 0; c < 3; ++c) add(s2a[s], pexp[l + k], comp[1][c]);
      } else {
        for (int k = 0; k < pps[s]; ++k)
          for (int c = 0; c < ncomp[a]; ++c) add(s2a[s], pexp[l + k], comp[a][c]);
      }
      l += pps[s];
    }
  }
  m.nprim = static_cast<int>(m.alpha.size());
}

// filebas (src/mod_read_files.f90:695-726): per primitive, after the '#' line:
// Z, X, Y, Z (bohr), exponent, nx, ny, nz -- in .dm2p order; overwrites the .fchk list.
void read_bas(const std::string& path, Molecule& m) {
  const auto L = read_lines(path);
  size_t i = 0;
  while (i < L.size() && L[i].find('#') == std::string::npos) ++i;
  if (i == L.size()) die("Section not found -> #");
  ++i;
  const int n = m.nprim;
  for (int p = 0; p < n; ++p, ++i) {
    if (i >= L.size()) die("end of file in " + path);
    std::istringstream is(L[i]);
    std::string k, x, y, z, a, t0, t1, t2;
    if (!(is >> k >> x >> y >> z >> a >> t0 >> t1 >> t2)) die("bad primitive line in " + path);
    m.x[p] = to_double(x);
    m.y[p] = to_double(y);
    m.z[p] = to_double(z);
    m.alpha[p] = to_double(a);
    m.tmn[3 * p] = std::atoi(t0.c_str());
    m.tmn[3 * p + 1] = std::atoi(t1.c_str());
    m.tmn[3 * p + 2] = std::atoi(t2.c_str());
  }
}

void check(inca_ctx* ctx, int st) {
  if (st != INCA_OK) die(std::string(inca_last_error(ctx)));
}

std::string es(double v, int w, int d) {  // Fortran ESw.d
  char buf[64];
  std::snprintf(buf, sizeof buf, "%*.*E", w, d, v);
  return buf;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::printf(" =====================================================\n");
    std::printf("  INCA: Intracule Calculator (GB300)\n");
    std::printf(" =====================================================\n");
    std::printf("  ERROR: No input file provided.\n  USAGE: ./inca_gpu <input_file.txt>\n");
    return 1;
  }
  const auto t_start = std::chrono::steady_clock::now();
  Input in = read_all_input(argv[1]);
  if (!in.wfx.empty() && in.fchk.empty()) die(".wfx input is not supported by this program; provide the .fchk");
  Molecule mol;
  read_fchk(in.fchk, mol);
  if (!in.bas.empty()) read_bas(in.bas, mol);
  const bool intracalc = !in.calc_type.empty() || in.zero || in.two_points;
  if (in.c1calc) std::printf(" NOTE: the C1 Coulomb hole (c1calc) is not part of this program.\n");
  if (!intracalc) return 0;
  if (in.bas.empty()) {
    std::printf(" CAUTION: Primitive info comes from .wfx or .fchk file\n");
    std::printf("  i primtive may not coincide with that of the .dm2p file\n");
  }
  if ((in.radial_integral || in.radial_plot || in.cubeintra) && (in.zero || in.two_points))
    die("intracule_at_zero / intracule_two_points cannot be combined with calc_type in one run");

  inca_ctx* ctx = nullptr;
  if (inca_ctx_create(&ctx, 0) != INCA_OK) die("no usable GB300 (sm_103) device");
  std::vector<int> tmn_cm(3 * mol.nprim);
  for (int p = 0; p < mol.nprim; ++p)
    for (int d = 0; d < 3; ++d) tmn_cm[p + mol.nprim * d] = mol.tmn[3 * p + d];
  check(ctx, inca_set_primitives(ctx, mol.nprim, mol.alpha.data(), tmn_cm.data(), mol.x.data(), mol.y.data(),
                                 mol.z.data()));

  // grids (setup_grids + the grid selection of calculate_intracule)
  int nquad = 0;
  std::vector<double> cent, Ps, sfalpha;
  std::vector<int> nradc, nangc;
  int64_t maxgrid = 0, rgrid = 0, ngrid = 0;
  int32_t nradi = 0;
  if (in.radial_integral) {
    if (in.multicenter) {
      if (in.manual_grid) {
        nquad = in.nquad_in;
        for (int i = 0; i < nquad; ++i) {
          for (int d = 0; d < 3; ++d) cent.push_back(in.cent_in[3 * i + d]);
          nradc.push_back(in.nradc_in[i]);
          nangc.push_back(in.nangc_in[i]);
          sfalpha.push_back(in.sfalpha_in[i]);
          Ps.push_back(in.Ps_in[i]);
        }
      } else {
        const int cap = mol.natoms * (mol.natoms - 1) + 1;
        std::vector<double> cart_cm(3 * mol.natoms);
        for (int a = 0; a < mol.natoms; ++a)
          for (int d = 0; d < 3; ++d) cart_cm[a + mol.natoms * d] = mol.cartes[3 * a + d];
        cent.resize(3 * cap);
        Ps.resize(cap);
        sfalpha.resize(cap);
        int32_t nq = 0;
        if (inca_centercalc(mol.natoms, mol.an.data(), cart_cm.data(), in.nohydro, in.betaone, &nq, cent.data(),
                            Ps.data(), sfalpha.data()) != INCA_OK)
          die("centercalc failed");
        nquad = nq;
        cent.resize(3 * nquad);
        Ps.resize(nquad);
        sfalpha.resize(nquad);
        nradc.assign(nquad, in.nrad);
        nangc.assign(nquad, in.nang);
      }
    } else {
      nquad = 1;
      cent = {0, 0, 0};
      nradc = {in.nrad};
      nangc = {in.nang};
      sfalpha = {in.sfalpha_in[0]};
      Ps = {1.0};
    }
    check(ctx, inca_grid_radial(ctx, nquad, nradc.data(), nangc.data(), sfalpha.data(), cent.data(), Ps.data(),
                                in.nosym, &maxgrid, &rgrid, &ngrid));
  }
  std::vector<double> start, end, step;
  std::vector<int> nang;
  if (in.radial_plot) {
    for (int b = 0; b < in.nblock; ++b) {
      start.push_back(in.scan_start[b]);
      end.push_back(in.scan_end[b]);
      step.push_back(in.scan_step[b]);
      nang.push_back(in.scan_nang[b]);
    }
    check(ctx, inca_grid_scan(ctx, in.nblock, start.data(), end.data(), step.data(), nang.data(), in.nosym, &nradi,
                              &ngrid));
    rgrid = ngrid;
  }
  if (in.cubeintra) {
    check(ctx, inca_grid_cube(ctx, in.center_i, in.step_i, in.np_i, &ngrid));
    rgrid = ngrid;
  }
  if (in.zero) {
    const double r0[3] = {0, 0, 0};
    check(ctx, inca_grid_points(ctx, 1, r0));
    ngrid = 1;
  }
  if (in.two_points) {
    const double r2[6] = {in.p1[0], in.p1[1], in.p1[2], in.p2[0], in.p2[1], in.p2[2]};
    check(ctx, inca_grid_points(ctx, 2, r2));
    ngrid = 2;
  }
  std::printf(" Number of grid points to compute intracule: %lld\n", static_cast<long long>(ngrid));
  const auto t_grid = std::chrono::steady_clock::now();

  // quartets, screening, evaluation
  if (in.dm2.empty()) die("no .dm2p file (dm2name) given");
  int64_t nread = 0;
  check(ctx, inca_load_dm2p(ctx, in.dm2.c_str(), &nread));
  inca_counts counts;
  check(ctx, inca_prepare(ctx, in.thresh, 1, &counts));
  const int mode = in.precision == "fp64" ? INCA_FP64 : INCA_MIXED;
  std::vector<double> ivec(ngrid);
  check(ctx, inca_eval(ctx, mode, in.tolerance, ivec.data()));
  const auto t_loop = std::chrono::steady_clock::now();
  const int64_t P = static_cast<int64_t>(mol.nprim) * (mol.nprim + 1) / 2;
  const int64_t refval = ((P + 1) * P) / 2;
  if (counts.read > refval) {
    std::printf(" Full DM2prim read\n");
  } else {
    std::printf(" Symmetry reduced DM2prim.\n");
    if (!in.nosym) std::printf(" Run with NOSYM option.\n");
  }
  const double lim = in.thresh * (1.0 / (double(mol.nprim) * (double(mol.nprim) + 1.0) * 0.5));

  // ---------------- .out report (src/mod_intracule.f90:410-504)
  FILE* out = std::fopen(in.outname.c_str(), "w");
  if (!out) die("cannot write " + in.outname);
  std::fprintf(out, " ==========================================================\n");
  std::fprintf(out, "                INCA INTRACULE CALCULATION                 \n");
  std::fprintf(out, " ==========================================================\n");
  std::fprintf(out, " --- GRID AND ACCURACY SETTINGS ---\n");
  std::fprintf(out, " Original grid points:             %12lld\n", static_cast<long long>(maxgrid));
  std::fprintf(out, " Symmetry reduced grid points:     %12lld\n", static_cast<long long>(rgrid));
  std::fprintf(out, " Total surviving grid points:      %12lld\n", static_cast<long long>(in.radial_integral ? ngrid : 0));
  std::fprintf(out, " Quartets in the dm2p file:        %12lld\n", static_cast<long long>(counts.read));
  std::fprintf(out, " Quartets after 1st screening:     %12lld\n", static_cast<long long>(counts.after_screen1));
  std::fprintf(out, " Quartets actually computed:       %12lld\n", static_cast<long long>(counts.after_screen2));
  std::fprintf(out, "Screening limit (lim):            %s\n", es(lim, 12, 4).c_str());
  std::fprintf(out, " Evaluation precision:             %s (tolerance %s)\n", in.precision.c_str(),
               es(in.tolerance, 10, 2).c_str());
  std::fprintf(out, " \n --- RESULTS ---\n");
  if (in.radial_integral) {
    std::fprintf(out, " Calculation Type: Radial Integral\n");
    std::fprintf(out, " Number of centres: %12d\n", nquad);
    if (nquad > 1) std::fprintf(out, " Centres for radial integration:\n");
    for (int i = 0; i < nquad; ++i)
      std::fprintf(out, " %12d :::  %25.16E %25.16E %25.16E\n", i + 1, cent[3 * i], cent[3 * i + 1], cent[3 * i + 2]);
    std::fprintf(out, " Weights for centres: ");
    for (double p : Ps) std::fprintf(out, " %25.16E", p);
    std::fprintf(out, "\n Alpha parameter:     ");
    for (double a : sfalpha) std::fprintf(out, " %25.16E", a);
    std::fprintf(out, "\n Gauss-Legendre nodes:");
    for (int n : nradc) std::fprintf(out, " %12d", n);
    std::fprintf(out, "\n Gauss-Lebedev nodes: ");
    for (int n : nangc) std::fprintf(out, " %12d", n);
    std::fprintf(out, "\n");
    double total = 0, vee = 0;
    std::vector<double> rl(nquad), vl(nquad);
    check(ctx, inca_radial_integral(ctx, &total, &vee, rl.data(), vl.data()));
    std::fprintf(out, " ---------------------------------------------\n");
    std::fprintf(out, "TOTAL VALUE OF INTRACULE = %s\n", es(total, 25, 16).c_str());
    std::fprintf(out, "TOTAL VALUE OF Vee       = %s\n", es(vee, 25, 16).c_str());
    const int npairs = mol.nelec * (mol.nelec - 1) / 2;
    std::fprintf(out, "Radial_integral error    = %s\n", es(total - npairs, 15, 6).c_str());
    std::fprintf(out, " ---------------------------------------------\n");
    std::fprintf(out, " -------LOCAL DECOMPOSITION (TFVC)-------\n");
    std::fprintf(out, "%6s %20s %15s %15s\n", "Center", "Coordinates", "Pairs(N_pairs)", "Vee(Hartree)");
    for (int i = 0; i < nquad; ++i)
      std::fprintf(out, "%6d %7.3f%7.3f%7.3f %15.8f %15.8f %s\n", i + 1, cent[3 * i], cent[3 * i + 1], cent[3 * i + 2],
                   rl[i], vl[i], i == 0 ? "(INTRA-ATOMIC)" : "(INTER/DISP)");
    std::fprintf(out, " ---------------------------------------------\n");
    // radial smearing side output (mod_intracule.f90:535-550)
    double umax = 0;
    for (int i = 0; i < nquad; ++i)
      umax = std::max(umax, std::sqrt(cent[3 * i] * cent[3 * i] + cent[3 * i + 1] * cent[3 * i + 1] +
                                      cent[3 * i + 2] * cent[3 * i + 2]));
    umax += 5.0;
    std::vector<double> u(1000), Pu(1000), Ia(1000);
    check(ctx, inca_radial_smearing(ctx, umax, 1000, 0.15, u.data(), Pu.data(), Ia.data()));
    const size_t dot = in.outname.rfind('.');
    const std::string sm = (dot == std::string::npos ? in.outname : in.outname.substr(0, dot)) + "_smearing.dat";
    FILE* fs = std::fopen(sm.c_str(), "w");
    if (fs) {
      std::fprintf(fs, " #   u (bohr)       P(u) [Prob]      I_avg(u) [Density]\n");
      for (int j = 0; j < 1000; ++j) std::fprintf(fs, "%s%s%s\n", es(u[j], 16, 8).c_str(), es(Pu[j], 16, 8).c_str(),
                                                  es(Ia[j], 16, 8).c_str());
      std::fclose(fs);
    }
  } else if (in.radial_plot) {
    std::vector<double> radi(nradi), rin(nradi);
    check(ctx, inca_radial_plot(ctx, radi.data(), rin.data()));
    std::fprintf(out, " Calculation Type: Radial Plot, I(s) vs s\n");
    std::fprintf(out, " Radius evaluated from %25.16E  to %25.16E  bohr\n", radi.front(), radi.back());
    std::fprintf(out, " Data written to: %s\n", in.radname.c_str());
    FILE* fr = std::fopen(in.radname.c_str(), "w");
    if (!fr) die("cannot write " + in.radname);
    std::fprintf(fr, " # --------------------------------------------------------\n");
    std::fprintf(fr, " # RADIAL INTRACULE DATA\n");
    std::fprintf(fr, " # Col 1: Distance s (bohr)\n");
    std::fprintf(fr, " # Col 2: I(s) (Radial Intracule)\n");
    std::fprintf(fr, " # Col 3: P(s) = 2 * pi * s^2 * I(s) (Probability Density)\n");
    std::fprintf(fr, " # Col 4: s * I(s)\n");
    std::fprintf(fr, " # --------------------------------------------------------\n");
    const double pi = 4.0 * std::atan(1.0);
    for (int i = 0; i < nradi; ++i)
      std::fprintf(fr, "%12.6f%s%s%s\n", radi[i], es(rin[i], 20, 8).c_str(),
                   es(rin[i] * 2.0 * pi * radi[i] * radi[i], 20, 8).c_str(), es(rin[i] * 2.0 * pi * radi[i], 20, 8).c_str());
    std::fclose(fr);
  } else if (in.cubeintra) {
    std::fprintf(out, " Calculation Type: Vectorial Cubefile\n");
    std::fprintf(out, " Data written to: %s\n", in.cubename.c_str());
    FILE* fc = std::fopen(in.cubename.c_str(), "w");
    if (!fc) die("cannot write " + in.cubename);
    std::fprintf(fc, " CUBE FILE\n OUTER LOOP:X, MIDDLE LOOP:Y, INNER LOOP:Z\n");
    std::fprintf(fc, " %11d %25.16E %25.16E %25.16E\n", mol.natoms, in.center_i[0], in.center_i[1], in.center_i[2]);
    std::fprintf(fc, " %11d %25.16E %25.16E %25.16E\n", in.np_i[0], in.step_i[0], 0.0, 0.0);
    std::fprintf(fc, " %11d %25.16E %25.16E %25.16E\n", in.np_i[1], 0.0, in.step_i[1], 0.0);
    std::fprintf(fc, " %11d %25.16E %25.16E %25.16E\n", in.np_i[2], 0.0, 0.0, in.step_i[2]);
    for (int a = 0; a < mol.natoms; ++a)
      std::fprintf(fc, " %11d %25.16E %25.16E %25.16E %25.16E\n", mol.an[a], double(mol.an[a]), mol.cartes[3 * a],
                   mol.cartes[3 * a + 1], mol.cartes[3 * a + 2]);
    for (int64_t g = 0; g < ngrid; ++g) std::fprintf(fc, " %25.16E\n", ivec[g]);
    std::fclose(fc);
  }
  if (in.zero) std::fprintf(out, "INTRACULE AT ZERO = %s\n", es(ivec[0] / 2.0, 25, 16).c_str());
  if (in.two_points) {
    std::fprintf(out, " Point 1: %25.16E %25.16E %25.16E  Intracule: %25.16E\n", in.p1[0], in.p1[1], in.p1[2], ivec[0]);
    std::fprintf(out, " Point 2: %25.16E %25.16E %25.16E  Intracule: %25.16E\n", in.p2[0], in.p2[1], in.p2[2], ivec[1]);
  }
  const auto t_end = std::chrono::steady_clock::now();
  auto sec = [](auto a, auto b) { return std::chrono::duration<double>(b - a).count(); };
  double ktot = 0, kk = 0;
  int32_t kl = 0, ll = 0;
  inca_last_eval_timing(ctx, &ktot, &kk, &kl, &ll);
  std::fprintf(out, " \n --- COMPUTATIONAL TIME ---\n");
  std::fprintf(out, "Total CPU time:             %10.3f seconds\n", sec(t_start, t_end));
  std::fprintf(out, "Grid generation time:       %10.3f seconds\n", sec(t_start, t_grid));
  std::fprintf(out, "Integration loop time:      %10.3f seconds\n", sec(t_grid, t_loop));
  std::fprintf(out, "GPU evaluation time:        %10.3f seconds\n", ktot / 1000.0);
  std::fprintf(out, " ==========================================================\n");
  std::fclose(out);
  inca_ctx_destroy(ctx);
  std::printf(" >> INCA job finished successfully. Output written to: %s\n", in.outname.c_str());
  return 0;
}
