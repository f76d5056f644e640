// Host-side tables and file input of libinca_gpu.so: Lebedev-Laikov rules, Gauss-Legendre
// nodes, the .dm2p reader and the automatic integration centres. All small or I/O-bound;
// the grids themselves are built on the device (grid_build.cu).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "inca_internal.h"
#include "lebedev_table.h"

namespace inca {

// Points of one Lebedev-Laikov rule from its octahedral orbit generators. Orbit types as in
// gen_oh (src/lebedev.f:1-588): (0,0,1) 6 points, (0,a,a) 12, (a,a,a) 8, (a,a,b) 24,
// (a,b,0) 24, (a,b,c) 48. Weights sum to 1.
int lebedev_rule(int nang, std::vector<double>& x, std::vector<double>& y, std::vector<double>& z,
                 std::vector<double>& w) {
  int rule = -1;
  for (int r = 0; r < inca_leb::kNumRules; ++r)
    if (inca_leb::kRulePoints[r] == nang) rule = r;
  if (rule < 0) return -1;
  x.clear(); y.clear(); z.clear(); w.clear();
  auto put = [&](double a, double b, double c, double v) {
    x.push_back(a); y.push_back(b); z.push_back(c); w.push_back(v);
  };
  for (int o = inca_leb::kRuleOffset[rule]; o < inca_leb::kRuleOffset[rule + 1]; ++o) {
    const inca_leb::Orbit& g = inca_leb::kOrbits[o];
    const double v = g.v;
    if (g.code == 1) {
      put(1, 0, 0, v); put(-1, 0, 0, v); put(0, 1, 0, v);
      put(0, -1, 0, v); put(0, 0, 1, v); put(0, 0, -1, v);
    } else if (g.code == 2) {
      const double a = std::sqrt(0.5);
      for (int s1 = 0; s1 < 2; ++s1)
        for (int s2 = 0; s2 < 2; ++s2) {
          const double p = s2 ? -a : a, q = s1 ? -a : a;
          put(0, p, q, v); put(p, 0, q, v); put(p, q, 0, v);
        }
    } else if (g.code == 3) {
      const double a = std::sqrt(1.0 / 3.0);
      for (int s = 0; s < 8; ++s) put((s & 1) ? -a : a, (s & 2) ? -a : a, (s & 4) ? -a : a, v);
    } else if (g.code == 4) {
      const double a = g.a, b = std::sqrt(1.0 - 2.0 * a * a);
      for (int s = 0; s < 8; ++s) {
        const double p = (s & 1) ? -a : a, q = (s & 2) ? -a : a, r = (s & 4) ? -b : b;
        put(p, q, r, v); put(p, r, q, v); put(r, p, q, v);
      }
    } else if (g.code == 5) {
      const double a = g.a, b = std::sqrt(1.0 - a * a);
      for (int s = 0; s < 4; ++s) {
        const double p = (s & 1) ? -a : a, q = (s & 2) ? -b : b;
        put(p, q, 0, v); put(q, p, 0, v); put(p, 0, q, v);
        put(q, 0, p, v); put(0, p, q, v); put(0, q, p, v);
      }
    } else if (g.code == 6) {
      const double a = g.a, b = g.b, c = std::sqrt(1.0 - a * a - b * b);
      for (int s = 0; s < 8; ++s) {
        const double p = (s & 1) ? -a : a, q = (s & 2) ? -b : b, r = (s & 4) ? -c : c;
        put(p, q, r, v); put(p, r, q, v); put(q, p, r, v);
        put(q, r, p, v); put(r, p, q, v); put(r, q, p, v);
      }
    } else {
      return -1;
    }
  }
  return static_cast<int>(x.size()) == nang ? 0 : -1;
}

// Gauss-Legendre on [-1,1] by Newton iteration on the three-term recurrence, stopping at
// |dz| <= 1e-14 with the weight from the derivative at the previous iterate
// (sub_GauLeg, src/mod_quadratures.f90:37-86). Nodes ascending.
void gauss_legendre(int n, double* t, double* w) {
  const double pi = std::acos(-1.0);
  const int m = static_cast<int>((double(n) + 1.0) / 2.0);
  for (int i = 1; i <= m; ++i) {
    double z = std::cos(pi * (double(i) - 0.25) / (double(n) + 0.5));
    double z1, dp;
    do {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        const double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * double(j) - 1.0) * z * p2 - (double(j) - 1.0) * p3) / double(j);
      }
      dp = double(n) * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / dp;
    } while (std::fabs(z - z1) > 1e-14);
    t[i - 1] = -z;
    t[n - i] = z;
    w[i - 1] = 2.0 / ((1.0 - z * z) * dp * dp);
    w[n - i] = w[i - 1];
  }
}

// .dm2p reader (src/mod_intracule.f90:164-262). The first two int32 of the file decide the
// format: (24, 0) -> 8-byte record markers (rejected), 24 -> sequential records with 4-byte
// markers, 0 -> zero markers (rejected), anything else -> flat stream of 24-byte records
// <int32 i,j,k,l; float64 v>. Records are read until end of file (a partial trailing record
// is dropped) or until the first record with i outside 1..nprim or j,k,l < 1. Unlike the
// reference, which reads out of bounds in that case, j, k or l above nprim is an error.
int read_dm2p(const char* path, int nprim, std::vector<int4>& ijkl, std::vector<double>& v,
              std::string& err) {
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    err = std::string("cannot open .dm2p file: ") + path;
    return INCA_E_IO;
  }
  int32_t head[2] = {0, 0};
  size_t got = std::fread(head, sizeof(int32_t), 2, f);
  std::fseek(f, 0, SEEK_SET);
  int format = 0;
  if (got == 2) {
    if (head[0] == 24 && head[1] == 0) format = 3;
    else if (head[0] == 24) format = 1;
    else if (head[0] == 0) format = 2;
  }
  if (format == 2 || format == 3) {
    std::fclose(f);
    err = "unsupported .dm2p format with markers (8-byte or zero); convert to stream format";
    return INCA_E_FORMAT;
  }
  ijkl.clear();
  v.clear();
  const size_t rec = format == 1 ? 32 : 24;
  const size_t kBatch = 1 << 16;
  std::vector<unsigned char> buf(rec * kBatch);
  bool done = false;
  int status = INCA_OK;
  while (!done) {
    size_t n = std::fread(buf.data(), rec, kBatch, f);
    if (n < kBatch) done = true;
    for (size_t r = 0; r < n; ++r) {
      const unsigned char* p = buf.data() + r * rec + (format == 1 ? 4 : 0);
      if (format == 1) {
        int32_t m0, m1;
        std::memcpy(&m0, buf.data() + r * rec, 4);
        std::memcpy(&m1, buf.data() + r * rec + 28, 4);
        if (m0 != 24 || m1 != 24) {  // err= branch of the reference read
          done = true;
          break;
        }
      }
      int32_t q[4];
      double val;
      std::memcpy(q, p, 16);
      std::memcpy(&val, p + 16, 8);
      if (q[0] < 1 || q[0] > nprim || q[1] < 1 || q[2] < 1 || q[3] < 1) {
        done = true;
        break;
      }
      if (q[1] > nprim || q[2] > nprim || q[3] > nprim) {
        err = "record " + std::to_string(v.size() + 1) + " of " + path +
              " has an index above nprim=" + std::to_string(nprim);
        status = INCA_E_FORMAT;
        done = true;
        break;
      }
      ijkl.push_back(make_int4(q[0], q[1], q[2], q[3]));
      v.push_back(val);
    }
  }
  if (std::ferror(f) && status == INCA_OK) {
    err = std::string("read error on ") + path;
    status = INCA_E_IO;
  }
  std::fclose(f);
  return status;
}

}  // namespace inca

// Bragg-Slater radii in Angstrom (Slater 1964; H from Becke 1988; He, Ne by convention;
// 1.00 for the rest), as tabulated by get_bs_radius (src/mod_autogrid.f90:142-185).
static double bs_radius_bohr(int z) {
  static const double r[37] = {1.00, 0.35, 0.35, 1.45, 1.05, 0.85, 0.70, 0.65, 0.60, 0.50,
                               0.38, 1.80, 1.50, 1.25, 1.10, 1.00, 1.00, 1.00, 1.00, 2.20,
                               1.80, 1.60, 1.40, 1.35, 1.40, 1.40, 1.40, 1.35, 1.35, 1.35,
                               1.35, 1.30, 1.25, 1.15, 1.15, 1.15, 1.00};
  const double a = (z >= 1 && z <= 35) ? r[z] : 1.00;
  return a * 1.8897;
}

// centercalc (src/mod_autogrid.f90:12-134): the origin (pair population sum Z(Z-1)/2,
// alpha the population-weighted radius) plus +-(R_j - R_k) for atom pairs (heavy atoms only
// with nohydro), z snapped to 0 below 0.5 bohr, centres merged within 0.1 bohr per component.
extern "C" int inca_centercalc(int32_t natoms, const int32_t* an, const double* cartes,
                               int nohydro, int betaone, int32_t* nquad_out, double* cent,
                               double* Ps, double* sfalpha) {
  if (natoms < 1 || !an || !cartes || !nquad_out || !cent || !Ps || !sfalpha) return INCA_E_ARG;
  auto X = [&](int atom, int d) { return cartes[atom + static_cast<size_t>(natoms) * d]; };
  int cap = natoms * (natoms - 1) + 1;
  std::vector<double> c1(3 * static_cast<size_t>(cap), 0.0), pop(cap, 0.0), al(cap, 0.0);
  double tot = 0, wsum = 0;
  for (int i = 0; i < natoms; ++i) {
    const double pairs = an[i] * (an[i] - 1.0) / 2.0;
    tot += pairs;
    wsum += pairs * bs_radius_bohr(an[i]);
  }
  pop[0] = tot;
  al[0] = tot > 1e-15 ? wsum / tot : bs_radius_bohr(1);
  int sm = 0;
  for (int j = 0; j < natoms - 1; ++j)
    for (int k = j + 1; k < natoms; ++k) {
      if (nohydro && !(an[j] > 1 && an[k] > 1)) continue;
      ++sm;
      for (int d = 0; d < 3; ++d) c1[3 * sm + d] = X(j, d) - X(k, d);
      pop[sm] = an[j] * an[k] * 0.5;
      al[sm] = (bs_radius_bohr(an[j]) + bs_radius_bohr(an[k])) / 2.0;
      if (std::fabs(c1[3 * sm + 2]) < 0.5) c1[3 * sm + 2] = 0.0;
      const int sp = sm++;
      for (int d = 0; d < 3; ++d) c1[3 * sm + d] = -c1[3 * sp + d];
      pop[sm] = pop[sp];
      al[sm] = al[sp];
    }
  const int nq = sm + 1;
  for (int i = 1; i < nq - 1; ++i) {
    if (std::fabs(c1[3 * i]) + std::fabs(c1[3 * i + 1]) + std::fabs(c1[3 * i + 2]) == 0.0) continue;
    for (int j = i + 1; j < nq; ++j) {
      bool same = true;
      for (int d = 0; d < 3; ++d)
        if (!(std::fabs(c1[3 * i + d] - c1[3 * j + d]) < 0.1)) same = false;
      if (!same) continue;
      al[i] = (al[i] * pop[i] + al[j] * pop[j]) / (pop[i] + pop[j]);
      pop[i] += pop[j];
      c1[3 * j] = c1[3 * j + 1] = c1[3 * j + 2] = 0.0;
      pop[j] = 0.0;
    }
  }
  int out = 0;
  for (int i = 0; i < nq; ++i) {
    const double z = std::fabs(c1[3 * i]) + std::fabs(c1[3 * i + 1]) + std::fabs(c1[3 * i + 2]);
    if (i != 0 && z == 0.0) continue;
    for (int d = 0; d < 3; ++d) cent[3 * out + d] = c1[3 * i + d];
    Ps[out] = betaone ? 1.0 : pop[i];
    sfalpha[out] = betaone ? 1.0 : al[i];
    ++out;
  }
  *nquad_out = out;
  return INCA_OK;
}
