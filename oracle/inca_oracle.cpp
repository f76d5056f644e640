// INCA intracule oracle -- TEST INFRASTRUCTURE ONLY.
//
// This is a plain C++ FP64 (+OpenMP) restatement of the reference's intracule path
// (markelgtx/INCA_parallel, Fortran 90). It exists only to check the GPU product: tests/,
// __graft_entry__.smoke() and the CPU-baseline leg of bench.py may load it, nothing else.
// The product (inca_parallel_gb300/) never links or calls it.
//
// Parity pin: its CH4 outputs are checked against the reference's own golden values
// (tests/run_tests.py:24-28, tests/refs/ch4_ref.rad, tests/refs/ch4_ref.cube) by
// tests/test_oracle_golden.py.
//
// Every function cites the reference lines it restates. Shared with the product are only
// the two generated constant tables (Lebedev-Laikov orbit generators and Gauss-Hermite
// nodes/weights), which are published numbers, validated independently in the tests.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#include <omp.h>

#include "../inca_parallel_gb300/csrc/lebedev_table.h"
#include "../inca_parallel_gb300/csrc/hermite_table.h"

namespace {

const double kPi = 4.0 * std::atan(1.0);  // mod_numbers.f90:6
const double kPi15 = kPi * std::sqrt(kPi); // pi**1.5 (mod_intrastuff.f90:115)
const int kMaxDeg = 16;                    // per-dimension polynomial degree (g shells)
const int kMaxCoef = kMaxDeg + 1;

// dfact: double factorial with dfact(-1) = 1 (mod_numbers.f90:14-28)
long long dfact(int a) {
  long long r = 1;
  if (a % 2 == 0) {
    for (int i = 1; i <= a / 2; ++i) r *= 2 * i;
  } else {
    for (int i = 1; i <= (a + 1) / 2; ++i) r *= 2 * i - 1;
  }
  return r;
}

// Gauss-Legendre nodes/weights on [-1,1] by Newton iteration on the Legendre three-term
// recurrence (mod_quadratures.f90:37-86). Nodes ascending; the weight uses the derivative
// evaluated at the last-but-one iterate, as the reference does.
void gauleg(int n, double* t, double* w) {
  const double eps = 1e-14;
  const double pi = std::acos(-1.0);
  int m = (int)((double(n) + 1.0) / 2.0);
  for (int i = 1; i <= m; ++i) {
    double z = std::cos(pi * (double(i) - 0.25) / (double(n) + 0.5));
    double z1, pp;
    do {
      double p1 = 1.0, p2 = 0.0, p3;
      for (int j = 1; j <= n; ++j) {
        p3 = p2;
        p2 = p1;
        p1 = ((2.0 * double(j) - 1.0) * z * p2 - (double(j) - 1.0) * p3) / double(j);
      }
      pp = double(n) * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    } while (std::fabs(z - z1) > eps);
    t[i - 1] = -z;
    t[n - i] = z;
    w[i - 1] = 2.0 / ((1.0 - z * z) * pp * pp);
    w[n - i] = w[i - 1];
  }
}

// Expand the orbit generators of one Lebedev-Laikov rule into points (gen_oh semantics,
// src/lebedev.f:1-588: six orbit types of 6, 12, 8, 24, 24 and 48 points).
int lebedev(int nang, std::vector<double>& x, std::vector<double>& y, std::vector<double>& z,
            std::vector<double>& w) {
  int rule = -1;
  for (int r = 0; r < inca_leb::kNumRules; ++r)
    if (inca_leb::kRulePoints[r] == nang) rule = r;
  if (rule < 0) return -1;
  x.clear(); y.clear(); z.clear(); w.clear();
  auto add = [&](double a, double b, double c, double v) {
    x.push_back(a); y.push_back(b); z.push_back(c); w.push_back(v);
  };
  for (int o = inca_leb::kRuleOffset[rule]; o < inca_leb::kRuleOffset[rule + 1]; ++o) {
    const inca_leb::Orbit& ob = inca_leb::kOrbits[o];
    double v = ob.v;
    switch (ob.code) {
      case 1:
        add(1, 0, 0, v); add(-1, 0, 0, v); add(0, 1, 0, v);
        add(0, -1, 0, v); add(0, 0, 1, v); add(0, 0, -1, v);
        break;
      case 2: {
        double a = std::sqrt(0.5);
        for (int s1 = 0; s1 < 2; ++s1)
          for (int s2 = 0; s2 < 2; ++s2) {
            double p = s2 ? -a : a, q = s1 ? -a : a;
            add(0, p, q, v); add(p, 0, q, v); add(p, q, 0, v);
          }
        break;
      }
      case 3: {
        double a = std::sqrt(1.0 / 3.0);
        for (int s = 0; s < 8; ++s)
          add((s & 1) ? -a : a, (s & 2) ? -a : a, (s & 4) ? -a : a, v);
        break;
      }
      case 4: {
        double a = ob.a, b = std::sqrt(1.0 - 2.0 * a * a);
        for (int s = 0; s < 8; ++s) {
          double p = (s & 1) ? -a : a, q = (s & 2) ? -a : a, r = (s & 4) ? -b : b;
          add(p, q, r, v); add(p, r, q, v); add(r, p, q, v);
        }
        break;
      }
      case 5: {
        double a = ob.a, b = std::sqrt(1.0 - a * a);
        for (int s = 0; s < 4; ++s) {
          double p = (s & 1) ? -a : a, q = (s & 2) ? -b : b;
          add(p, q, 0, v); add(q, p, 0, v); add(p, 0, q, v);
          add(q, 0, p, v); add(0, p, q, v); add(0, q, p, v);
        }
        break;
      }
      case 6: {
        double a = ob.a, b = ob.b, c = std::sqrt(1.0 - a * a - b * b);
        for (int s = 0; s < 8; ++s) {
          double p = (s & 1) ? -a : a, q = (s & 2) ? -b : b, r = (s & 4) ? -c : c;
          add(p, q, r, v); add(p, r, q, v); add(q, p, r, v);
          add(q, r, p, v); add(r, p, q, v); add(r, q, p, v);
        }
        break;
      }
      default:
        return -1;
    }
  }
  return (int)x.size() == nang ? 0 : -1;
}

// ---- Deterministic FP64 arithmetic for the screening quantities.
// The reference evaluates its bounds with Fortran ** and dexp (libm). The oracle fixes the
// operation sequence instead, so the GPU's screening can be checked bit for bit:
//  * x**n for integer n >= 0: left-to-right repeated multiplication (x**0 = 1);
//  * exp: Cody-Waite reduction x = k ln2 + r (ln2 split in a 32-bit head and a tail),
//    Taylor polynomial of degree 13 for e^r by Horner, scaled by 2^k.
// Compiled without FMA contraction; the results differ from libm by at most a few ulp.
double ipow(double x, int n) {
  if (n <= 0) return 1.0;
  double r = x;
  for (int i = 1; i < n; ++i) r = r * x;
  return r;
}

double pexp(double x) {
  if (x != x) return x;
  if (x > 709.0) return HUGE_VAL;
  if (x < -708.0) return 0.0;  // no subnormal results
  const double kInvLn2 = 1.4426950408889634;
  const double kLn2Hi = 0.6931471803691238;      // 0x1.62e42feep-1: 32 significant bits
  const double kLn2Lo = 1.9082149292705877e-10;  // ln 2 - kLn2Hi
  double k = std::nearbyint(x * kInvLn2);
  double r = (x - k * kLn2Hi) - k * kLn2Lo;
  // 1/i! for i = 13..0, correctly rounded
  static const double c[14] = {1.6059043836821613e-10, 2.08767569878681e-09, 2.505210838544172e-08,
                               2.755731922398589e-07, 2.7557319223985893e-06, 2.48015873015873e-05,
                               0.0001984126984126984, 0.001388888888888889, 0.008333333333333333,
                               0.041666666666666664, 0.16666666666666666, 0.5, 1.0, 1.0};
  double p = c[0];
  for (int i = 1; i < 14; ++i) p = p * r + c[i];
  return std::ldexp(p, (int)k);
}

// Number of Gauss-Hermite nodes for total power L (mod_intrastuff.f90:210-220).
inline int gh_nodes(int L) { return L / 2 + 1; }

// Largest root of the Hermite polynomial with n roots, n = t_i + t_k + 1
// (mod_intrastuff.f90:43-113, the x_max table of JA8).
inline double hermite_xmax(int n) { return inca_gh::kNode[n][n - 1]; }

struct Prim {
  double alpha, x[3];
  int t[3];
};

// JA8: upper bound J of the pair (i,k) for the first screening (mod_intrastuff.f90:32-123).
double ja8(const Prim& pi_, const Prim& pk, double Rik2, double aik, double eik) {
  int sumt = pi_.t[0] + pk.t[0] + pi_.t[1] + pk.t[1] + pi_.t[2] + pk.t[2];
  double s2a = std::sqrt(2.0 / aik);
  // pi^1.5 (2 aik)^-(sumt+1.5) e^(-2 eik Rik2) with (2a)^-(s+1.5) = 1/((2a)^(s+1) sqrt(2a))
  double two_a = 2.0 * aik;
  double v = kPi15 / (ipow(two_a, sumt + 1) * std::sqrt(two_a));
  v = v * pexp((-2.0 * eik) * Rik2);
  for (int d = 0; d < 3; ++d) {
    double xm = hermite_xmax(pi_.t[d] + pk.t[d] + 1);
    double dx = std::fabs(pk.x[d] - pi_.x[d]);
    v = v * ipow(xm + (pk.alpha * s2a) * dx, 2 * pi_.t[d]);
    v = v * ipow(xm + (pi_.alpha * s2a) * dx, 2 * pk.t[d]);
  }
  return v;
}

// LU with partial pivoting and solve, LAPACK dgesv semantics (dgetf2 + dgetrs): the pivot is
// the first entry of largest magnitude; info > 0 if an exact zero pivot occurs.
int lu_solve(int n, double* M /*row-major n*n*/, double* b) {
  int info = 0;
  int piv[kMaxCoef];
  for (int j = 0; j < n; ++j) {
    int p = j;
    double big = std::fabs(M[j * n + j]);
    for (int i = j + 1; i < n; ++i) {
      double a = std::fabs(M[i * n + j]);
      if (a > big) { big = a; p = i; }
    }
    piv[j] = p;
    if (M[p * n + j] != 0.0) {
      if (p != j)
        for (int c = 0; c < n; ++c) std::swap(M[j * n + c], M[p * n + c]);
      double inv = 1.0 / M[j * n + j];
      for (int i = j + 1; i < n; ++i) M[i * n + j] *= inv;
    } else if (info == 0) {
      info = j + 1;
    }
    for (int i = j + 1; i < n; ++i) {
      double l = M[i * n + j];
      for (int c = j + 1; c < n; ++c) M[i * n + c] -= l * M[j * n + c];
    }
  }
  if (info) return info;
  for (int j = 0; j < n; ++j)
    if (piv[j] != j) std::swap(b[j], b[piv[j]]);
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < i; ++c) b[i] -= M[i * n + c] * b[c];
  for (int i = n - 1; i >= 0; --i) {
    for (int c = i + 1; c < n; ++c) b[i] -= M[i * n + c] * b[c];
    b[i] /= M[i * n + i];
  }
  return 0;
}

// polycoef: coefficients (highest degree first) of the per-dimension polynomial V(r') that
// interpolates sum_h w_h W(rh_h, x_m) at x_m = m - 1/2 (mod_intrastuff.f90:127-194).
// Returns the LAPACK info; coefficients are zeroed if info != 0 or any |C| > 1e3.
int polycoef(const double R[4], double Pik, double Pjl, double Pijkl, const int t[4], double sqe,
             double invz, double alf, double* C) {
  int L = t[0] + t[1] + t[2] + t[3];
  int np = L + 1;
  int nn = gh_nodes(L);
  const double* rh = inca_gh::kNode[nn];
  const double* wh = inca_gh::kWeight[nn];
  if (np == 1) {
    C[0] = wh[0];
    return 0;
  }
  double M[kMaxCoef * kMaxCoef];
  for (int i = 0; i < np; ++i) {
    double xx = -0.5 + double(i + 1);
    double base = sqe * ((xx + Pik) - Pjl);
    for (int j = 0; j < np; ++j) M[i * np + j] = ipow(base, L - j);
    double rhs = 0.0;
    double am = (alf - 0.5) * xx, ap = (alf + 0.5) * xx;
    for (int h = 0; h < nn; ++h) {
      double zr = invz * rh[h];
      double W = ipow((zr + am) + (Pijkl - R[0]), t[0]) * ipow((zr + ap) + (Pijkl - R[1]), t[1]);
      W = W * ipow((zr + am) + (Pijkl - R[2]), t[2]);
      W = W * ipow((zr + ap) + (Pijkl - R[3]), t[3]);
      rhs = rhs + wh[h] * W;
    }
    C[i] = rhs;
  }
  int info = lu_solve(np, M, C);
  bool blow = false;
  for (int i = 0; i < np; ++i)
    if (std::fabs(C[i]) > 1e3) blow = true;
  if (info != 0 || blow)
    for (int i = 0; i < np; ++i) C[i] = 0.0;
  return info;
}

// One surviving quartet: everything the point loop needs (mod_intracule.f90:307-343).
struct Quartet {
  double A, sqe, d[3];  // d = P_ik - P_jl
  int L[3];
  double C[3][kMaxCoef];
};

struct Setup {
  std::vector<Prim> prims;
  std::vector<double> norm;
  double wm[kMaxCoef + 8];
  double lim;
};

void make_setup(Setup& S, int nprim, const double* alpha, const int* tmn, const double* xyz,
                int normalize, double thresh) {
  S.prims.resize(nprim);
  S.norm.assign(nprim, 1.0);
  for (int p = 0; p < nprim; ++p) {
    S.prims[p].alpha = alpha[p];
    for (int d = 0; d < 3; ++d) {
      S.prims[p].t[d] = tmn[p * 3 + d];
      S.prims[p].x[d] = xyz[p * 3 + d];
    }
    if (normalize) {  // normprim (mod_intracule.f90:145-152)
      const Prim& q = S.prims[p];
      int L = q.t[0] + q.t[1] + q.t[2];
      double df = double(dfact(2 * q.t[0] - 1) * dfact(2 * q.t[1] - 1) * dfact(2 * q.t[2] - 1));
      S.norm[p] = std::pow(2.0 * q.alpha / kPi, 0.75) *
                  std::sqrt(std::pow(4.0 * q.alpha, double(L)) * (1.0 / df));
    }
  }
  // wmarray (mod_intracule.f90:136-143): w_1 = 1, w_m = (m/2)^(m/2) e^(-m/2)
  for (int m = 1; m <= kMaxCoef + 8; ++m)
    S.wm[m - 1] = (m == 1) ? 1.0 : std::pow(double(m) * 0.5, double(m) * 0.5) * std::exp(-double(m) * 0.5);
  // lim = thresh / (nprim (nprim+1) / 2)  (mod_intracule.f90:163)
  S.lim = thresh * (1.0 / (double(nprim) * (double(nprim) + 1.0) * 0.5));
}

// Screening and set-up of one quartet (mod_intracule.f90:282-343). Returns a bitmask
// (1 = passed screen 1, 2 = passed screen 2) and fills q when both pass.
// Jtab (optional): JA8 of every primitive pair, Jtab[i * nprim + k], computed by ja8 with the
// same arguments as here (so the same bits).
int prepare_one(const Setup& S, int i, int j, int k, int l, double v, Quartet* q, double* s1out,
                double* s2out, const double* Jtab = nullptr) {
  const Prim &Pi = S.prims[i], &Pj = S.prims[j], &Pk = S.prims[k], &Pl = S.prims[l];
  double DMval = v * (S.norm[i] * S.norm[j] * S.norm[k] * S.norm[l]);
  double aik = Pi.alpha + Pk.alpha, ajl = Pj.alpha + Pl.alpha;
  double eik = Pi.alpha * Pk.alpha * (1.0 / aik), ejl = Pj.alpha * Pl.alpha * (1.0 / ajl);
  double Rik2 = 0, Rjl2 = 0;
  for (int d = 0; d < 3; ++d) {
    Rik2 += (Pi.x[d] - Pk.x[d]) * (Pi.x[d] - Pk.x[d]);
    Rjl2 += (Pj.x[d] - Pl.x[d]) * (Pj.x[d] - Pl.x[d]);
  }
  const size_t np = S.prims.size();
  double Jik = Jtab ? Jtab[i * np + k] : ja8(Pi, Pk, Rik2, aik, eik);
  double Jjl = Jtab ? Jtab[j * np + l] : ja8(Pj, Pl, Rjl2, ajl, ejl);
  double screen1 = std::fabs(DMval) * std::sqrt(Jik * Jjl);
  if (s1out) *s1out = screen1;
  if (!(screen1 >= S.lim)) return 0;
  double zeta = aik + ajl;
  double eijkl = (aik * ajl) * (1.0 / zeta);
  double sqe = std::sqrt(eijkl);
  double Pik[3], Pjl[3], Pijkl[3];
  for (int d = 0; d < 3; ++d) {
    Pik[d] = (Pi.alpha * Pi.x[d] + Pk.alpha * Pk.x[d]) * (1.0 / aik);
    Pjl[d] = (Pj.alpha * Pj.x[d] + Pl.alpha * Pl.x[d]) * (1.0 / ajl);
  }
  for (int d = 0; d < 3; ++d) Pijkl[d] = (aik * Pik[d] + ajl * Pjl[d]) * (1.0 / zeta);
  double invz = 1.0 / std::sqrt(zeta);
  double alf = (0.5 * (aik - ajl)) * (1.0 / zeta);
  double A = DMval * (1.0 / (zeta * std::sqrt(zeta)));
  A = A * pexp((-eik) * Rik2 - ejl * Rjl2);
  Quartet Q;
  double U[3];
  for (int d = 0; d < 3; ++d) {
    double R[4] = {Pi.x[d], Pj.x[d], Pk.x[d], Pl.x[d]};
    int t[4] = {Pi.t[d], Pj.t[d], Pk.t[d], Pl.t[d]};
    Q.L[d] = t[0] + t[1] + t[2] + t[3];
    polycoef(R, Pik[d], Pjl[d], Pijkl[d], t, sqe, invz, alf, Q.C[d]);
    U[d] = 0.0;
    for (int m = 0; m <= Q.L[d]; ++m) U[d] = U[d] + Q.C[d][m] * S.wm[m];
  }
  double screen2 = std::fabs(((A * U[0]) * U[1]) * U[2]);
  if (s2out) *s2out = screen2;
  if (!(screen2 >= S.lim)) return 1;
  Q.A = A;
  Q.sqe = sqe;
  for (int d = 0; d < 3; ++d) Q.d[d] = Pik[d] - Pjl[d];
  if (q) *q = Q;
  return 3;
}

// The point loop (mod_intracule.f90:345-358): Ivec[g] += A exp(-|r'|^2) Vx Vy Vz.
inline void accumulate(const Quartet& Q, long ngrid, const double* r, double* Iv) {
  for (long g = 0; g < ngrid; ++g) {
    double rp[3], V[3];
    for (int d = 0; d < 3; ++d) {
      rp[d] = Q.sqe * (r[3 * g + d] + Q.d[d]);
      double acc = 0.0;
      for (int m = 0; m <= Q.L[d]; ++m) acc = acc * rp[d] + Q.C[d][m];
      V[d] = acc;
    }
    Iv[g] += Q.A * std::exp(-(rp[0] * rp[0] + rp[1] * rp[1] + rp[2] * rp[2])) * V[0] * V[1] * V[2];
  }
}

// Becke/TFVC partition weights (mod_build_grid.f90:474-575).
double tfvc_fk(double v) {
  for (int i = 0; i < 4; ++i) v = 1.5 * v - 0.5 * ((v * v) * v);  // pf: 1.5 v - 0.5 v**3
  return v;
}

}  // namespace

extern "C" {

int orc_lebedev(int nang, double* x, double* y, double* z, double* w) {
  std::vector<double> a, b, c, v;
  if (lebedev(nang, a, b, c, v)) return -1;
  for (int i = 0; i < nang; ++i) { x[i] = a[i]; y[i] = b[i]; z[i] = c[i]; w[i] = v[i]; }
  return 0;
}

int orc_gauleg(int n, double* t, double* w) {
  gauleg(n, t, w);
  return 0;
}

double orc_normprim(double alpha, int t, int m, int n) {
  Setup S;
  int tmn[3] = {t, m, n};
  double xyz[3] = {0, 0, 0};
  make_setup(S, 1, &alpha, tmn, xyz, 1, 1.0);
  return S.norm[0];
}

// Dense LU solve (exposed for the dgesv cross-check). M row-major, overwritten.
int orc_lu_solve(int n, double* M, double* b) { return lu_solve(n, M, b); }

// Automatic integration centres (mod_autogrid.f90:12-185, centercalc + get_bs_radius).
// cartes is natoms x 3 row-major (bohr). Output arrays must hold natoms*(natoms-1)+1 entries.
int orc_centercalc(int natoms, const int* an, const double* cartes, int nohydro, int betaone,
                   int* nquad_out, double* cent, double* Ps, double* sfalpha) {
  auto bs = [](int z) -> double {
    double r;
    switch (z) {
      case 1: r = 0.35; break;  case 2: r = 0.35; break;  case 3: r = 1.45; break;
      case 4: r = 1.05; break;  case 5: r = 0.85; break;  case 6: r = 0.70; break;
      case 7: r = 0.65; break;  case 8: r = 0.60; break;  case 9: r = 0.50; break;
      case 10: r = 0.38; break; case 11: r = 1.80; break; case 12: r = 1.50; break;
      case 13: r = 1.25; break; case 14: r = 1.10; break; case 15: r = 1.00; break;
      case 16: r = 1.00; break; case 17: r = 1.00; break; case 19: r = 2.20; break;
      case 20: r = 1.80; break; case 21: r = 1.60; break; case 22: r = 1.40; break;
      case 23: r = 1.35; break; case 24: r = 1.40; break; case 25: r = 1.40; break;
      case 26: r = 1.40; break; case 27: r = 1.35; break; case 28: r = 1.35; break;
      case 29: r = 1.35; break; case 30: r = 1.35; break; case 31: r = 1.30; break;
      case 32: r = 1.25; break; case 33: r = 1.15; break; case 34: r = 1.15; break;
      case 35: r = 1.15; break; default: r = 1.00; break;
    }
    return r * 1.8897;
  };
  int nqmax = natoms * (natoms - 1) + 1;
  std::vector<double> c1(3 * nqmax, 0.0), ne(nqmax, 0.0), al(nqmax, 0.0);
  double tot = 0, wsum = 0;
  for (int i = 0; i < natoms; ++i) {
    double rj = bs(an[i]);
    double pairs = an[i] * (an[i] - 1.0) / 2.0;
    tot += pairs;
    wsum += pairs * rj;
  }
  ne[0] = tot;
  al[0] = tot > 1e-15 ? wsum / tot : bs(1);
  int sm = 0;
  for (int j = 0; j < natoms - 1; ++j)
    for (int k = j + 1; k < natoms; ++k) {
      if (!nohydro || (an[j] > 1 && an[k] > 1)) {
        ++sm;
        for (int d = 0; d < 3; ++d) c1[3 * sm + d] = cartes[3 * j + d] - cartes[3 * k + d];
        ne[sm] = an[j] * an[k] * 0.5;
        al[sm] = (bs(an[j]) + bs(an[k])) / 2.0;
        if (std::fabs(c1[3 * sm + 2]) < 0.5) c1[3 * sm + 2] = 0.0;
        int smp = sm;
        ++sm;
        for (int d = 0; d < 3; ++d) c1[3 * sm + d] = -c1[3 * smp + d];
        ne[sm] = ne[smp];
        al[sm] = al[smp];
      }
    }
  nqmax = sm + 1;
  int merged = 0;
  for (int i = 1; i < nqmax - 1; ++i) {
    double z = std::fabs(c1[3 * i]) + std::fabs(c1[3 * i + 1]) + std::fabs(c1[3 * i + 2]);
    if (z != 0.0) {
      for (int j = i + 1; j < nqmax; ++j) {
        bool eq = true;
        for (int d = 0; d < 3; ++d)
          if (!(std::fabs(c1[3 * i + d] - c1[3 * j + d]) < 0.1)) eq = false;
        if (eq) {
          al[i] = (al[i] * ne[i] + al[j] * ne[j]) / (ne[i] + ne[j]);
          ne[i] = ne[i] + ne[j];
          ++merged;
          c1[3 * j] = c1[3 * j + 1] = c1[3 * j + 2] = 0.0;
          ne[j] = 0.0;
        }
      }
    }
  }
  int nq = 0;
  for (int i = 0; i < nqmax; ++i) {
    double z = std::fabs(c1[3 * i]) + std::fabs(c1[3 * i + 1]) + std::fabs(c1[3 * i + 2]);
    if (i == 0 || z != 0.0) {
      for (int d = 0; d < 3; ++d) cent[3 * nq + d] = c1[3 * i + d];
      Ps[nq] = ne[i];
      sfalpha[nq] = al[i];
      ++nq;
    }
  }
  if (betaone)
    for (int i = 0; i < nq; ++i) { sfalpha[i] = 1.0; Ps[i] = 1.0; }
  *nquad_out = nq;
  return nq == nqmax - merged ? 0 : -1;
}

// Multicentre radial x Lebedev grid with z-halving and TFVC weights
// (mod_build_grid.f90:13-277). Outputs (capacity = sum nradc*nangc): points r (3 per point),
// weights w, Vee weights wvee, centre index (0-based). Returns the final point count.
long orc_gridpoints(int nquad, const int* nradc, const int* nangc, const double* sfalpha,
                    const double* cent, const double* Ps, int nosym, double* r_out, double* w_out,
                    double* wvee_out, int* cmap_out, long* maxgrid_out, long* rgrid_out) {
  const double pi = 4.0 * std::atan(1.0);
  const double tol = 1e-100, trsh2 = 1e-106;
  std::vector<double> gr, wt;
  std::vector<int> cm, smn(nquad, 0);
  long maxgrid = 0;
  for (int c = 0; c < nquad; ++c) maxgrid += (long)nradc[c] * nangc[c];
  for (int c = 0; c < nquad; ++c) {
    int nrad = nradc[c], nang = nangc[c];
    std::vector<double> xl(nrad), wl(nrad), rad(nrad), lx, ly, lz, lw;
    gauleg(nrad, xl.data(), wl.data());
    if (lebedev(nang, lx, ly, lz, lw)) return -1;
    for (int ir = 0; ir < nrad; ++ir) {
      rad[ir] = (1.0 + xl[ir]) / (1.0 - xl[ir]) * sfalpha[c];
      if (nquad > 1 && rad[ir] > 15.0)
        wl[ir] = 0.0;
      else
        wl[ir] = 2 * pi * (2.0 * sfalpha[c] / std::pow(1.0 - xl[ir], 2.0)) * wl[ir] * rad[ir] * rad[ir];
    }
    for (int ir = 0; ir < nrad; ++ir)
      for (int ia = 0; ia < nang; ++ia) {
        double p[3] = {rad[ir] * lx[ia] + cent[3 * c], rad[ir] * ly[ia] + cent[3 * c + 1],
                       rad[ir] * lz[ia] + cent[3 * c + 2]};
        double wgt;
        if (nosym) {
          wgt = lw[ia] * wl[ir];
        } else {
          if (!(p[2] >= -tol)) continue;
          wgt = (std::fabs(p[2]) < tol) ? lw[ia] * wl[ir] : 2.0 * lw[ia] * wl[ir];
        }
        gr.insert(gr.end(), p, p + 3);
        wt.push_back(wgt);
        cm.push_back(c);
        ++smn[c];
      }
  }
  long rgrid = (long)wt.size();
  if (nquad > 1) {
    // TFVC weights (mod_build_grid.f90:474-575)
    std::vector<double> Rij(nquad * nquad), Xi(nquad * nquad);
    for (int i = 0; i < nquad; ++i)
      for (int j = 0; j < nquad; ++j) {
        double s = 0;
        for (int d = 0; d < 3; ++d) s += std::pow(cent[3 * i + d] - cent[3 * j + d], 2.0);
        Rij[i * nquad + j] = std::sqrt(s);
        Xi[i * nquad + j] = Ps[j] > 1e-12 ? std::pow(Ps[i] / Ps[j], 1.0 / 3.0) : 1.0;
      }
#pragma omp parallel for schedule(static)
    for (long g = 0; g < rgrid; ++g) {
      std::vector<double> P(nquad);
      double ptot = 0;
      for (int i = 0; i < nquad; ++i) {
        P[i] = 1.0;
        for (int j = 0; j < nquad; ++j) {
          if (i == j) continue;
          double ri = 0, rj = 0;
          for (int d = 0; d < 3; ++d) {
            ri += std::pow(gr[3 * g + d] - cent[3 * i + d], 2.0);
            rj += std::pow(gr[3 * g + d] - cent[3 * j + d], 2.0);
          }
          ri = std::sqrt(ri);
          rj = std::sqrt(rj);
          double mu = Rij[i * nquad + j] > 1e-12 ? (ri - rj) * std::pow(Rij[i * nquad + j], -1.0) : 0.0;
          double term = Xi[i * nquad + j] * (1.0 - mu);
          double vij = (1.0 + mu - term) / (1.0 + mu + term);
          P[i] *= 0.5 * (1.0 - tfvc_fk(vij));
        }
        ptot += P[i];
      }
      double wb = P[cm[g]];
      if (ptot > 1e-15) wb = wb * std::pow(ptot, -1.0);
      wt[g] *= wb;
    }
  }
  long n = 0;
  for (long g = 0; g < rgrid; ++g) {
    if (!(wt[g] > trsh2)) continue;
    double dist = std::sqrt(gr[3 * g] * gr[3 * g] + gr[3 * g + 1] * gr[3 * g + 1] + gr[3 * g + 2] * gr[3 * g + 2]);
    for (int d = 0; d < 3; ++d) r_out[3 * n + d] = gr[3 * g + d];
    w_out[n] = wt[g];
    wvee_out[n] = wt[g] * std::pow(dist, -1.0);
    cmap_out[n] = cm[g];
    ++n;
  }
  if (maxgrid_out) *maxgrid_out = maxgrid;
  if (rgrid_out) *rgrid_out = rgrid;
  return n;
}

// Radial-scan shells (mod_build_grid.f90:281-408). Capacity of r/w_ang: sum npb*nang.
// Outputs: points, angular weights, points per shell (smn), shell radii (radi), nradi.
long orc_gridpoints2(int nblock, const double* start, const double* end, const double* step,
                     const int* nang, int nosym, double* r_out, double* wang_out, int* smn_out,
                     double* radi_out, int* nradi_out) {
  const double tol = std::sqrt(2.220446049250313e-16);
  int nr = 0;
  std::vector<int> npb(nblock);
  for (int b = 0; b < nblock; ++b) {
    npb[b] = (int)((end[b] - start[b]) / step[b]) + 1;
    nr += npb[b];
  }
  int sr = 0;
  for (int b = 0; b < nblock; ++b)
    for (int j = 0; j < npb[b]; ++j) radi_out[sr++] = start[b] + step[b] * double(j);
  long n = 0;
  int shell = 0;
  for (int b = 0; b < nblock; ++b) {
    std::vector<double> lx, ly, lz, lw;
    if (lebedev(nang[b], lx, ly, lz, lw)) return -1;
    for (int ir = 0; ir < npb[b]; ++ir, ++shell) {
      smn_out[shell] = 0;
      double s = radi_out[shell];
      for (int ia = 0; ia < nang[b]; ++ia) {
        double z = s * lz[ia];
        if (!nosym && !(z >= -tol)) continue;
        r_out[3 * n] = s * lx[ia];
        r_out[3 * n + 1] = s * ly[ia];
        r_out[3 * n + 2] = z;
        wang_out[n] = (nosym || std::fabs(z) < tol) ? lw[ia] : 2.0 * lw[ia];
        ++smn_out[shell];
        ++n;
      }
    }
  }
  *nradi_out = nr;
  return n;
}

// Uniform cube lattice, x outer / z inner (mod_build_grid.f90:412-440).
long orc_gridpoints3(const double* center, const double* step, const int* np, double* r_out) {
  double xm[3];
  for (int i = 0; i < 3; ++i) {
    if (std::fmod(double(np[i]), 2.0) == 0.0)
      xm[i] = center[i] - (step[i] / 2.0) - ((double(np[i]) - 2.0) / 2.0) * step[i];
    else
      xm[i] = center[i] - ((double(np[i]) - 1.0) / 2.0) * step[i];
  }
  long n = 0;
  for (int i = 0; i < np[0]; ++i)
    for (int j = 0; j < np[1]; ++j)
      for (int k = 0; k < np[2]; ++k) {
        r_out[3 * n] = xm[0] + step[0] * i;
        r_out[3 * n + 1] = xm[1] + step[1] * j;
        r_out[3 * n + 2] = xm[2] + step[2] * k;
        ++n;
      }
  return n;
}

// Per-quartet screening (mod_intracule.f90:282-343). ijkl: 1-based, 4 per quartet.
// flags[q] = 0 (fails screen 1), 1 (passes 1, fails 2), 3 (passes both).
// Optional outputs s1/s2: the screening values (s2 only where screen 1 passed).
// Survivor records (optional, capacity nq): A, sqe, d[3], L[3], C[3][17] (highest first).
long orc_prepare(int nprim, const double* alpha, const int* tmn, const double* xyz, int normalize,
                 double thresh, long nq, const int* ijkl, const double* v, unsigned char* flags,
                 double* s1, double* s2, double* recA, double* recSqe, double* recD, int* recL,
                 double* recC, long* counts) {
  Setup S;
  make_setup(S, nprim, alpha, tmn, xyz, normalize, thresh);
  long n1 = 0, n2 = 0;
  std::vector<long> pos(nq, -1);
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : n1, n2)
  for (long q = 0; q < nq; ++q) {
    Quartet Q;
    double a1 = 0, a2 = 0;
    int f = prepare_one(S, ijkl[4 * q] - 1, ijkl[4 * q + 1] - 1, ijkl[4 * q + 2] - 1,
                        ijkl[4 * q + 3] - 1, v[q], &Q, &a1, &a2);
    if (flags) flags[q] = (unsigned char)f;
    if (s1) s1[q] = a1;
    if (s2) s2[q] = (f & 1) ? a2 : 0.0;
    if (f & 1) ++n1;
    if (f & 2) ++n2;
  }
  if (recA) {
    long s = 0;
    for (long q = 0; q < nq; ++q) {
      Quartet Q;
      if (prepare_one(S, ijkl[4 * q] - 1, ijkl[4 * q + 1] - 1, ijkl[4 * q + 2] - 1,
                      ijkl[4 * q + 3] - 1, v[q], &Q, nullptr, nullptr) != 3)
        continue;
      recA[s] = Q.A;
      recSqe[s] = Q.sqe;
      for (int d = 0; d < 3; ++d) {
        recD[3 * s + d] = Q.d[d];
        recL[3 * s + d] = Q.L[d];
        for (int m = 0; m < kMaxCoef; ++m) recC[(s * 3 + d) * kMaxCoef + m] = m <= Q.L[d] ? Q.C[d][m] : 0.0;
      }
      ++s;
    }
  }
  if (counts) { counts[0] = nq; counts[1] = n1; counts[2] = n2; }
  return n2;
}

// The full hot path: screening + point loop over all quartets, with the reference's
// structure (mod_intracule.f90:203-388): batches of 40960 records, dynamic schedule, a
// private Ivec per thread, reduced at the end (here in thread order, for reproducibility).
// r: 3 per point. Ivec: ngrid outputs. counts: read / after screen 1 / after screen 2.
int orc_intracule(int nprim, const double* alpha, const int* tmn, const double* xyz, int normalize,
                  double thresh, long nq, const int* ijkl, const double* v, long ngrid,
                  const double* r, double* Ivec, long* counts, int nthreads) {
  Setup S;
  make_setup(S, nprim, alpha, tmn, xyz, normalize, thresh);
  const long kBatch = 40960;
  if (nthreads > 0) omp_set_num_threads(nthreads);
  int nt = 1;
#pragma omp parallel
  {
#pragma omp single
    nt = omp_get_num_threads();
  }
  std::vector<std::vector<double>> priv(nt, std::vector<double>(ngrid, 0.0));
  long n1 = 0, n2 = 0;
  for (long b0 = 0; b0 < nq; b0 += kBatch) {
    long b1 = std::min(nq, b0 + kBatch);
#pragma omp parallel for schedule(dynamic) reduction(+ : n1, n2)
    for (long q = b0; q < b1; ++q) {
      Quartet Q;
      int f = prepare_one(S, ijkl[4 * q] - 1, ijkl[4 * q + 1] - 1, ijkl[4 * q + 2] - 1,
                          ijkl[4 * q + 3] - 1, v[q], &Q, nullptr, nullptr);
      if (f & 1) ++n1;
      if (f & 2) {
        ++n2;
        accumulate(Q, ngrid, r, priv[omp_get_thread_num()].data());
      }
    }
  }
  for (long g = 0; g < ngrid; ++g) {
    double s = 0.0;
    for (int t = 0; t < nt; ++t) s += priv[t][g];
    Ivec[g] = s;
  }
  if (counts) { counts[0] = nq; counts[1] = n1; counts[2] = n2; }
  return 0;
}

// The hot path over a closed-shell DM2 generated from the 1-RDM D (nprim x nprim, column-major)
// instead of read from a file: Gamma_{ik,jl} = D_ik D_jl - 1/2 D_il D_jk summed over the distinct
// orderings (i,k)/(k,i) x (j,l)/(l,j), records (i,j,k,l) with i <= k and j <= l; unique != 0
// keeps pair(ik) <= pair(jl) and doubles the off-diagonal pairs. The records are enumerated and
// their values formed exactly as the library's device generator does (pairs in row-major packed
// order), so screening sees the same values; they are evaluated in batches of 40960 as
// orc_intracule does, without storing the list (the full lists of the larger synthetic workloads
// do not fit in host memory as records).
int orc_intracule_closed_shell(int nprim, const double* alpha, const int* tmn, const double* xyz, int normalize,
                               double thresh, const double* D, int unique, long ngrid, const double* r,
                               double* Ivec, long* counts, int nthreads) {
  Setup S;
  make_setup(S, nprim, alpha, tmn, xyz, normalize, thresh);
  const long n = nprim;
  std::vector<double> Jtab(n * n);
  for (long i = 0; i < n; ++i)
    for (long k = 0; k < n; ++k) {
      const Prim &Pi = S.prims[i], &Pk = S.prims[k];
      const double aik = Pi.alpha + Pk.alpha, eik = Pi.alpha * Pk.alpha * (1.0 / aik);
      double Rik2 = 0;
      for (int d = 0; d < 3; ++d) Rik2 += (Pi.x[d] - Pk.x[d]) * (Pi.x[d] - Pk.x[d]);
      Jtab[i * n + k] = ja8(Pi, Pk, Rik2, aik, eik);
    }
  const long npair = n * (n + 1) / 2;
  const long nrec = unique ? npair * (npair + 1) / 2 : npair * npair;
  // packed pair p -> (a, b), a <= b, rows a = 0..m-1 of m - a entries
  auto unpack = [](long p, long m, long* a, long* b) {
    long lo = 0, hi = m - 1;
    while (lo < hi) {
      const long mid = (lo + hi + 1) / 2;
      if (mid * m - mid * (mid - 1) / 2 <= p) lo = mid; else hi = mid - 1;
    }
    *a = lo;
    *b = lo + (p - (lo * m - lo * (lo - 1) / 2));
  };
  auto gam = [&](long i, long k, long j, long l) {
    return D[i + n * k] * D[j + n * l] - 0.5 * D[i + n * l] * D[j + n * k];
  };
  if (nthreads > 0) omp_set_num_threads(nthreads);
  int nt = 1;
#pragma omp parallel
  {
#pragma omp single
    nt = omp_get_num_threads();
  }
  std::vector<std::vector<double>> priv(nt, std::vector<double>(ngrid, 0.0));
  long n1 = 0, n2 = 0;
  const long kBatch = 40960;
  for (long b0 = 0; b0 < nrec; b0 += kBatch) {
    const long b1 = std::min(nrec, b0 + kBatch);
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : n1, n2)
    for (long rr = b0; rr < b1; ++rr) {
      long pa, pb, i, k, j, l;
      if (unique) unpack(rr, npair, &pa, &pb); else { pa = rr / npair; pb = rr % npair; }
      unpack(pa, n, &i, &k);
      unpack(pb, n, &j, &l);
      const long ik[2][2] = {{i, k}, {k, i}}, jl[2][2] = {{j, l}, {l, j}};
      const int nik = (i == k) ? 1 : 2, njl = (j == l) ? 1 : 2;
      double v = 0.0;
      for (int a = 0; a < nik; ++a)
        for (int b = 0; b < njl; ++b) v += gam(ik[a][0], ik[a][1], jl[b][0], jl[b][1]);
      if (unique && pa != pb) v *= 2.0;
      Quartet Q;
      const int f = prepare_one(S, int(i), int(j), int(k), int(l), v, &Q, nullptr, nullptr, Jtab.data());
      if (f & 1) ++n1;
      if (f & 2) {
        ++n2;
        accumulate(Q, ngrid, r, priv[omp_get_thread_num()].data());
      }
    }
  }
  for (long g = 0; g < ngrid; ++g) {
    double s = 0.0;
    for (int t = 0; t < nt; ++t) s += priv[t][g];
    Ivec[g] = s;
  }
  if (counts) { counts[0] = nrec; counts[1] = n1; counts[2] = n2; }
  return 0;
}

// Point loop only, over survivor records in the layout written by orc_prepare.
int orc_eval_records(long ns, const double* recA, const double* recSqe, const double* recD,
                     const int* recL, const double* recC, long ngrid, const double* r, double* Ivec) {
  int nt = 1;
#pragma omp parallel
  {
#pragma omp single
    nt = omp_get_num_threads();
  }
  std::vector<std::vector<double>> priv(nt, std::vector<double>(ngrid, 0.0));
#pragma omp parallel for schedule(dynamic, 16)
  for (long s = 0; s < ns; ++s) {
    Quartet Q;
    Q.A = recA[s];
    Q.sqe = recSqe[s];
    for (int d = 0; d < 3; ++d) {
      Q.d[d] = recD[3 * s + d];
      Q.L[d] = recL[3 * s + d];
      for (int m = 0; m < kMaxCoef; ++m) Q.C[d][m] = recC[(s * 3 + d) * kMaxCoef + m];
    }
    accumulate(Q, ngrid, r, priv[omp_get_thread_num()].data());
  }
  for (long g = 0; g < ngrid; ++g) {
    double s = 0.0;
    for (int t = 0; t < nt; ++t) s += priv[t][g];
    Ivec[g] = s;
  }
  return 0;
}

// Gaussian-smeared radial distribution from the multicentre grid
// (mod_intracule.f90:576-649). Outputs u_axis, P_u, I_avg (n_bins each).
int orc_radial_smearing(long ngrid, const double* r, const double* w, const double* dens,
                        double u_max, int n_bins, double sigma, double* u_axis, double* P_u,
                        double* I_avg) {
  const double pi = 4.0 * std::atan(1.0);
  double bw = u_max / double(n_bins - 1);
  for (int j = 0; j < n_bins; ++j) { u_axis[j] = double(j) * bw; P_u[j] = 0.0; }
  double pref = 1.0 / (sigma * std::sqrt(2.0 * pi));
  for (long i = 0; i < ngrid; ++i) {
    double ui = std::sqrt(r[3 * i] * r[3 * i] + r[3 * i + 1] * r[3 * i + 1] + r[3 * i + 2] * r[3 * i + 2]);
    double val = w[i] * dens[i];
    int jmin = std::max(1, (int)((ui - 4.0 * sigma) / bw) + 1);
    int jmax = std::min(n_bins, (int)((ui + 4.0 * sigma) / bw) + 1);
    for (int j = jmin; j <= jmax; ++j) {
      double dist = u_axis[j - 1] - ui;
      P_u[j - 1] += val * (pref * std::exp(-(dist * dist) / (2.0 * sigma * sigma)));
    }
  }
  for (int j = 0; j < n_bins; ++j)
    I_avg[j] = u_axis[j] > 1e-6 ? P_u[j] * (1.0 / (4.0 * pi * u_axis[j] * u_axis[j])) : 0.0;
  return 0;
}

}  // extern "C"
