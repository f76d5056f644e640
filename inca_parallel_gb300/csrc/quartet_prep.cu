// K1: per-quartet screening and set-up on the device (FP64).
//
// Restates the per-quartet part of calculate_intracule (src/mod_intracule.f90:282-343) and
// its helpers JA8 / polycoef / gauherm (src/mod_intrastuff.f90:32-341): normalisation,
// screen 1 |v| sqrt(J_ik J_jl) >= lim, Gaussian products, the three per-dimension
// polynomials (Gauss-Hermite right-hand side, Vandermonde system solved by LU with partial
// pivoting, zeroed on a singular matrix or |C| > 1e3) and screen 2 |A Ux Uy Uz| >= lim.
//
// One thread per quartet. The arithmetic is spelled out operation by operation (integer
// powers by repeated multiplication, half-integer powers through sqrt, a Cody-Waite/Taylor
// exponential) and this translation unit is compiled with -fmad=false, so every screening
// value is bit-identical to the CPU oracle's and the screening decisions are identical.
//
// Survivors are then sorted by angular class (Lx, Ly, Lz) with a stable radix sort and
// written as class-segmented FP64 records (for the FP64 evaluation) and FP32 records (for
// the mixed evaluation, see intracule_eval.cu for their use).
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "hermite_table.h"
#include "inca_internal.h"

namespace inca {
namespace {


struct PrepConst {
  double wm[kMaxCoef];
  double gh_node[kMaxGH + 1][kMaxGH];
  double gh_w[kMaxGH + 1][kMaxGH];
  double pi15;
  double thresh;
  double c_u;  // sqrt(1/ln 2): u = c_u r' turns e^(-r'^2) into 2^(-u^2)
  int nprim;
  int normalize;
};
__constant__ PrepConst cP;

__device__ __forceinline__ double ipow(double x, int n) {
  if (n <= 0) return 1.0;
  double r = x;
  for (int i = 1; i < n; ++i) r = r * x;
  return r;
}

// Cody-Waite reduction x = k ln2 + r (ln2 with a 32-bit head), Taylor degree 13 by Horner.
__device__ double pexp(double x) {
  if (x != x) return x;
  if (x > 709.0) return HUGE_VAL;
  if (x < -708.0) return 0.0;
  const double kInvLn2 = 1.4426950408889634;
  const double kLn2Hi = 0.6931471803691238;
  const double kLn2Lo = 1.9082149292705877e-10;
  const double k = rint(x * kInvLn2);
  const double r = (x - k * kLn2Hi) - k * kLn2Lo;
  const double c[14] = {1.6059043836821613e-10, 2.08767569878681e-09, 2.505210838544172e-08,
                        2.755731922398589e-07, 2.7557319223985893e-06, 2.48015873015873e-05,
                        0.0001984126984126984, 0.001388888888888889, 0.008333333333333333,
                        0.041666666666666664, 0.16666666666666666, 0.5, 1.0, 1.0};
  double p = c[0];
#pragma unroll
  for (int i = 1; i < 14; ++i) p = p * r + c[i];
  return ldexp(p, static_cast<int>(k));
}

__device__ __forceinline__ double xmax(int n) { return cP.gh_node[n][n - 1]; }

// JA8 (src/mod_intrastuff.f90:32-123).
__device__ double ja8(const PrimD& a, const PrimD& b, double R2, double aik, double eik) {
  const int sumt = a.t[0] + b.t[0] + a.t[1] + b.t[1] + a.t[2] + b.t[2];
  const double s2a = sqrt(2.0 / aik);
  const double two_a = 2.0 * aik;
  double v = cP.pi15 / (ipow(two_a, sumt + 1) * sqrt(two_a));
  v = v * pexp((-2.0 * eik) * R2);
  const double ax[3] = {a.x, a.y, a.z}, bx[3] = {b.x, b.y, b.z};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double xm = xmax(a.t[d] + b.t[d] + 1);
    const double dx = fabs(bx[d] - ax[d]);
    v = v * ipow(xm + (b.alpha * s2a) * dx, 2 * a.t[d]);
    v = v * ipow(xm + (a.alpha * s2a) * dx, 2 * b.t[d]);
  }
  return v;
}

// LU with partial pivoting (first maximum), reciprocal pivot scaling, then the two
// triangular solves: LAPACK dgesv semantics (dgetf2 + dgetrs). Returns info.
__device__ int lu_solve(int n, double* M, double* b) {
  int info = 0;
  int piv[kMaxCoef];
  for (int j = 0; j < n; ++j) {
    int p = j;
    double big = fabs(M[j * n + j]);
    for (int i = j + 1; i < n; ++i) {
      const double a = fabs(M[i * n + j]);
      if (a > big) { big = a; p = i; }
    }
    piv[j] = p;
    if (M[p * n + j] != 0.0) {
      if (p != j)
        for (int c = 0; c < n; ++c) {
          const double t = M[j * n + c];
          M[j * n + c] = M[p * n + c];
          M[p * n + c] = t;
        }
      const double inv = 1.0 / M[j * n + j];
      for (int i = j + 1; i < n; ++i) M[i * n + j] = M[i * n + j] * inv;
    } else if (info == 0) {
      info = j + 1;
    }
    for (int i = j + 1; i < n; ++i) {
      const double l = M[i * n + j];
      for (int c = j + 1; c < n; ++c) M[i * n + c] = M[i * n + c] - l * M[j * n + c];
    }
  }
  if (info) return info;
  for (int j = 0; j < n; ++j)
    if (piv[j] != j) {
      const double t = b[j];
      b[j] = b[piv[j]];
      b[piv[j]] = t;
    }
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < i; ++c) b[i] = b[i] - M[i * n + c] * b[c];
  for (int i = n - 1; i >= 0; --i) {
    for (int c = i + 1; c < n; ++c) b[i] = b[i] - M[i * n + c] * b[c];
    b[i] = b[i] / M[i * n + i];
  }
  return 0;
}

// polycoef (src/mod_intrastuff.f90:127-194); C highest degree first.
__device__ void polycoef(const double R[4], double Pik, double Pjl, double Pijkl, const int t[4],
                         double sqe, double invz, double alf, double* C) {
  const int L = t[0] + t[1] + t[2] + t[3];
  const int np = L + 1;
  const int nn = L / 2 + 1;
  if (np == 1) {
    C[0] = cP.gh_w[1][0];
    return;
  }
  double M[kMaxCoef * kMaxCoef];
  for (int i = 0; i < np; ++i) {
    const double xx = -0.5 + double(i + 1);
    const double base = sqe * ((xx + Pik) - Pjl);
    for (int j = 0; j < np; ++j) M[i * np + j] = ipow(base, L - j);
    const double am = (alf - 0.5) * xx, ap = (alf + 0.5) * xx;
    double rhs = 0.0;
    for (int h = 0; h < nn; ++h) {
      const double zr = invz * cP.gh_node[nn][h];
      double W = ipow((zr + am) + (Pijkl - R[0]), t[0]) * ipow((zr + ap) + (Pijkl - R[1]), t[1]);
      W = W * ipow((zr + am) + (Pijkl - R[2]), t[2]);
      W = W * ipow((zr + ap) + (Pijkl - R[3]), t[3]);
      rhs = rhs + cP.gh_w[nn][h] * W;
    }
    C[i] = rhs;
  }
  const int info = lu_solve(np, M, C);
  bool blow = false;
  for (int i = 0; i < np; ++i)
    if (fabs(C[i]) > 1e3) blow = true;
  if (info != 0 || blow)
    for (int i = 0; i < np; ++i) C[i] = 0.0;
}

struct QRec {
  double A, sqe, d[3];
  int L[3];
  double C[3][kMaxCoef];
};

// JA8 of every ordered primitive pair (i, k), with the arithmetic of prepare_one (Rik2, aik,
// eik), so a quartet's screen-1 value reads two table entries instead of evaluating JA8 twice
// and the values are the same bits.
__global__ void k_pair_ja8(int nprim, const PrimD* __restrict__ prims, double* __restrict__ J) {
  const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<int64_t>(nprim) * nprim) return;
  const PrimD Pi = prims[t / nprim], Pk = prims[t % nprim];
  const double aik = Pi.alpha + Pk.alpha;
  const double eik = (Pi.alpha * Pk.alpha) * (1.0 / aik);
  const double Xi[3] = {Pi.x, Pi.y, Pi.z}, Xk[3] = {Pk.x, Pk.y, Pk.z};
  double Rik2 = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d) Rik2 = Rik2 + (Xi[d] - Xk[d]) * (Xi[d] - Xk[d]);
  J[t] = ja8(Pi, Pk, Rik2, aik, eik);
}

constexpr int kPairTableMax = 4096;
// inca_prepare keeps its sort scratch (about 24 B per quartet plus the radix sort's temporary
// storage) in the context for lists of up to 2^26 quartets (about 1.6 GB)
constexpr int64_t kPrepKeepQuartets = int64_t(1) << 26;
// Up to this many quartets the screening kernel keeps each survivor's quartet (QRec, 272 B: at
// most 272 MiB) for the record build, which then reads it instead of repeating the FP64
// normalisation, Gaussian products and Vandermonde solves (same values, so the same bits);
// larger lists rebuild each survivor from its indices.
constexpr int64_t kQRecCacheQuartets = int64_t(1) << 20;

// One quartet (src/mod_intracule.f90:282-343). Returns 0 / 1 (screen 1) / 3 (both).
// Jtab (optional): the JA8 table of k_pair_ja8.
__device__ int prepare_one(const PrimD* prims, int4 q, double v, QRec* out, double* s1o,
                           double* s2o, const double* __restrict__ Jtab = nullptr) {
  const PrimD Pi = prims[q.x - 1], Pj = prims[q.y - 1], Pk = prims[q.z - 1], Pl = prims[q.w - 1];
  double DMval = v;
  if (cP.normalize) DMval = v * (((Pi.norm * Pj.norm) * Pk.norm) * Pl.norm);
  const double aik = Pi.alpha + Pk.alpha, ajl = Pj.alpha + Pl.alpha;
  const double eik = (Pi.alpha * Pk.alpha) * (1.0 / aik);
  const double ejl = (Pj.alpha * Pl.alpha) * (1.0 / ajl);
  const double Xi[3] = {Pi.x, Pi.y, Pi.z}, Xj[3] = {Pj.x, Pj.y, Pj.z};
  const double Xk[3] = {Pk.x, Pk.y, Pk.z}, Xl[3] = {Pl.x, Pl.y, Pl.z};
  double Rik2 = 0.0, Rjl2 = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    Rik2 = Rik2 + (Xi[d] - Xk[d]) * (Xi[d] - Xk[d]);
    Rjl2 = Rjl2 + (Xj[d] - Xl[d]) * (Xj[d] - Xl[d]);
  }
  const double Jik = Jtab ? Jtab[static_cast<int64_t>(q.x - 1) * cP.nprim + (q.z - 1)] : ja8(Pi, Pk, Rik2, aik, eik);
  const double Jjl = Jtab ? Jtab[static_cast<int64_t>(q.y - 1) * cP.nprim + (q.w - 1)] : ja8(Pj, Pl, Rjl2, ajl, ejl);
  const double lim = cP.thresh * Pi.lim_scale;
  const double screen1 = fabs(DMval) * sqrt(Jik * Jjl);
  *s1o = screen1;
  *s2o = 0.0;
  if (!(screen1 >= lim)) return 0;
  const double zeta = aik + ajl;
  const double eijkl = (aik * ajl) * (1.0 / zeta);
  const double sqe = sqrt(eijkl);
  double Pik[3], Pjl[3], Pijkl[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    Pik[d] = (Pi.alpha * Xi[d] + Pk.alpha * Xk[d]) * (1.0 / aik);
    Pjl[d] = (Pj.alpha * Xj[d] + Pl.alpha * Xl[d]) * (1.0 / ajl);
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) Pijkl[d] = (aik * Pik[d] + ajl * Pjl[d]) * (1.0 / zeta);
  const double invz = 1.0 / sqrt(zeta);
  const double alf = (0.5 * (aik - ajl)) * (1.0 / zeta);
  double A = DMval * (1.0 / (zeta * sqrt(zeta)));
  A = A * pexp((-eik) * Rik2 - ejl * Rjl2);
  double U[3];
  for (int d = 0; d < 3; ++d) {
    const double R[4] = {Xi[d], Xj[d], Xk[d], Xl[d]};
    const int t[4] = {Pi.t[d], Pj.t[d], Pk.t[d], Pl.t[d]};
    out->L[d] = t[0] + t[1] + t[2] + t[3];
    polycoef(R, Pik[d], Pjl[d], Pijkl[d], t, sqe, invz, alf, out->C[d]);
    U[d] = 0.0;
    for (int m = 0; m <= out->L[d]; ++m) U[d] = U[d] + out->C[d][m] * cP.wm[m];
  }
  const double screen2 = fabs(((A * U[0]) * U[1]) * U[2]);
  *s2o = screen2;
  if (!(screen2 >= lim)) return 1;
  out->A = A;
  out->sqe = sqe;
#pragma unroll
  for (int d = 0; d < 3; ++d) out->d[d] = Pik[d] - Pjl[d];
  return 3;
}

__device__ __forceinline__ uint32_t class_key(const int L[3]) {
  return (static_cast<uint32_t>(L[0]) << 10) | (static_cast<uint32_t>(L[1]) << 5) |
         static_cast<uint32_t>(L[2]);
}

__device__ __noinline__ int screen_one(int64_t q, const int4* __restrict__ ijkl, const double* __restrict__ v,
                                       const PrimD* __restrict__ prims, uint8_t* flags, double* s1, double* s2,
                                       uint32_t* key, int64_t* idx, int* bad_index, const double* Jtab,
                                       QRec* qcache);

// Pass 1: screening of every quartet; class key of survivors (others sort last).
__global__ void k_screen(int64_t n, const int4* __restrict__ ijkl, const double* __restrict__ v,
                         const PrimD* __restrict__ prims, uint8_t* flags, double* s1, double* s2,
                         uint32_t* key, int64_t* idx, int* bad_index,
                         unsigned long long* n_screen1, const double* __restrict__ Jtab, QRec* qcache) {
  const int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const bool live = q < n;
  int f = 0;
  if (live) f = screen_one(q, ijkl, v, prims, flags, s1, s2, key, idx, bad_index, Jtab, qcache);
  // warp-aggregated count of screen-1 survivors
  const unsigned ballot = __ballot_sync(0xffffffffu, live && (f & 1));
  if ((threadIdx.x & 31) == 0 && ballot) atomicAdd(n_screen1, static_cast<unsigned long long>(__popc(ballot)));
}

__device__ __noinline__ int screen_one(int64_t q, const int4* __restrict__ ijkl, const double* __restrict__ v,
                                       const PrimD* __restrict__ prims, uint8_t* flags, double* s1, double* s2,
                                       uint32_t* key, int64_t* idx, int* bad_index, const double* Jtab,
                                       QRec* qcache) {
  const int4 r = ijkl[q];
  idx[q] = q;
  if (r.x < 1 || r.y < 1 || r.z < 1 || r.w < 1 || r.x > cP.nprim || r.y > cP.nprim ||
      r.z > cP.nprim || r.w > cP.nprim) {
    atomicExch(bad_index, 1);
    flags[q] = 0;
    key[q] = 0xFFFFFFFFu;
    if (s1) s1[q] = 0.0;
    if (s2) s2[q] = 0.0;
    return 0;
  }
  QRec rec;
  double a1, a2;
  const int f = prepare_one(prims, r, v[q], &rec, &a1, &a2, Jtab);
  flags[q] = static_cast<uint8_t>(f);
  if (qcache && f == 3) qcache[q] = rec;
  if (s1) s1[q] = a1;
  if (s2) s2[q] = a2;
  // sort key: molecule (batches), then angular class; quartets that fail screening sort last
  key[q] = (f == 3) ? (static_cast<uint32_t>(prims[r.x - 1].mol) << 16) | class_key(rec.L) : 0xFFFFFFFFu;
  return f;
}

// Pass 2: rebuild each survivor (identical arithmetic) and write its records into the
// class segments:
//   FP64 record [A, sqe, d0, d1, d2, A', Cx.., Cy.., Cz..] (C highest degree first);
//   FP32 record [s_hi, s_lo, b_hi[3], b_lo[3], A'_hi, A'_lo, la, 0, Cn_hi (x,y,z), Cn_lo (x,y,z)]
// with s = sqe c_u, b_d = s d_d, u = s (r + d) = c_u r', the polynomials rewritten in u and
// scaled by kappa_d (largest |coefficient|) so that Cn has max |coefficient| 1, A' = A prod
// kappa_d, and la = log2(|A'| prod_d sum_k |Cn_dk|). hi/lo pairs carry the FP64 value to
// ~2^-48 relative (see mixed_eval.cu).
__global__ void k_build(int64_t nsurv, const int64_t* __restrict__ sorted_idx,
                        const int4* __restrict__ ijkl, const double* __restrict__ v,
                        const PrimD* __restrict__ prims, const ClassSeg* __restrict__ segs,
                        int nseg, double* rec64, float* rec32, int64_t* surv_src,
                        const double* __restrict__ Jtab, const QRec* __restrict__ qcache) {
  const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (p >= nsurv) return;
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {  // segment containing p
    const int mid = (lo + hi + 1) / 2;
    if (segs[mid].first <= p) lo = mid; else hi = mid - 1;
  }
  const ClassSeg sg = segs[lo];
  const int64_t src = sorted_idx[p];
  surv_src[p] = src;
  QRec rec;
  if (qcache) {
    rec = qcache[src];
  } else {
    double a1, a2;
    prepare_one(prims, ijkl[src], v[src], &rec, &a1, &a2, Jtab);
  }
  const int64_t local = p - sg.first;
  double* r64 = rec64 + sg.off64 + local * sg.stride;
  // u-space polynomials: V_d(r') = sum_k C_k r'^k = sum_k (C_k c^-k) u^k, u = c r'
  double Cu[3][kMaxCoef], kappa[3];
  double Bmax = 1.0;
  for (int d = 0; d < 3; ++d) {
    const int L = rec.L[d];
    double big = 0.0;
    for (int m = 0; m <= L; ++m) {
      const double ck = rec.C[d][m] * ipow(1.0 / cP.c_u, L - m);
      Cu[d][m] = ck;
      big = fmax(big, fabs(ck));
    }
    kappa[d] = big > 0.0 ? big : 1.0;
    Bmax = Bmax * kappa[d];
  }
  // a constant polynomial (L_d = 0) normalises to +-1: fold the sign into A' so the
  // evaluation can skip that dimension (V_d = 1 exactly)
  double sign = 1.0;
  for (int d = 0; d < 3; ++d)
    if (rec.L[d] == 0 && Cu[d][0] < 0.0) {
      sign = -sign;
      Cu[d][0] = -Cu[d][0];
    }
  const double Aprime = sign * rec.A * Bmax;
  r64[0] = rec.A;
  r64[1] = rec.sqe;
  r64[2] = rec.d[0];
  r64[3] = rec.d[1];
  r64[4] = rec.d[2];
  r64[5] = Aprime;
  int o = kRecHeader;
  for (int d = 0; d < 3; ++d)
    for (int m = 0; m <= rec.L[d]; ++m) r64[o++] = rec.C[d][m];
  for (; o < sg.stride; ++o) r64[o] = 0.0;

  float* r32 = rec32 + sg.off32 + local * sg.stride32;
  const double s = rec.sqe * cP.c_u;
  const float s_hi = static_cast<float>(s);
  r32[0] = s_hi;
  r32[1] = static_cast<float>(s - static_cast<double>(s_hi));
  for (int d = 0; d < 3; ++d) {
    const double b = s * rec.d[d];
    const float b_hi = static_cast<float>(b);
    r32[2 + d] = b_hi;
    r32[5 + d] = static_cast<float>(b - static_cast<double>(b_hi));
  }
  // A' = m 2^k with |m| in [0.5, 1): m as an FP32 pair, k applied exactly in the exponent
  // scaling of the evaluation's exp2 (A' itself can exceed the FP32 range for tight d shells)
  int kA = 0;
  const double mA = Aprime != 0.0 ? frexp(Aprime, &kA) : 0.0;
  const float A_hi = static_cast<float>(mA);
  r32[8] = A_hi;
  r32[9] = static_cast<float>(mA - static_cast<double>(A_hi));
  // log2 of |A'| prod_d sum_k |Cn_dk|: the tile bounds of the mixed evaluation start from it
  double la = log2(fabs(Aprime));
  for (int d = 0; d < 3; ++d) {
    double sd = 0.0;
    for (int m = 0; m <= rec.L[d]; ++m) sd += fabs(Cu[d][m] / kappa[d]);
    la += log2(sd);
  }
  r32[10] = static_cast<float>(la);
  r32[11] = static_cast<float>(kA);
  const int nc = rec.L[0] + rec.L[1] + rec.L[2] + 3;
  o = 12;
  for (int d = 0; d < 3; ++d)
    for (int m = 0; m <= rec.L[d]; ++m) {
      const double cn = Cu[d][m] / kappa[d];
      const float hi = static_cast<float>(cn);
      r32[o] = hi;
      r32[o + nc] = static_cast<float>(cn - static_cast<double>(hi));
      ++o;
    }
  for (o += nc; o < sg.stride32; ++o) r32[o] = 0.0f;
}

}  // namespace

int prepare_device(inca_ctx* c, double thresh, int normalize) {
  if (c->nprim <= 0) return set_error(c, INCA_E_STATE, "inca_prepare: primitives not set");
  if (c->nq <= 0) return set_error(c, INCA_E_STATE, "inca_prepare: no quartets loaded");
  if (!(thresh > 0.0)) return set_error(c, INCA_E_ARG, "inca_prepare: thresh must be > 0");
  for (int p = 0; p < c->nprim; ++p)
    for (int d = 0; d < 3; ++d)
      if (c->h_tmn[3 * p + d] < 0 || c->h_tmn[3 * p + d] > 4)
        return set_error(c, INCA_E_LIMIT, "inca_prepare: Cartesian power above 4 (g) in primitive " +
                                              std::to_string(p + 1));
  // constants (computed on the host with the same expressions as the reference)
  PrepConst hc;
  std::memset(&hc, 0, sizeof(hc));
  const double pi = 4.0 * std::atan(1.0);
  for (int m = 1; m <= kMaxCoef; ++m)
    hc.wm[m - 1] = (m == 1) ? 1.0 : std::pow(double(m) * 0.5, double(m) * 0.5) * std::exp(-double(m) * 0.5);
  for (int n = 0; n <= kMaxGH; ++n)
    for (int h = 0; h < kMaxGH; ++h) {
      hc.gh_node[n][h] = inca_gh::kNode[n][h];
      hc.gh_w[n][h] = inca_gh::kWeight[n][h];
    }
  hc.pi15 = pi * std::sqrt(pi);
  hc.thresh = thresh;
  hc.c_u = std::sqrt(1.0 / std::log(2.0));
  hc.nprim = c->nprim;
  hc.normalize = normalize ? 1 : 0;
  c->lim = thresh * (1.0 / (double(c->nprim) * (double(c->nprim) + 1.0) * 0.5));
  INCA_CUDA(c, cudaMemcpyToSymbolAsync(cP, &hc, sizeof(hc), 0, cudaMemcpyHostToDevice, c->stream));

  const int64_t n = c->nq;
  const bool keep_values = n <= (int64_t(1) << 27);
  if (c->d_flags.reserve(n) != cudaSuccess) return set_error(c, INCA_E_NOMEM, "flags");
  if (keep_values) {
    if (c->d_s1.reserve(n) != cudaSuccess || c->d_s2.reserve(n) != cudaSuccess)
      return set_error(c, INCA_E_NOMEM, "screening values");
  }
  c->have_screen_values = keep_values;
  // sort and run-length scratch, owned by the context: kept between calls for lists of up to
  // kPrepKeepQuartets quartets (a repeated preparation then allocates and frees nothing, and no
  // cudaFree stalls the stream), given back after the call for larger lists
  DevBuf<uint32_t>& key = c->d_pkey;
  DevBuf<uint32_t>& key2 = c->d_pkey2;
  DevBuf<int64_t>& idx = c->d_pidx;
  DevBuf<int64_t>& idx2 = c->d_pidx2;
  DevBuf<int>& bad = c->d_pbad;
  DevBuf<unsigned long long>& n1dev = c->d_pn1;
  DevBuf<unsigned char>& tmp = c->d_ptmp;
  DevBuf<uint32_t>& ukeys = c->d_pukeys;
  DevBuf<int64_t>& ucounts = c->d_pucounts;
  DevBuf<int>& nruns = c->d_pnruns;
  DevBuf<unsigned char>& qrec = c->d_pqrec;
  auto release_all = [&]() {
    key.release(); key2.release(); idx.release(); idx2.release(); bad.release(); n1dev.release();
    tmp.release(); ukeys.release(); ucounts.release(); nruns.release(); qrec.release();
  };
  const bool keep_scratch = n <= kPrepKeepQuartets;
  auto cleanup = [&]() {
    if (!keep_scratch) release_all();
  };
  if (key.reserve(n) || key2.reserve(n) || idx.reserve(n) || idx2.reserve(n) || bad.reserve(1) || n1dev.reserve(1)) {
    release_all();
    return set_error(c, INCA_E_NOMEM, "inca_prepare: sort buffers");
  }
  QRec* qcache = nullptr;
  if (n <= kQRecCacheQuartets) {
    if (qrec.reserve(sizeof(QRec) * std::max<int64_t>(n, 1)) == cudaSuccess)
      qcache = reinterpret_cast<QRec*>(qrec.p);
    else
      (void)cudaGetLastError();  // no room: build the records from the indices instead
  }
  cudaError_t e = cudaMemsetAsync(bad.p, 0, sizeof(int), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(n1dev.p, 0, sizeof(unsigned long long), c->stream);
  const int bs = 128;
  const int64_t grid = (n + bs - 1) / bs;
  // JA8 of every primitive pair, once (up to kPairTableMax primitives: 128 MiB); beyond that each
  // quartet evaluates its two JA8 bounds itself
  const double* jtab = nullptr;
  if (e == cudaSuccess && c->nprim <= kPairTableMax) {
    const int64_t np2 = static_cast<int64_t>(c->nprim) * c->nprim;
    if (c->d_ja8.reserve(np2) == cudaSuccess) {
      INCA_LAUNCH(c, k_pair_ja8, static_cast<unsigned>((np2 + 127) / 128), 128, 0, c->nprim, c->d_prims.p,
                  c->d_ja8.p);
      e = cudaGetLastError();
      jtab = c->d_ja8.p;
    }
  }
  if (e == cudaSuccess) {
    INCA_LAUNCH(c, k_screen, static_cast<unsigned>(grid), bs, 0, n, c->d_ijkl.p, c->d_v.p, c->d_prims.p, c->d_flags.p,
                                                                keep_values ? c->d_s1.p : nullptr,
                                                                keep_values ? c->d_s2.p : nullptr, key.p, idx.p, bad.p,
                                                                n1dev.p, jtab, qcache);
    e = cudaGetLastError();
  }
  size_t tmp_bytes = 0;
  if (e == cudaSuccess)
    e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, key.p, key2.p, idx.p, idx2.p, n, 0, 32, c->stream);
  if (e == cudaSuccess && tmp_bytes > tmp.n) e = tmp.reserve(tmp_bytes);
  if (e == cudaSuccess)
    e = cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, key.p, key2.p, idx.p, idx2.p, n, 0, 32, c->stream);
  // class histogram from the sorted keys: copy keys to host (4 B per quartet) is too
  // large for big lists, so run-length encode on the device.
  if (e == cudaSuccess) e = ukeys.reserve(4096);
  if (e == cudaSuccess) e = ucounts.reserve(4096);
  if (e == cudaSuccess) e = nruns.reserve(1);
  size_t tmp2 = 0;
  if (e == cudaSuccess)
    e = cub::DeviceRunLengthEncode::Encode(nullptr, tmp2, key2.p, ukeys.p, ucounts.p, nruns.p, n, c->stream);
  if (e == cudaSuccess && tmp2 > tmp.n) e = tmp.reserve(tmp2);
  if (e == cudaSuccess)
    e = cub::DeviceRunLengthEncode::Encode(tmp.p, tmp2, key2.p, ukeys.p, ucounts.p, nruns.p, n, c->stream);
  int h_runs = 0, h_bad = 0;
  unsigned long long h_n1 = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h_n1, n1dev.p, sizeof(h_n1), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h_runs, nruns.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  std::vector<uint32_t> hk(std::max(h_runs, 1));
  std::vector<int64_t> hcnt(std::max(h_runs, 1));
  if (e == cudaSuccess && h_runs > 0) {
    e = cudaMemcpy(hk.data(), ukeys.p, sizeof(uint32_t) * h_runs, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(hcnt.data(), ucounts.p, sizeof(int64_t) * h_runs, cudaMemcpyDeviceToHost);
  }
  if (e != cudaSuccess) {
    release_all();
    return cuda_error(c, e, "inca_prepare (screening)");
  }
  if (h_bad) {
    cleanup();
    return set_error(c, INCA_E_ARG, "inca_prepare: quartet index outside 1..nprim");
  }
  // class segments
  c->classes.clear();
  int64_t nsurv = 0, off64 = 0, off32 = 0;
  int maxL = 0;
  for (int r = 0; r < h_runs; ++r) {
    if (hk[r] == 0xFFFFFFFFu) continue;
    ClassSeg s;
    s.mol = static_cast<int>(hk[r] >> 16);
    s.L[0] = (hk[r] >> 10) & 31;
    s.L[1] = (hk[r] >> 5) & 31;
    s.L[2] = hk[r] & 31;
    const int nc = s.L[0] + s.L[1] + s.L[2] + 3;
    s.stride = (kRecHeader + nc + 1) & ~1;
    s.stride32 = (12 + 2 * nc + 3) & ~3;
    s.first = nsurv;
    s.count = hcnt[r];
    s.off64 = off64;
    s.off32 = off32;
    off64 += s.count * s.stride;
    off32 += s.count * s.stride32;
    nsurv += s.count;
    maxL = std::max(maxL, std::max(s.L[0], std::max(s.L[1], s.L[2])));
    c->classes.push_back(s);
  }
  c->nsurv = nsurv;
  c->max_L = maxL;
  // work chunks of <= 32 records within a class; each molecule's chunks are contiguous
  c->chunks.clear();
  const int nmol = std::max(c->batch_molecules, 1);
  c->mol_chunks.assign(nmol, ChunkRange{0, 0});
  c->mol_surv.assign(nmol, 0);
  std::vector<bool> seen(nmol, false);
  for (int s = 0; s < static_cast<int>(c->classes.size()); ++s) {
    const int mol = c->classes[s].mol;
    if (mol < 0 || mol >= nmol) {
      cleanup();
      return set_error(c, INCA_E_STATE, "inca_prepare: molecule index outside the batch");
    }
    if (!seen[mol]) {
      seen[mol] = true;
      c->mol_chunks[mol].begin = static_cast<int>(c->chunks.size());
    }
    c->mol_surv[mol] += c->classes[s].count;
    for (int64_t f = 0; f < c->classes[s].count; f += 32) {
      WorkChunk w;
      w.cls = s;
      w.count = static_cast<int>(std::min<int64_t>(32, c->classes[s].count - f));
      w.rec = c->classes[s].first + f;
      c->chunks.push_back(w);
    }
    c->mol_chunks[mol].end = static_cast<int>(c->chunks.size());
  }
  for (int m = 0; m < nmol; ++m)
    if (!seen[m]) c->mol_chunks[m] = ChunkRange{0, 0};
  e = cudaSuccess;
  if (c->d_rec64.reserve(std::max<int64_t>(off64, 2)) || c->d_rec32.reserve(std::max<int64_t>(off32, 4)) ||
      c->d_surv_src.reserve(std::max<int64_t>(nsurv, 1)) ||
      c->d_classes.reserve(std::max<size_t>(c->classes.size(), 1)) ||
      c->d_chunks.reserve(std::max<size_t>(c->chunks.size(), 1))) {
    release_all();
    return set_error(c, INCA_E_NOMEM, "inca_prepare: survivor records");
  }
  if (!c->classes.empty())
    e = cudaMemcpyAsync(c->d_classes.p, c->classes.data(), sizeof(ClassSeg) * c->classes.size(),
                        cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && !c->chunks.empty())
    e = cudaMemcpyAsync(c->d_chunks.p, c->chunks.data(), sizeof(WorkChunk) * c->chunks.size(),
                        cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && nsurv > 0) {
    INCA_LAUNCH(c, k_build, static_cast<unsigned>((nsurv + bs - 1) / bs), bs, 0, 
        nsurv, idx2.p, c->d_ijkl.p, c->d_v.p, c->d_prims.p, c->d_classes.p,
        static_cast<int>(c->classes.size()), c->d_rec64.p, c->d_rec32.p, c->d_surv_src.p, jtab, qcache);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    release_all();
    return cuda_error(c, e, "inca_prepare (records)");
  }
  cleanup();
  c->counts.read = n;
  c->counts.after_screen1 = static_cast<int64_t>(h_n1);
  c->counts.after_screen2 = nsurv;
  c->prepared = true;
  ++c->prepare_count;
  c->evaluated = false;
  return INCA_OK;
}

// ---------------------------------------------------------------- closed-shell DM2 records
namespace {
// Record r of the folded list: pairs (i<=k) enumerated as p = index in the packed upper
// triangle; record = (pair_a, pair_b) for all pair_a, pair_b (unique: pair_a <= pair_b).
__device__ __forceinline__ void unpack_pair(int64_t p, int n, int* i, int* k) {
  // pairs ordered (0,0),(0,1)..(0,n-1),(1,1),...: row i has n-i entries
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    const int64_t start = static_cast<int64_t>(mid) * n - static_cast<int64_t>(mid) * (mid - 1) / 2;
    if (start <= p) lo = mid; else hi = mid - 1;
  }
  const int64_t start = static_cast<int64_t>(lo) * n - static_cast<int64_t>(lo) * (lo - 1) / 2;
  *i = lo;
  *k = lo + static_cast<int>(p - start);
}

__device__ __forceinline__ double gam(const double* D, int n, int i, int k, int j, int l) {
  return D[i + static_cast<int64_t>(n) * k] * D[j + static_cast<int64_t>(n) * l] -
         0.5 * D[i + static_cast<int64_t>(n) * l] * D[j + static_cast<int64_t>(n) * k];
}

__global__ void k_closed_shell(int64_t nrec, int n, int64_t npair, int unique, const double* D, int base,
                               int4* ijkl, double* v) {
  const int64_t r = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (r >= nrec) return;
  int64_t pa, pb;
  if (unique) {  // r enumerates pa <= pb in the packed triangle of the pair list
    int a, b;
    unpack_pair(r, static_cast<int>(npair), &a, &b);
    pa = a;
    pb = b;
  } else {
    pa = r / npair;
    pb = r % npair;
  }
  int i, k, j, l;
  unpack_pair(pa, n, &i, &k);
  unpack_pair(pb, n, &j, &l);
  // sum over the distinct orderings (i,k)/(k,i) x (j,l)/(l,j)
  double s = 0.0;
  const int ik[2][2] = {{i, k}, {k, i}}, jl[2][2] = {{j, l}, {l, j}};
  const int nik = (i == k) ? 1 : 2, njl = (j == l) ? 1 : 2;
  for (int a = 0; a < nik; ++a)
    for (int b = 0; b < njl; ++b) s += gam(D, n, ik[a][0], ik[a][1], jl[b][0], jl[b][1]);
  if (unique && pa != pb) s *= 2.0;  // Gamma_{ik,jl} + Gamma_{jl,ik}
  ijkl[r] = make_int4(base + i + 1, base + j + 1, base + k + 1, base + l + 1);
  v[r] = s;
}
}  // namespace

int64_t closed_shell_records(int n, int unique) {
  const int64_t npair = static_cast<int64_t>(n) * (n + 1) / 2;
  return unique ? npair * (npair + 1) / 2 : npair * npair;
}

// Records of one molecule's closed-shell DM2 (n primitives, 1-RDM D) into the context's quartet
// arrays at record offset `at`, with primitive indices offset by `base` (batches).
int gen_closed_shell_into(inca_ctx* c, int n, const double* D, int unique, int base, int64_t at) {
  const int64_t npair = static_cast<int64_t>(n) * (n + 1) / 2;
  const int64_t nrec = closed_shell_records(n, unique);
  DevBuf<double> dD;
  if (dD.reserve(static_cast<size_t>(n) * n)) return set_error(c, INCA_E_NOMEM, "D");
  cudaError_t e = cudaMemcpyAsync(dD.p, D, sizeof(double) * n * n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && nrec > 0) {
    INCA_LAUNCH(c, k_closed_shell, static_cast<unsigned>((nrec + 255) / 256), 256, 0, nrec, n, npair, unique, dD.p,
                base, c->d_ijkl.p + at, c->d_v.p + at);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  dD.release();
  if (e != cudaSuccess) return cuda_error(c, e, "closed-shell DM2");
  return INCA_OK;
}

int gen_closed_shell_device(inca_ctx* c, const double* D, int unique, int64_t* nrec_out) {
  if (c->nprim <= 0) return set_error(c, INCA_E_STATE, "primitives not set");
  if (!D) return set_error(c, INCA_E_ARG, "D is null");
  const int n = c->nprim;
  const int64_t nrec = closed_shell_records(n, unique);
  if (c->d_ijkl.reserve(nrec) || c->d_v.reserve(nrec)) return set_error(c, INCA_E_NOMEM, "quartet records");
  const int st = gen_closed_shell_into(c, n, D, unique, 0, 0);
  if (st) return st;
  c->nq = nrec;
  c->prepared = false;
  c->evaluated = false;
  if (nrec_out) *nrec_out = nrec;
  return INCA_OK;
}

}  // namespace inca
