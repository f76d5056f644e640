// K2 (mixed): FP32 evaluation with exact accumulation, plus a double-float correction of the
// terms whose FP32 error could exceed the requested tolerance. Everything runs on the FP32
// pipe (GB300's FP64 rate is ~1/64 of it); accumulation per point is exact (TwoSum in FP32,
// moved to FP64 every few chunks).
//
// Why a correction. A term evaluated in FP32 carries ~2^-24 relative rounding; on a grid those
// errors average only over the few terms that dominate each output, and symmetry-equivalent
// quartets at symmetry-equivalent points round identically, so pure FP32 stalls near 1e-8
// relative on the CH4 radial integral. The large terms are therefore re-evaluated in
// double-float arithmetic (~2^-44) and the difference is added.
//
// Work layout. Points are evaluated in Morton order (a sorted copy of the grid). A CTA is one
// warp owning a tile of 32 kPPT consecutive points (kPPT = 3, 4 or 5 per lane, set by the
// schedule; 32-point sub-tiles p = lane + 32 k), each a compact region with a bounding box. The
// CTA walks a strided subset of the class-uniform chunks (<= 32 quartet records of one angular
// class); each chunk is staged into shared memory
// by a 1-D TMA bulk copy (cp.async.bulk + mbarrier), double-buffered so the next chunk's copy
// overlaps the current chunk's arithmetic. All waits are bounded; a wait that gives up sets an
// error word that the host turns into INCA_E_TIMEOUT.
//
// Pass 1 (k_pass1): every (quartet, point) term in FP32 (compensated: hi/lo splits of the
//   scale, the shift and the point), accumulated exactly; also the sum per point of e_t, a
//   bound on each term's FP32 rounding error (see terms32). Pairs whose bound is below 2^-120
//   (under FP32's normal range) are skipped.
// Thresholds: for an output O = sum_g w_g I_g (radial integral: TFVC weights; I(s): angular
//   weights of the shell; cube: max-norm; explicit points: each point) with tolerance eps,
//   the rounding errors of the uncorrected terms are independent, unbiased and bounded by e_t
//   (variance <= e_t^2 / 3), so correcting every term with e_t > tau_g =
//   (eps |O|)^2 / (3 w_g E_O) keeps 3 sigma of their sum (variance <= tau_g E_O / 3) below
//   eps |O| (E_O = sum_g w_g sum_q e_qg). |O| is replaced by the lower bound |O~| - E_O.
// Pass 2 (k_pass2): per (quartet, 32-point sub-tile) the log2 upper bound
//   lb = log2(|A'| prod_d sum_k |Cn_dk|) + sum_d [L_d log2 max(1, M_d) - m_d^2]
//   (m_d/M_d: min/max |u_d| over the sub-tile's box, u = c_u r', e^-r'^2 = 2^-u^2), turned into
//   a bound of e_t, selects the sub-tiles that may need a correction; there, every point with
//   e_t > tau_g gets t_df - t_32 (t_32 recomputed by the same instruction sequence as in
//   pass 1).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cub/cub.cuh>

#include "inca_internal.h"
#include "stage_df.cuh"

namespace inca {

int choose_splits(int64_t tiles, int64_t nchunks, int num_sms, int ctas_per_sm);

namespace {

// Points per lane (kPPT, a template parameter of the kernels): a one-warp CTA owns a tile of
// 32 kPPT consecutive sorted points, as kPPT sub-tiles of 32 (points lane + 32 p). The schedule
// picks 3, 4 or 5; the grid sample behind the threshold estimates always uses 4.
constexpr int kDefaultPPT = 4;
constexpr int kSamplePPT = 4;
// the default is 3 up to kFewRecords surviving records per molecule and 5 from kManyRecords
constexpr double kFewRecords = 1e6, kManyRecords = 1e7;
constexpr int kMaxStride32 = (12 + 2 * 3 * kMaxCoef + 3) & ~3;
// tau = kTauScale (eps |O|)^2 / E_O: the error of an uncorrected term is a sum of independent
// round-to-nearest errors bounded in total by e_t, so its variance is <= e_t^2 / 3, and
// 3 sigma <= eps |O| gives tau <= 3 (eps |O| / 3)^2 / E_O.
constexpr double kTauScale = 1.0 / 3.0;
constexpr double kTestScale = 1.0 / 1.01;  // correct when e > tau / 1.01
// One-pass form (grids of at least kFuseMinPoints points): thresholds are estimated from every
// kSampleStride-th grid point, scaled down by kEstSafety (and, for the max-norm of cubes, with
// the largest sampled error sum times kCubeMargin standing in for each point's); where the
// exact thresholds after the pass are lower than the estimates, a correction pass covers the
// difference.
// (2 048: on the 3 050-point CH4 radial-integral grid at 1e-10 the one-pass form takes 3.1 ms
// in its evaluation pass against 1.1 + 4.2 ms for the two passes; every 16th point still gives
// a usable estimate, and the exact thresholds and the band pass keep the tolerance regardless)
constexpr int64_t kFuseMinPoints = 2048;
constexpr int64_t kSampleStride = 16;  // smallest default stride (see sample_stride_for)
constexpr double kEstSafety = 0.7;
constexpr double kCubeMargin = 2.0;
// Share of the tolerance given to terms left out of the one-pass form (their bounds over the
// tile sum to at most this share of eps |O|, checked after the pass).
constexpr double kDropFrac = 0.1;
constexpr int kCheapSlack = 4;           // default slack of the cheap tier (powers of two)
constexpr float kSkipLog2 = -120.0f;     // pass-1 skip: bound below 2^-120
constexpr int kFold = 8;                 // chunks between FP64 folds
constexpr int kItemsPerCta = 24;         // persistent passes: work items per resident CTA
// Records whose |u_d| stays below kFastU over a tile (so y >= -3 kFastU^2 > -1000 and the
// polynomials cannot overflow) and whose scale ks <= 100 take the term code without clamps.
#ifndef INCA_FAST_TERMS
#define INCA_FAST_TERMS 1
#endif
constexpr float kFastU = 18.0f;
// Resident one-warp CTAs per SM the pass kernels are compiled for (register budget).
#ifndef INCA_PASS_CTAS_PER_SM
#define INCA_PASS_CTAS_PER_SM 16
#endif

// 2^y for y <= 0 in FP32 without systematic bias: y = n + f (n = rint(y), |f| <= 1/2),
// 2^f by a polynomial evaluated by FMA Horner, times 2^(n + ks) built from the exponent bits
// (exact; 0 below 2^-126). ks: an integer power of two applied exactly in the final scaling.
// Polynomials (coefficients highest degree first, FP32): degree 6, minimax relative
// approximation of 2^x on [-1/2, 1/2] (1.9e-9; with the FP32 Horner steps 7.9e-8 = 1.32 u32
// measured over 2e6 points, mean 2.6e-10; a degree-7 Chebyshev interpolant, 3.2e-9 and 1.13
// u32 with Horner, was measured 3 % slower in the kernel). The error bound of a term allows 2 u32 for E. The
// hardware ex2.approx was measured biased by -5e-8 relative on this range, which the error
// model of the correction pass cannot absorb.
// Rounding: y is clamped to [-1000, 0] (below -1000 the scale is zero for every ks used here)
// and t = y + 1.5 * 2^23 rounds it to an integer in the low mantissa bits (ties to even, as
// rint), so n = t - 1.5 * 2^23 and f = y - n are exact and the exponent field is the integer
// bits of t plus a per-record constant: no conversion instructions.
constexpr int kExp2Deg = 6;
__device__ constexpr float kExp2C[7] = {1.534581242594868e-4f, 1.3399930903688073e-3f, 9.618489071726799e-3f,
                                        5.550328642129898e-2f, 0.24022646248340607f, 0.6931471824645996f, 1.0f};
constexpr float kRoundShift = 12582912.0f;  // 1.5 * 2^23
constexpr int kRoundShiftBits = 0x4B400000;

// kSafe = false: the caller guarantees y >= -1000 and ks <= 100 (then the clamp of y and the
// upper clamp of the exponent field change nothing, so both forms give the same bits).
template <bool kSafe = true>
__device__ __forceinline__ float exp2_fp32(float y, int ks) {
  const float yc = kSafe ? fmaxf(y, -1000.0f) : y;
  const float t = __fadd_rn(yc, kRoundShift);
  const float n = __fsub_rn(t, kRoundShift);
  const float f = __fsub_rn(yc, n);
  float p = kExp2C[0];
#pragma unroll
  for (int i = 1; i <= kExp2Deg; ++i) p = __fmaf_rn(p, f, kExp2C[i]);
  const int eb = max(__float_as_int(t) + (ks + 127 - kRoundShiftBits), 0);
  const int e = kSafe ? min(eb, 254) : eb;
  return __fmul_rn(p, __int_as_float(e << 23));
}

// The hardware 2^y (MUFU ex2.approx, flushing results below 2^-126 to zero): one instruction.
// Its relative error is at most 2.42 u over [-126, 0] (measured on a GB300 against exp2 in FP64
// over every FP32 argument there) but not unbiased enough for the statistical error model, so
// only the cheap tier (with its rigorous bound) and the threshold estimates use it.
__device__ __forceinline__ float ex2_approx(float y) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
  return r;
}

// ---------------------------------------------------------------- FP32 term (both passes)
// Each dimension's value polynomial and its absolute-coefficient bound share one Horner loop
// (one coefficient load and one branch per dimension; as two separate loops the kernel took
// 12 % longer, with the same bits): poly2_pts evaluates a polynomial of a class-uniform
// (warp-uniform) degree L at NP points by Horner with FMA and, with kErr, the bound
// sum_k |C_k| |u|^k, which bounds |V(u)| and, times 2 L u32, its Horner rounding error. A loop
// over the degree (not unrolled) keeps the kernel's code small enough for the instruction cache.
// L >= 1 (constant polynomials are skipped): the first Horner step starts from C[0] directly.
template <int NP, bool kErr>
__device__ __forceinline__ void poly2_pts(int L, const float* __restrict__ C, const float (&u)[NP], float (&v)[NP],
                                          float (&a)[NP]) {
  const float c0 = C[0], c1 = C[1];
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    v[p] = __fmaf_rn(c0, u[p], c1);
    if (kErr) a[p] = __fmaf_rn(fabsf(c0), fabsf(u[p]), fabsf(c1));
  }
#pragma unroll 1
  for (int m = 2; m <= L; ++m) {
    const float c = C[m];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      v[p] = __fmaf_rn(v[p], u[p], c);
      if (kErr) a[p] = __fmaf_rn(a[p], fabsf(u[p]), fabsf(c));
    }
  }
}

// The FP32 term of quartet record R at NP points, and a bound e on its rounding error:
//   u_d = fma(s_hi, r_hi, b_hi) + [s_hi r_lo + s_lo r_hi + b_lo]  (error <= u32 |u_d|)
//   y = -|u|^2 (error <= 4 u32 |y| with the u errors), E = exp2_fp32(y) (<= 2 u32)
//   V_d by Horner (absolute error <= 2 L_d u32 P_d, P_d = sum_k |C_k| |u_d|^k), 4 products
//   e = u32 |A'| E prod_d P_d (10 + 2 L + 3 |y|).
// Explicit round-to-nearest intrinsics only, so both passes produce the same bits.
// kSafe = false (records whose |u_d| stays below kFastU over the tile, and ks <= 100): the
// clamps of u and y are left out; they would change nothing there, so the bits are the same.
// kComp = false (threshold estimates only): u_d = fma(s_hi, r_hi, b_hi) without the low parts,
// an absolute error of about u32 (|s r| + |b|) instead of u32 |u_d|, and the hardware exp2; the
// error bound keeps its form, so it estimates the bound of the compensated term at that point.
template <int NP, bool kErr, bool kSafe = true, bool kComp = true>
__device__ __forceinline__ void terms32(const float* __restrict__ R, const int L[3], const float (&rh)[3][NP],
                                        const float (&rl)[3][NP], float (&t)[NP], float (&err)[NP]) {
  // the record head in three 16-byte loads (records are 16-byte aligned: strides of 4 floats)
  const float4 R0 = *reinterpret_cast<const float4*>(R);
  const float4 R1 = *reinterpret_cast<const float4*>(R + 4);
  const float4 R2 = *reinterpret_cast<const float4*>(R + 8);
  const float s_hi = R0.x, s_lo = R0.y, A_hi = R2.x, A_lo = R2.y;
  const int ks = static_cast<int>(R2.w);
  const float bh[3] = {R0.z, R0.w, R1.x}, bl[3] = {R1.y, R1.z, R1.w};
  float u[3][NP];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float b_hi = bh[d], b_lo = bl[d];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      if (kComp) {
        float t1 = __fmaf_rn(s_lo, rh[d][p], b_lo);
        t1 = __fmaf_rn(s_hi, rl[d][p], t1);
        u[d][p] = __fadd_rn(__fmaf_rn(s_hi, rh[d][p], b_hi), t1);
      } else {
        u[d][p] = __fmaf_rn(s_hi, rh[d][p], b_hi);
      }
    }
  }
  float E[NP], Y[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    float y = __fmul_rn(-u[0][p], u[0][p]);
    y = __fmaf_rn(-u[1][p], u[1][p], y);
    y = __fmaf_rn(-u[2][p], u[2][p], y);
    Y[p] = y;
    // the estimate pass (kComp = false) only sets thresholds: the hardware exp2 serves there
    // (the scale 2^ks folded into the argument, saturated below FP32's overflow)
    E[p] = kComp ? exp2_fp32<kSafe>(y, ks) : ex2_approx(fminf(__fadd_rn(y, static_cast<float>(ks)), 127.0f));
  }
  // the polynomials see u clamped to +-kUClamp: wherever E is non-zero |u_d| is far below it,
  // and far points (E = 0) cannot overflow the polynomial into inf (0 * inf = NaN)
  if (kSafe) {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (L[d]) {
#pragma unroll
        for (int p = 0; p < NP; ++p) u[d][p] = fminf(fmaxf(u[d][p], -kUClamp), kUClamp);
      }
  }
  const float* Cx = R + 12;
  const float* Cy = Cx + L[0] + 1;
  const float* Cz = Cy + L[1] + 1;
  // dimensions with L_d = 0 have V_d = 1 exactly (sign folded into A'): skipped. E becomes the
  // product E V_x V_y V_z in place, err its bound.
  float v[NP], a[NP];
  if (kErr) {
    const float k0 = 5.9604645e-08f * static_cast<float>(10 + 2 * (L[0] + L[1] + L[2]));
    const float aA = 5.9604645e-08f * fabsf(A_hi);
#pragma unroll
    for (int p = 0; p < NP; ++p) err[p] = __fmul_rn(E[p], __fmaf_rn(fabsf(Y[p]), 3.0f * aA, k0 * fabsf(A_hi)));
  }
  const float* Cd[3] = {Cx, Cy, Cz};
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (L[d]) {
      poly2_pts<NP, kErr>(L[d], Cd[d], u[d], v, a);
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        E[p] = __fmul_rn(E[p], v[p]);
        if (kErr) err[p] = __fmul_rn(err[p], a[p]);
      }
    }
#pragma unroll
  for (int p = 0; p < NP; ++p) t[p] = __fmaf_rn(E[p], A_hi, __fmul_rn(E[p], A_lo));
}

// ---------------------------------------------------------------- cheap tier (one-pass form)
// A (record, tile) pair whose terms are all small next to the tile's drop threshold is
// evaluated in plain FP32: u_d = fma(s_hi, x_d, b_hi) from the point rounded to nearest,
// the hardware ex2.approx, the FP32 coefficients and an FP32 sum over the chunk. Instead of
// entering the statistical error model, each such term carries a rigorous bound of its error,
// c 2^lb (2^lb bounds |term| over the tile), which is added to the tile's left-out bound mass
// like a dropped term's 2^lb: the pair qualifies when c 2^lb is at most 2^slack times the drop
// threshold (slack 0 keeps the a-priori bound of the left-out mass; with a larger slack the
// check after the pass -- repeat without leaving out if the mass took more than half the
// budget -- guards the tolerance).
//
// The bound, with u = 2^-24, K_d = 2 s X_d + |b_d| (X_d: largest |x_d| over the tile box) and
// m_d / M_d the smallest / largest |u_d| over the box (as in log2_bound):
//  * |u^_d - u_d| <= D_d = u (K_d + |u_d|)  (s, b and x each rounded once, then the FMA);
//  * y = -|u|^2 in three roundings: |y^ - y| <= sum_d 2 |u_d| D_d + 3 u |u|^2 (+ D_d^2);
//    2^-|u|^2 |u_d| <= 2^-sum m^2 max(m_d, 1/sqrt(2 ln 2)) and 2^-S S <= 2^-sum m^2
//    max(sum m^2, 1/ln 2), so E |y^ - y| ln 2 <= 2^-sum m^2 u ln2 (2 sum_d K_d max(m_d, 0.8494)
//    + 5 max(sum m^2, 1.4427));
//  * ex2.approx.ftz.f32: relative error at most kEx2RelErr over [-126, 0] (measured against
//    exp2 in FP64 over every FP32 argument there on a GB300: largest 2.42 u, mean -0.07 u), and
//    a result below 2^-126 flushed to zero: at most 2^(sum m^2 - 126) of 2^lb;
//  * Horner in FP32 with FP32 coefficients: (2 L_d + 1) u of P_d(M_d), and the error of u^_d
//    through V_d': L_d D_d of P_d(M_d);
//  * four products and the FP32 mantissa of A': 5 u; the FP32 sum of at most 32 terms: 31 u.
// Pairs qualify only where the argument bounds keep every piece small: |u_d| < kFastU (the
// polynomials cannot overflow), K_d <= 80 (so D_d stays inside the 1e-5 widening of the box
// bounds of log2_bound), and |ks| <= 100 (A' = m 2^ks is a normal FP32 number). Explicit
// round-to-nearest intrinsics: the one-pass kernel and the correction pass take the same
// decision from the same record, box and threshold.
constexpr float kEx2RelErr = 2.5f * 5.9604645e-08f;
constexpr float kCheapKMax = 80.0f;
constexpr int kCheapKsMax = 100;

// log2 of the cheap tier's error bound for record R over the tile box, or +inf when the pair
// does not qualify. lb: the pair's log2_bound over the same box.
__device__ __forceinline__ float cheap_log2_err(const float* __restrict__ R, const int L[3], const float* box,
                                                float lb) {
  const float s = R[0];
  const float ks = R[11];
  bool ok = ks >= -static_cast<float>(kCheapKsMax) && ks <= static_cast<float>(kCheapKsMax);
  float S = 0.0f, kt = 0.0f, vp = 0.0f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float b = R[2 + d];
    const float a0 = __fmaf_rn(s, box[d], b), a1 = __fmaf_rn(s, box[3 + d], b);
    float m = (a0 <= 0.0f && a1 >= 0.0f) ? 0.0f : fminf(fabsf(a0), fabsf(a1));
    float M = fmaxf(fabsf(a0), fabsf(a1));
    m = fmaxf(0.0f, __fsub_rn(__fmul_rn(m, 1.0f - 1e-5f), 1e-5f));
    M = __fadd_rn(__fmul_rn(M, 1.0f + 1e-5f), 1e-5f);
    const float X = fmaxf(fabsf(box[d]), fabsf(box[3 + d]));
    const float K = __fmaf_rn(__fmul_rn(2.0f, s), X, fabsf(b));
    ok = ok && K <= kCheapKMax && M < kFastU;
    S = __fmaf_rn(m, m, S);
    kt = __fmaf_rn(K, fmaxf(m, 0.8494f), kt);
    const float Lf = static_cast<float>(L[d]);
    vp = __fadd_rn(vp, __fmaf_rn(Lf, __fadd_rn(K, M), __fmaf_rn(2.0f, Lf, 1.0f)));
  }
  // c / u, with margins of 1 % (first-order expansions; every piece is below 1e-3 here)
  float cu = __fmul_rn(0.7002f, __fmaf_rn(2.0f, kt, __fmul_rn(5.0f, fmaxf(S, 1.4427f))));
  cu = __fadd_rn(cu, __fadd_rn(__fmul_rn(1.01f, vp), 36.0f + kEx2RelErr / 5.9604645e-08f));
  const float c = __fadd_rn(__fmul_rn(__fmul_rn(cu, 1.0001f), 5.9604645e-08f), exp2f(__fsub_rn(S, 125.99f)));
  return ok ? __fadd_rn(lb, __fadd_rn(__log2f(c), 0.02f)) : HUGE_VALF;
}


// Cheap-tier terms of record R at NP points (rn: the points rounded to nearest), added to sc.
template <int NP>
__device__ __forceinline__ void terms_cheap(const float* __restrict__ R, const int L[3], const float (&rn)[3][NP],
                                            float (&sc)[NP]) {
  const float4 R0 = *reinterpret_cast<const float4*>(R);
  const float4 R1 = *reinterpret_cast<const float4*>(R + 4);
  const float4 R2 = *reinterpret_cast<const float4*>(R + 8);
  const float s = R0.x;
  const float bh[3] = {R0.z, R0.w, R1.x};
  // A' = m 2^ks as one FP32 number (|ks| <= 100 for this tier)
  const float A = __fmul_rn(R2.x, __int_as_float((static_cast<int>(R2.w) + 127) << 23));
  float u[3][NP], E[NP];
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int p = 0; p < NP; ++p) u[d][p] = __fmaf_rn(s, rn[d][p], bh[d]);
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    float y = __fmul_rn(-u[0][p], u[0][p]);
    y = __fmaf_rn(-u[1][p], u[1][p], y);
    y = __fmaf_rn(-u[2][p], u[2][p], y);
    E[p] = ex2_approx(y);
  }
  const float* Cx = R + 12;
  const float* Cd[3] = {Cx, Cx + L[0] + 1, Cx + L[0] + L[1] + 2};
  float v[NP], a[NP];
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (L[d]) {
      poly2_pts<NP, false>(L[d], Cd[d], u[d], v, a);
#pragma unroll
      for (int p = 0; p < NP; ++p) E[p] = __fmul_rn(E[p], v[p]);
    }
#pragma unroll
  for (int p = 0; p < NP; ++p) sc[p] = __fmaf_rn(E[p], A, sc[p]);
}

// The same FP32 term and error bound for one point with loop-based Horner (compact code for
// the correction pass; same operation sequence and rounding as terms32).
__device__ __noinline__ void term32_one(const float* __restrict__ R, int L0, int L1, int L2, float rx, float ry,
                                        float rz, float lx, float ly, float lz, float* t_out, float* e_out) {
  const int L[3] = {L0, L1, L2};
  const float rh[3] = {rx, ry, rz}, rl[3] = {lx, ly, lz};
  const float s_hi = R[0], s_lo = R[1], A_hi = R[8], A_lo = R[9];
  const int ks = static_cast<int>(R[11]);
  float u[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float t1 = __fmaf_rn(s_lo, rh[d], R[5 + d]);
    t1 = __fmaf_rn(s_hi, rl[d], t1);
    u[d] = __fadd_rn(__fmaf_rn(s_hi, rh[d], R[2 + d]), t1);
  }
  float y = __fmul_rn(-u[0], u[0]);
  y = __fmaf_rn(-u[1], u[1], y);
  y = __fmaf_rn(-u[2], u[2], y);
  const float E = exp2_fp32(y, ks);
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (L[d]) u[d] = fminf(fmaxf(u[d], -kUClamp), kUClamp);
  const float k0 = 5.9604645e-08f * static_cast<float>(10 + 2 * (L0 + L1 + L2));
  const float aA = 5.9604645e-08f * fabsf(A_hi);
  float P = E, Pe = __fmul_rn(E, __fmaf_rn(fabsf(y), 3.0f * aA, k0 * fabsf(A_hi)));
  const float* C = R + 12;
  for (int d = 0; d < 3; ++d) {
    if (L[d]) {
      float v = C[0], va = fabsf(C[0]);
      for (int m = 1; m <= L[d]; ++m) {
        v = __fmaf_rn(v, u[d], C[m]);
        va = __fmaf_rn(va, fabsf(u[d]), fabsf(C[m]));
      }
      P = __fmul_rn(P, v);
      Pe = __fmul_rn(Pe, va);
    }
    C += L[d] + 1;
  }
  *t_out = __fmaf_rn(P, A_hi, __fmul_rn(P, A_lo));
  *e_out = Pe;
}

// The double-float terms of N records of one class at one point (r_hi + r_lo per dimension);
// the N evaluations are independent, so N > 1 gives the scheduler independent chains.
template <int N>
__device__ __forceinline__ void term_df_n(const float* const (&R)[N], const int L[3], const float (&rh)[N][3],
                                          const float (&rl)[N][3], const float2* __restrict__ tab, f2 (&out)[N]) {
  const int nc = L[0] + L[1] + L[2] + 3;
  f2 u[N][3];
#pragma unroll
  for (int n = 0; n < N; ++n) {
    const float s_hi = R[n][0], s_lo = R[n][1];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float p = __fmul_rn(s_hi, rh[n][d]);
      float e = __fmaf_rn(s_hi, rh[n][d], -p);
      const f2 t = two_sum(p, R[n][2 + d]);
      e = __fadd_rn(e, t.lo);
      e = __fmaf_rn(s_hi, rl[n][d], e);
      e = __fmaf_rn(s_lo, rh[n][d], e);
      e = __fadd_rn(e, R[n][5 + d]);
      u[n][d] = fast_two_sum(t.hi, e);  // |e| << |t.hi| except near u = 0, where it is harmless
    }
  }
  f2 t[N];
#pragma unroll
  for (int n = 0; n < N; ++n) {
    f2 y = df_add(df_add(df_sqr(u[n][0]), df_sqr(u[n][1])), df_sqr(u[n][2]));
    y.hi = -y.hi;
    y.lo = -y.lo;
    t[n] = df_exp2(y, static_cast<int>(R[n][11]), tab);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (fabsf(u[n][d].hi) > kUClamp) u[n][d] = {copysignf(kUClamp, u[n][d].hi), 0.0f};
  }
  int o = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (L[d] == 0) {  // normalised constant polynomial: exactly +-1
#pragma unroll
      for (int n = 0; n < N; ++n)
        if (R[n][12 + o] < 0.0f) t[n] = {-t[n].hi, -t[n].lo};
      o += 1;
      continue;
    }
    f2 v[N];
#pragma unroll
    for (int n = 0; n < N; ++n) v[n] = {R[n][12 + o], R[n][12 + o + nc]};
    for (int m = 1; m <= L[d]; ++m) {
#pragma unroll
      for (int n = 0; n < N; ++n) v[n] = df_add(df_mul(v[n], u[n][d]), f2{R[n][12 + o + m], R[n][12 + o + m + nc]});
    }
    o += L[d] + 1;
#pragma unroll
    for (int n = 0; n < N; ++n) t[n] = df_mul(t[n], v[n]);
  }
#pragma unroll
  for (int n = 0; n < N; ++n) out[n] = df_mul(t[n], f2{R[n][8], R[n][9]});
}

struct f2x2 {
  f2 a, b;
};
// Two double-float terms (records Ra, Rb of one class) at two points (hi and lo parts of each).
__device__ __noinline__ f2x2 term_df2p(const float* __restrict__ Ra, const float* __restrict__ Rb, int L0, int L1,
                                       int L2, float4 ha, float4 la, float4 hb, float4 lb,
                                       const float2* __restrict__ tab) {
  const int L[3] = {L0, L1, L2};
  const float rh[2][3] = {{ha.x, ha.y, ha.z}, {hb.x, hb.y, hb.z}}, rl[2][3] = {{la.x, la.y, la.z}, {lb.x, lb.y, lb.z}};
  const float* const Rs[2] = {Ra, Rb};
  f2 out[2];
  term_df_n<2>(Rs, L, rh, rl, tab, out);
  return {out[0], out[1]};
}

template <int kPPT>
__device__ __forceinline__ void load_points(const float4* __restrict__ phi, const float4* __restrict__ plo,
                                            const TileInfo& T, int lane, float (&rh)[3][kPPT],
                                            float (&rl)[3][kPPT]) {
#pragma unroll
  for (int p = 0; p < kPPT; ++p) {
    const int j = lane + 32 * p;
    float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
    if (j < T.count) {
      h = phi[T.start + j];
      l = plo[T.start + j];
    }
    rh[0][p] = h.x; rh[1][p] = h.y; rh[2][p] = h.z;
    rl[0][p] = l.x; rl[1][p] = l.y; rl[2][p] = l.z;
  }
}

// The noted corrections of one chunk (nm[p]: records q whose term at the lane's point p is to be
// evaluated in double-float), two terms per lane and round, taken in (point, record) order from
// all the lane's points; each lane adds its results to its points' double-float sums corr_s.
// Every lane takes part in every round (lanes without a term left skip the work), so the
// class-uniform record data in shared memory serves the whole warp.
template <int kPPT>
__device__ __forceinline__ void correction_rounds(uint32_t (&nm)[kPPT], const float* __restrict__ st, int rs,
                                                  const int L[3], const TileInfo& T, int lane,
                                                  const float4* __restrict__ phi, const float4* __restrict__ plo,
                                                  const float2* __restrict__ tab, float2 (*corr_s)[32],
                                                  unsigned long long& nround, unsigned long long& ncorr) {
  uint32_t any_left = 0u;
#pragma unroll
  for (int p = 0; p < kPPT; ++p) any_left |= nm[p];
  while (__any_sync(0xffffffffu, any_left != 0u)) {
    ++nround;
    int pa = -1, qa = 0, pb = -1, qb = 0;
#pragma unroll
    for (int p = 0; p < kPPT; ++p)
      if (pa < 0 && nm[p]) {
        pa = p;
        qa = __ffs(nm[p]) - 1;
        nm[p] &= nm[p] - 1;
      }
#pragma unroll
    for (int p = 0; p < kPPT; ++p)
      if (pb < 0 && nm[p]) {
        pb = p;
        qb = __ffs(nm[p]) - 1;
        nm[p] &= nm[p] - 1;
      }
    any_left = 0u;
#pragma unroll
    for (int p = 0; p < kPPT; ++p) any_left |= nm[p];
    if (pa >= 0) {
      const bool two = pb >= 0;
      if (!two) {  // a lone term is paired with itself and the copy discarded
        pb = pa;
        qb = qa;
      }
      const int64_t ga = T.start + lane + 32 * pa, gb = T.start + lane + 32 * pb;
      const f2x2 r = term_df2p(st + qa * rs, st + qb * rs, L[0], L[1], L[2], phi[ga], plo[ga], phi[gb], plo[gb],
                               tab);
      float2 ca = corr_s[pa][lane];
      f2 c = df_add(f2{ca.x, ca.y}, r.a);
      if (two && pb == pa) c = df_add(c, r.b);
      corr_s[pa][lane] = make_float2(c.hi, c.lo);
      if (two && pb != pa) {
        const float2 cb = corr_s[pb][lane];
        const f2 d = df_add(f2{cb.x, cb.y}, r.b);
        corr_s[pb][lane] = make_float2(d.hi, d.lo);
      }
      ncorr += two ? 2 : 1;
    }
  }
}

// ---------------------------------------------------------------- pass 1
// kFuse = false: estimate pass (every term in FP32, exact accumulation, error-bound sums).
// kFuse = true: one-pass form. Thresholds tau_g estimated beforehand (pt_tau) select the terms
//   to correct while they are evaluated: such a term's FP32 value is left out of the sum, the
//   lanes note (quartet, point) in a mask, and after each chunk the warp evaluates the noted
//   terms in double-float, each lane working down its own list (the chunk is class-uniform,
//   so the lanes run the same instruction sequence on different quartets).
// kEst = true (with kFuse = false): the estimate pass of the one-pass form on the grid sample.
//   Its sums only set the estimated thresholds (an estimate that is off costs corrections or a
//   band pass, never accuracy), so its terms skip the compensation of u (kComp = false) and are
//   summed in plain FP32, moved to FP64 after every chunk; the error bounds are the same.
template <bool kFuse, bool kEst = false, int kCtas = INCA_PASS_CTAS_PER_SM, bool kWaitTest = false,
          int kPPT = kDefaultPPT>
__global__ void __launch_bounds__(32, kCtas)
k_pass1(const WorkChunk* __restrict__ chunks, const MolWork* __restrict__ mw, int nmol,
        const ClassSeg* __restrict__ segs, const float* __restrict__ rec32, const float4* __restrict__ phi,
        const float4* __restrict__ plo, const TileInfo* __restrict__ tiles, const float* __restrict__ wtbox,
        int64_t nitems, int stage_floats, const float* __restrict__ pt_tau,
        const float2* __restrict__ exp_tab, const float* __restrict__ lt_drop, int cheap_tier,
        double* __restrict__ part, double* __restrict__ part_abs, double* __restrict__ drop_mass,
        unsigned long long* __restrict__ work, unsigned long long* __restrict__ stats, int* __restrict__ err,
        int wait_test) {
  static_assert(!(kFuse && kEst), "the estimate pass has no corrections");
  // kWaitTest (an instantiation for the test of the bounded waits only): no staging copy is
  // started and every wait gives up after wait_test tries, so the error path runs. Production
  // instantiations keep both as constants (as a runtime choice they cost about 3 % of the pass).
  const bool issue = !kWaitTest;
  const int wlim = kWaitTest ? wait_test : kWaitLimit;
  extern __shared__ __align__(128) unsigned char dsm[];
  const Stage S = stage_view(dsm, stage_floats);
  __shared__ float2 tab[kFuse ? kExpTab + 1 : 1];
  // per-point double-float correction sums of the one-pass form (shared memory: the rounds of
  // inline corrections reach any of the lane's points)
  __shared__ float2 corr_s[kFuse ? kPPT : 1][32];
  const int lane = threadIdx.x;
  if (kFuse)
    for (int i = lane; i <= kExpTab; i += 32) tab[i] = exp_tab[i];
  stage_init(S);
  unsigned long long nskip = 0, nlive = 0, ncorr = 0, nround = 0, ncheap = 0;
  int k = 0;  // chunks taken by this CTA so far: selects buffer and barrier phase
  for (;;) {
    const int64_t item = next_item(work);
    if (item >= nitems) break;
    int64_t wtile, pat, dat;
    int nsplit, first;
    ChunkRange cr;
    {
      const MolWork& W = mw[mol_of_item(mw, nmol, item)];
      const int64_t local = item - W.item0;
      const int64_t tl = local / W.nsplit;
      const int split = static_cast<int>(local - tl * W.nsplit);
      nsplit = W.nsplit;
      wtile = W.tile0 + tl;
      cr = ChunkRange{W.cb, W.ce};
      first = cr.begin + split;
      pat = W.poff + static_cast<int64_t>(split) * W.np - W.p0;  // + sorted point index
      dat = W.doff + static_cast<int64_t>(split) * W.ntiles + tl;
    }
    const TileInfo T = tiles[wtile];
    if (first < cr.end) stage_first(S, chunks, segs, rec32, k, first, issue);
    float rh[3][kPPT], rl[3][kPPT];
    load_points(phi, plo, T, lane, rh, rl);
    float tau[kPPT];
    if (kFuse) {
#pragma unroll
      for (int p = 0; p < kPPT; ++p) {
        const int j = lane + 32 * p;
        tau[p] = j < T.count ? pt_tau[T.start + j] : HUGE_VALF;
        corr_s[p][lane] = make_float2(0.0f, 0.0f);
      }
    }
    float box[6];
#pragma unroll
    for (int b = 0; b < 6; ++b) box[b] = wtbox[wtile * 8 + b];
    // quartets whose bound over the tile is at most 2^thr are left out; the one-pass form
    // raises thr to the tile's drop threshold and sums the bounds it left out (dm)
    const float thr = (kFuse && lt_drop) ? fmaxf(kSkipLog2, lt_drop[wtile]) : kSkipLog2;
    float dm = 0.0f;
    double acc[kPPT];
#pragma unroll
    for (int p = 0; p < kPPT; ++p) acc[p] = 0.0;
    float sh[kPPT], sl[kPPT], sa[kPPT];
#pragma unroll
    for (int p = 0; p < kPPT; ++p) sh[p] = sl[p] = sa[p] = 0.0f;
    __syncwarp();
    int nfold = 0;
    bool ok = true;
    for (int ch = first; ch < cr.end; ch += nsplit, ++k) {
      ok = __all_sync(0xffffffffu, stage_next(S, chunks, segs, rec32, k, ch + nsplit, cr.end, wlim, issue));
      if (!ok) break;
      const WorkChunk w = chunks[ch];
      const ClassSeg sg = segs[w.cls];
      const float* st = S.buf(k);
      // the class's degrees and record stride pass through a warp reduction: its result is
      // warp-uniform by construction, so the degree tests and Horner loops of every term are
      // uniform branches (no reconvergence bookkeeping) and their counters leave the vector pipes
      const int L[3] = {__reduce_max_sync(0xffffffffu, sg.L[0]), __reduce_max_sync(0xffffffffu, sg.L[1]),
                        __reduce_max_sync(0xffffffffu, sg.L[2])};
      const int rs = __reduce_max_sync(0xffffffffu, sg.stride32);
      float umax = HUGE_VALF;
      const float lb = lane < w.count ? log2_bound(st + lane * rs, L, box, nullptr, &umax) : -HUGE_VALF;
      const bool live = lane < w.count && lb > thr;
      // cheap tier (one-pass form with dropping): pairs whose rigorous FP32 error bound stays
      // within the drop threshold; the bound joins the left-out mass
      uint32_t mc = 0u;
      if (kFuse && lt_drop && cheap_tier) {
        const float lc = live ? cheap_log2_err(st + lane * rs, L, box, lb) : HUGE_VALF;
        const bool cheap = lc <= thr + static_cast<float>(cheap_tier - 1);
        mc = __ballot_sync(0xffffffffu, cheap);
        if (cheap) dm += exp2f(lc);
      }
      uint32_t m = __ballot_sync(0xffffffffu, live) & ~mc;
      const uint32_t fast = INCA_FAST_TERMS ? __ballot_sync(0xffffffffu, lane < w.count && umax < kFastU &&
                                                                           st[lane * rs + 11] <= 100.0f)
                                            : 0u;
      if (kFuse && lane < w.count && !(lb > thr)) dm += exp2f(lb);
      if (lane == 0) {
        nskip += w.count - __popc(m) - __popc(mc);
        nlive += __popc(m);
        ncheap += __popc(mc);
      }
      if (kFuse && mc) {
        // the points rounded to nearest (the cheap terms' coordinates), once per chunk
        float rn[3][kPPT], sc[kPPT];
#pragma unroll
        for (int p = 0; p < kPPT; ++p) {
#pragma unroll
          for (int d = 0; d < 3; ++d) rn[d][p] = __fadd_rn(rh[d][p], rl[d][p]);
          sc[p] = 0.0f;
        }
        uint32_t mm = mc;
        while (mm) {
          const int q = __ffs(mm) - 1;
          mm &= mm - 1;
          terms_cheap<kPPT>(st + q * rs, L, rn, sc);
        }
#pragma unroll
        for (int p = 0; p < kPPT; ++p) {
          const f2 s2 = two_sum(sh[p], sc[p]);
          sh[p] = s2.hi;
          sl[p] = __fadd_rn(sl[p], s2.lo);
        }
      }
      uint32_t nm[kPPT];
#pragma unroll
      for (int p = 0; p < kPPT; ++p) nm[p] = 0u;
      while (m) {
        const int q = __ffs(m) - 1;
        m &= m - 1;
        float t[kPPT], e[kPPT];
        if ((fast >> q) & 1u)
          terms32<kPPT, true, false, !kEst>(st + q * rs, L, rh, rl, t, e);
        else
          terms32<kPPT, true, true, !kEst>(st + q * rs, L, rh, rl, t, e);
#pragma unroll
        for (int p = 0; p < kPPT; ++p) {
          if (kFuse && e[p] > tau[p]) {
            // corrected in double-float below: it carries no FP32 error, so neither its value
            // nor its error bound enters the sums (the exact thresholds then rest on the
            // uncorrected terms alone, which is all the variance bound needs)
            nm[p] |= 1u << q;
            t[p] = 0.0f;
            e[p] = 0.0f;
          }
          if (kEst) {
            sh[p] = __fadd_rn(sh[p], t[p]);
          } else {
            const f2 s2 = two_sum(sh[p], t[p]);
            sh[p] = s2.hi;
            sl[p] = __fadd_rn(sl[p], s2.lo);
          }
          sa[p] = __fadd_rn(sa[p], e[p]);
        }
      }
      if (kFuse) {
        correction_rounds(nm, st, rs, L, T, lane, phi, plo, tab, corr_s, nround, ncorr);
      }
      // renormalise the FP32 pair every chunk; move it to FP64 every kFold chunks (the plain
      // sums of the estimate pass after every chunk)
      const bool fold = ++nfold == (kEst ? 1 : kFold);
#pragma unroll
      for (int p = 0; p < kPPT; ++p) {
        const f2 r = fast_two_sum(sh[p], sl[p]);
        sh[p] = r.hi;
        sl[p] = r.lo;
        if (fold) {
          acc[p] += static_cast<double>(sh[p]) + static_cast<double>(sl[p]);
          sh[p] = sl[p] = 0.0f;
          if (kFuse) {
            const float2 c = corr_s[p][lane];
            acc[p] += static_cast<double>(c.x) + static_cast<double>(c.y);
            corr_s[p][lane] = make_float2(0.0f, 0.0f);
          }
        }
      }
      if (fold) nfold = 0;
      __syncwarp();
    }
    if (!ok) {
      if (lane == 0) atomicExch(err, 1);
      break;
    }
    float (&shs)[kPPT] = sh;
    float (&sls)[kPPT] = sl;
    float (&sas)[kPPT] = sa;
#pragma unroll
    for (int p = 0; p < kPPT; ++p) {
      acc[p] += static_cast<double>(shs[p]) + static_cast<double>(sls[p]);
      if (kFuse) {
        const float2 c = corr_s[p][lane];
        acc[p] += static_cast<double>(c.x) + static_cast<double>(c.y);
      }
      const int j = lane + 32 * p;
      if (j < T.count) {
        part[pat + T.start + j] = acc[p];
        part_abs[pat + T.start + j] = static_cast<double>(sas[p]);
      }
    }
    if (kFuse && drop_mass) {
      for (int o = 16; o > 0; o >>= 1) dm += __shfl_xor_sync(0xffffffffu, dm, o);
      // the FP32 sum of the left-out bounds, raised by a margin for its own rounding
      if (lane == 0) drop_mass[dat] = dm * 1.0001;
    }
  }
  if (kFuse)
    for (int o = 16; o > 0; o >>= 1) ncorr += __shfl_xor_sync(0xffffffffu, ncorr, o);
  if (lane == 0) {
    atomicAdd(&stats[2], nskip);
    if (kFuse) {
      atomicAdd(&stats[0], nlive);
      atomicAdd(&stats[1], nround);
      atomicAdd(&stats[3], ncorr);
      atomicAdd(&stats[13], ncheap);
    }
  }
}

// ---------------------------------------------------------------- FP64 form, screened
// The plain FP64 form with the one-pass form's leaving-out of negligible (quartet, tile) pairs:
// the same persistent work items, staging, tile bounds and drop thresholds as k_pass1<true>, and
// every remaining term in FP64 (the hi + lo pairs of the FP32 records carry each value to about
// 2^-48), without error bounds or corrections. It prices the precision alone: the mixed form
// against this kernel differs only in the arithmetic of the terms it evaluates.
template <int kPPT>
__device__ __forceinline__ void term_f64(const float* __restrict__ R, const int L[3], const double (&x)[3][kPPT],
                                         double (&acc)[kPPT]) {
  const double s = static_cast<double>(R[0]) + static_cast<double>(R[1]);
  const double b[3] = {static_cast<double>(R[2]) + static_cast<double>(R[5]),
                       static_cast<double>(R[3]) + static_cast<double>(R[6]),
                       static_cast<double>(R[4]) + static_cast<double>(R[7])};
  const double m = static_cast<double>(R[8]) + static_cast<double>(R[9]);
  const double ks = static_cast<double>(R[11]);
  const int nc = L[0] + L[1] + L[2] + 3;
  double u[3][kPPT], t[kPPT];
#pragma unroll
  for (int p = 0; p < kPPT; ++p) {
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d][p] = fma(s, x[d][p], b[d]);
    const double y = -(u[0][p] * u[0][p] + u[1][p] * u[1][p] + u[2][p] * u[2][p]);
    t[p] = m * exp2(y + ks);
  }
  int o = 12;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (L[d]) {
      double v[kPPT];
      const double c0 = static_cast<double>(R[o]) + static_cast<double>(R[o + nc]);
#pragma unroll
      for (int p = 0; p < kPPT; ++p) v[p] = c0;
#pragma unroll 1
      for (int k = 1; k <= L[d]; ++k) {
        const double ck = static_cast<double>(R[o + k]) + static_cast<double>(R[o + k + nc]);
#pragma unroll
        for (int p = 0; p < kPPT; ++p) v[p] = fma(v[p], u[d][p], ck);
      }
#pragma unroll
      for (int p = 0; p < kPPT; ++p) t[p] *= v[p];
    }
    o += L[d] + 1;
  }
#pragma unroll
  for (int p = 0; p < kPPT; ++p) acc[p] += t[p];
}

template <int kPPT>
__global__ void __launch_bounds__(32, INCA_PASS_CTAS_PER_SM)
k_pass_f64(const WorkChunk* __restrict__ chunks, const MolWork* __restrict__ mw, int nmol,
           const ClassSeg* __restrict__ segs, const float* __restrict__ rec32, const float4* __restrict__ phi,
           const float4* __restrict__ plo, const TileInfo* __restrict__ tiles, const float* __restrict__ wtbox,
           int64_t nitems, int stage_floats, const float* __restrict__ lt_drop, double* __restrict__ part,
           double* __restrict__ part_abs, double* __restrict__ drop_mass, unsigned long long* __restrict__ work,
           unsigned long long* __restrict__ stats, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char dsm[];
  const Stage S = stage_view(dsm, stage_floats);
  const int lane = threadIdx.x;
  stage_init(S);
  unsigned long long nskip = 0, nlive = 0;
  int k = 0;
  for (;;) {
    const int64_t item = next_item(work);
    if (item >= nitems) break;
    int64_t wtile, pat, dat;
    int nsplit, first;
    ChunkRange cr;
    {
      const MolWork& W = mw[mol_of_item(mw, nmol, item)];
      const int64_t local = item - W.item0;
      const int64_t tl = local / W.nsplit;
      const int split = static_cast<int>(local - tl * W.nsplit);
      nsplit = W.nsplit;
      wtile = W.tile0 + tl;
      cr = ChunkRange{W.cb, W.ce};
      first = cr.begin + split;
      pat = W.poff + static_cast<int64_t>(split) * W.np - W.p0;
      dat = W.doff + static_cast<int64_t>(split) * W.ntiles + tl;
    }
    const TileInfo T = tiles[wtile];
    if (first < cr.end) stage_first(S, chunks, segs, rec32, k, first);
    double x[3][kPPT], acc[kPPT];
    {
      float rh[3][kPPT], rl[3][kPPT];
      load_points(phi, plo, T, lane, rh, rl);
#pragma unroll
      for (int p = 0; p < kPPT; ++p) {
        acc[p] = 0.0;
#pragma unroll
        for (int d = 0; d < 3; ++d) x[d][p] = static_cast<double>(rh[d][p]) + static_cast<double>(rl[d][p]);
      }
    }
    float box[6];
#pragma unroll
    for (int b = 0; b < 6; ++b) box[b] = wtbox[wtile * 8 + b];
    const float thr = lt_drop ? fmaxf(kSkipLog2, lt_drop[wtile]) : kSkipLog2;
    float dm = 0.0f;
    __syncwarp();
    bool ok = true;
    for (int ch = first; ch < cr.end; ch += nsplit, ++k) {
      ok = __all_sync(0xffffffffu, stage_next(S, chunks, segs, rec32, k, ch + nsplit, cr.end));
      if (!ok) break;
      const WorkChunk w = chunks[ch];
      const ClassSeg sg = segs[w.cls];
      const float* st = S.buf(k);
      const int L[3] = {__reduce_max_sync(0xffffffffu, sg.L[0]), __reduce_max_sync(0xffffffffu, sg.L[1]),
                        __reduce_max_sync(0xffffffffu, sg.L[2])};
      const int rs = __reduce_max_sync(0xffffffffu, sg.stride32);
      const float lb = lane < w.count ? log2_bound(st + lane * rs, L, box) : -HUGE_VALF;
      uint32_t m = __ballot_sync(0xffffffffu, lane < w.count && lb > thr);
      if (lane < w.count && !(lb > thr)) dm += exp2f(lb);
      if (lane == 0) {
        nskip += w.count - __popc(m);
        nlive += __popc(m);
      }
      while (m) {
        const int q = __ffs(m) - 1;
        m &= m - 1;
        term_f64(st + q * rs, L, x, acc);
      }
      __syncwarp();
    }
    if (!ok) {
      if (lane == 0) atomicExch(err, 1);
      break;
    }
#pragma unroll
    for (int p = 0; p < kPPT; ++p) {
      const int j = lane + 32 * p;
      if (j < T.count) {
        part[pat + T.start + j] = acc[p];
        part_abs[pat + T.start + j] = 0.0;
      }
    }
    if (drop_mass) {
      for (int o = 16; o > 0; o >>= 1) dm += __shfl_xor_sync(0xffffffffu, dm, o);
      if (lane == 0) drop_mass[dat] = dm * 1.0001;
    }
  }
  if (lane == 0) {
    atomicAdd(&stats[0], nlive);
    atomicAdd(&stats[2], nskip);
  }
}

// ---------------------------------------------------------------- pass 2 (corrections)
template <int kPPT>
__global__ void __launch_bounds__(32, INCA_PASS_CTAS_PER_SM)
k_pass2(const WorkChunk* __restrict__ chunks, const MolWork* __restrict__ mw, int nmol,
        const ClassSeg* __restrict__ segs, const float* __restrict__ rec32, const float4* __restrict__ phi,
        const float4* __restrict__ plo, const TileInfo* __restrict__ tiles, const float* __restrict__ wtbox,
        const float* __restrict__ gbox, const float* __restrict__ g_lt, const float* __restrict__ pt_tau,
        const float* __restrict__ pt_tau_est, const float* __restrict__ lt_drop, int cheap_tier,
        const float2* __restrict__ exp_tab, int64_t nitems, int stage_floats, double* __restrict__ part,
        unsigned long long* __restrict__ work, unsigned long long* __restrict__ stats, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char dsm[];
  const Stage S = stage_view(dsm, stage_floats);
  __shared__ float2 tab[kExpTab + 1];
  __shared__ float2 corr_s[kPPT][32];
  const int lane = threadIdx.x;
  for (int i = lane; i <= kExpTab; i += 32) tab[i] = exp_tab[i];
  stage_init(S);
  unsigned long long n32 = 0, ndf = 0, npts = 0, nround = 0;
  int k = 0;
  for (;;) {
    const int64_t item = next_item(work);
    if (item >= nitems) break;
    int64_t wtile, pat;
    int nsplit, split;
    ChunkRange cr;
    {
      const MolWork& W = mw[mol_of_item(mw, nmol, item)];
      const int64_t local = item - W.item0;
      const int64_t tl = local / W.nsplit;
      split = static_cast<int>(local - tl * W.nsplit);
      nsplit = W.nsplit;
      wtile = W.tile0 + tl;
      cr = ChunkRange{W.cb, W.ce};
      pat = W.poff + static_cast<int64_t>(split) * W.np - W.p0;
    }
    const TileInfo T = tiles[wtile];
    // a tile none of whose sub-tiles can need a correction contributes zeros
    bool any_sub = false;
#pragma unroll
    for (int p = 0; p < kPPT; ++p) any_sub |= g_lt[wtile * kPPT + p] < HUGE_VALF;
    const int first = any_sub ? cr.begin + split : cr.end;
    if (first < cr.end) stage_first(S, chunks, segs, rec32, k, first);
    float rh[3][kPPT], rl[3][kPPT], tau[kPPT], tau_est[kPPT];
    load_points(phi, plo, T, lane, rh, rl);
#pragma unroll
    for (int p = 0; p < kPPT; ++p) {
      const int j = lane + 32 * p;
      tau[p] = j < T.count ? pt_tau[T.start + j] : HUGE_VALF;
      tau_est[p] = (pt_tau_est && j < T.count) ? pt_tau_est[T.start + j] : HUGE_VALF;
    }
    float wbox[6];
#pragma unroll
    for (int b = 0; b < 6; ++b) wbox[b] = wtbox[wtile * 8 + b];
    const float thr = lt_drop ? fmaxf(kSkipLog2, lt_drop[wtile]) : kSkipLog2;
    double acc[kPPT];
#pragma unroll
    for (int p = 0; p < kPPT; ++p) {
      acc[p] = 0.0;
      corr_s[p][lane] = make_float2(0.0f, 0.0f);
    }
    __syncwarp();
    int nfold = 0;
    bool ok = true;
    for (int ch = first; ch < cr.end; ch += nsplit, ++k) {
      ok = __all_sync(0xffffffffu, stage_next(S, chunks, segs, rec32, k, ch + nsplit, cr.end));
      if (!ok) break;
      const WorkChunk w = chunks[ch];
      const ClassSeg sg = segs[w.cls];
      const float* st = S.buf(k);
      const int L[3] = {__reduce_max_sync(0xffffffffu, sg.L[0]), __reduce_max_sync(0xffffffffu, sg.L[1]),
                        __reduce_max_sync(0xffffffffu, sg.L[2])};
      const float* Rq = st + lane * sg.stride32;
      // the skip decision of the pass over all terms (same box, arithmetic and threshold)
      const float lb = lane < w.count ? log2_bound(Rq, L, wbox) : -HUGE_VALF;
      // pairs of the one-pass kernel's cheap tier (same decision): their error is bounded
      // within the left-out mass, nothing to correct
      const bool cheap =
          lt_drop && cheap_tier && lane < w.count && lb > thr &&
          cheap_log2_err(Rq, L, wbox, lb) <= thr + static_cast<float>(cheap_tier - 1);
      const uint32_t live = __ballot_sync(0xffffffffu, lane < w.count && lb > thr && !cheap);
      uint32_t msub[kPPT];
      uint32_t any = 0;
#pragma unroll
      for (int p = 0; p < kPPT; ++p) {
        float lerr = -HUGE_VALF;
        if (lane < w.count) log2_bound(Rq, L, gbox + (wtile * kPPT + p) * 8, &lerr);
        msub[p] = __ballot_sync(0xffffffffu, lane < w.count && !cheap && lerr > g_lt[wtile * kPPT + p]);
        any |= msub[p];
      }
      if (lane == 0) {
        ndf += __popc(any);
        n32 += __popc(live & ~any);
      }
      // the terms to correct: above the exact threshold and not corrected by the one-pass kernel
      // (which corrected the live terms above the estimated one); the FP32 value a live term
      // put into the pass's sum comes off here, its double-float value goes on in the rounds
      uint32_t nm[kPPT];
#pragma unroll
      for (int p = 0; p < kPPT; ++p) {
        nm[p] = 0u;
        uint32_t m = msub[p];
        float2 c = corr_s[p][lane];
        f2 cp{c.x, c.y};
        while (m) {
          const int q = __ffs(m) - 1;
          m &= m - 1;
          const float* R = st + q * sg.stride32;
          float t32 = 0.0f, e32 = 0.0f;
          term32_one(R, L[0], L[1], L[2], rh[0][p], rh[1][p], rh[2][p], rl[0][p], rl[1][p], rl[2][p], &t32, &e32);
          const bool live_q = (live >> q) & 1u;
          const bool need = e32 > tau[p] && !(live_q && e32 > tau_est[p]);
          if (need) {
            nm[p] |= 1u << q;
            if (live_q) cp = df_add(cp, f2{-t32, 0.0f});
          }
        }
        corr_s[p][lane] = make_float2(cp.hi, cp.lo);
      }
      unsigned long long ncorr = 0;
      correction_rounds(nm, st, sg.stride32, L, T, lane, phi, plo, tab, corr_s, nround, ncorr);
      npts += ncorr;
      if (++nfold == kFold) {
        nfold = 0;
#pragma unroll
        for (int p = 0; p < kPPT; ++p) {
          const float2 c = corr_s[p][lane];
          acc[p] += static_cast<double>(c.x) + static_cast<double>(c.y);
          corr_s[p][lane] = make_float2(0.0f, 0.0f);
        }
      }
      __syncwarp();
    }
    if (!ok) {
      if (lane == 0) atomicExch(err, 1);
      break;
    }
#pragma unroll
    for (int p = 0; p < kPPT; ++p) {
      const float2 c = corr_s[p][lane];
      acc[p] += static_cast<double>(c.x) + static_cast<double>(c.y);
      const int j = lane + 32 * p;
      if (j < T.count) part[pat + T.start + j] = acc[p];
    }
  }
  for (int o = 16; o > 0; o >>= 1) npts += __shfl_xor_sync(0xffffffffu, npts, o);
  if (lane == 0) {
    atomicAdd(&stats[0], n32);
    atomicAdd(&stats[1], ndf + nround);
    atomicAdd(&stats[3], npts);
  }
}

// ---------------------------------------------------------------- grid preparation
// Morton keys of the points g = j * stride, j < n (stride 1: the whole grid). With pmol (a
// batch) the molecule occupies the top 7 bits and each coordinate 19 bits, so the sort keeps
// every molecule's points together.
// bb: the grid's bounding box lo[3], hi[3] and the key scale 2^21 - 1 over its largest extent
// (k_bbox), read on the device so that no host round trip separates the two kernels.
__global__ void k_morton(int64_t n, int64_t stride, const double* __restrict__ px, const double* __restrict__ py,
                         const double* __restrict__ pz, const int* __restrict__ pmol,
                         const double* __restrict__ bb, uint64_t* key, int64_t* idx) {
  const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (j >= n) return;
  const int64_t g = j * stride;
  const double inv = bb[6];
  const double c[3] = {(px[g] - bb[0]) * inv, (py[g] - bb[1]) * inv, (pz[g] - bb[2]) * inv};
  uint64_t k = 0;
  uint32_t q[3];
  for (int d = 0; d < 3; ++d) q[d] = static_cast<uint32_t>(fmin(fmax(c[d], 0.0), 2097151.0));
  const int low = pmol ? 2 : 0;
  for (int b = 20; b >= low; --b)
    for (int d = 0; d < 3; ++d) k = (k << 1) | ((q[d] >> b) & 1u);
  if (pmol) k |= static_cast<uint64_t>(pmol[g]) << 57;
  key[j] = k;
  idx[j] = g;
}

// Each coordinate x is stored as hi + lo (FP32 pair). The split is offset from the nearest
// float by a pseudo-random number of ulps (|k| <= 32, from a hash of the grid index and the
// axis): symmetry-equivalent points of a symmetric molecule then round differently in FP32, so
// the rounding errors of their terms are not copies of one another (the correction thresholds
// assume independent errors). The pair still represents x to ~2^-42 relative.
__device__ __forceinline__ int split_offset(int64_t g, int d) {
  uint64_t z = static_cast<uint64_t>(g) * 3u + static_cast<uint64_t>(d) + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return static_cast<int>(z % 65u) - 32;
}

__global__ void k_gather_points(int64_t n, const int64_t* __restrict__ perm, const double* __restrict__ px,
                                const double* __restrict__ py, const double* __restrict__ pz, float4* phi,
                                float4* plo) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int64_t g = perm[i];
  const double x[3] = {px[g], py[g], pz[g]};
  float h[3], l[3];
  for (int d = 0; d < 3; ++d) {
    h[d] = static_cast<float>(x[d]);
    if (fabsf(h[d]) >= 1.0e-30f) {  // normal and far from zero: step the magnitude by k ulps
      const int bits = __float_as_int(h[d]);
      h[d] = __int_as_float((bits & 0x80000000) | ((bits & 0x7FFFFFFF) + split_offset(g, d)));
    }
    l[d] = static_cast<float>(x[d] - static_cast<double>(h[d]));
  }
  phi[i] = make_float4(h[0], h[1], h[2], 0.0f);
  plo[i] = make_float4(l[0], l[1], l[2], 0.0f);
}

// Bounding box of n points (min x, y, z then max x, y, z), one block of 1024 threads: each
// thread strides over the points, then a shared-memory tree (min and max are exact, so the
// result does not depend on the order).
__global__ void __launch_bounds__(1024) k_bbox(int64_t n, const double* __restrict__ px, const double* __restrict__ py,
                                               const double* __restrict__ pz, double* out) {
  __shared__ double sh[6][1024];
  double v[6] = {HUGE_VAL, HUGE_VAL, HUGE_VAL, -HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
  for (int64_t g = threadIdx.x; g < n; g += blockDim.x) {
    const double x = px[g], y = py[g], z = pz[g];
    v[0] = fmin(v[0], x); v[1] = fmin(v[1], y); v[2] = fmin(v[2], z);
    v[3] = fmax(v[3], x); v[4] = fmax(v[4], y); v[5] = fmax(v[5], z);
  }
  for (int k = 0; k < 6; ++k) sh[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int k = 0; k < 6; ++k)
        sh[k][threadIdx.x] = k < 3 ? fmin(sh[k][threadIdx.x], sh[k][threadIdx.x + h])
                                   : fmax(sh[k][threadIdx.x], sh[k][threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x < 6) out[threadIdx.x] = sh[threadIdx.x][0];
  if (threadIdx.x == 0) {
    const double ext = fmax(fmax(sh[3][0] - sh[0][0], sh[4][0] - sh[1][0]), fmax(sh[5][0] - sh[2][0], 1e-12));
    out[6] = 2097151.0 / ext;
  }
}

// Bounding boxes (FP32, rounded outwards) of each tile of 32 kPPT points and its kPPT 32-point
// sub-tiles (points lane + 32 p). One warp per tile.
template <int kPPT>
__global__ void k_boxes(const TileInfo* __restrict__ tiles, int64_t nwt, const float4* __restrict__ phi,
                        const float4* __restrict__ plo, float* wbox, float* gbox) {
  const int64_t wt = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + (threadIdx.x >> 5);
  if (wt >= nwt) return;
  const int lane = threadIdx.x & 31;
  const TileInfo T = tiles[wt];
  float tlo[3] = {HUGE_VALF, HUGE_VALF, HUGE_VALF}, thi[3] = {-HUGE_VALF, -HUGE_VALF, -HUGE_VALF};
  for (int p = 0; p < kPPT; ++p) {
    const int j = lane + 32 * p;
    float lo[3] = {HUGE_VALF, HUGE_VALF, HUGE_VALF}, hi[3] = {-HUGE_VALF, -HUGE_VALF, -HUGE_VALF};
    if (j < T.count) {
      const float4 h = phi[T.start + j], l = plo[T.start + j];
      const float x[3] = {h.x + l.x, h.y + l.y, h.z + l.z};
      for (int d = 0; d < 3; ++d) lo[d] = hi[d] = x[d];
    }
    for (int o = 16; o > 0; o >>= 1)
      for (int d = 0; d < 3; ++d) {
        lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
        hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
      }
    for (int d = 0; d < 3; ++d) {
      const float l = lo[d] - (fabsf(lo[d]) * 1e-6f + 1e-6f), h = hi[d] + (fabsf(hi[d]) * 1e-6f + 1e-6f);
      if (lane == 0) {
        gbox[(wt * kPPT + p) * 8 + d] = l;
        gbox[(wt * kPPT + p) * 8 + 3 + d] = h;
      }
      tlo[d] = fminf(tlo[d], l);
      thi[d] = fmaxf(thi[d], h);
    }
  }
  if (lane == 0)
    for (int d = 0; d < 3; ++d) {
      wbox[wt * 8 + d] = tlo[d];
      wbox[wt * 8 + 3 + d] = thi[d];
    }
}

// Per-point test thresholds (sorted order) and their minimum per 32-point sub-tile (log2).
// A term is corrected when its error bound e exceeds tau_g / 1.01 (the stored value).
// mode 0: tau = T_seg / w_g; mode 1 (max-norm): tau = T / E_g; mode 2: per point;
// mode 3: tau = T (uniform).
template <int kPPT>
__global__ void k_thresholds(const TileInfo* __restrict__ tiles, int64_t ngroups, int mode,
                             const int64_t* __restrict__ perm, const int* __restrict__ seg_of,
                             const double* __restrict__ segT, const double* __restrict__ w,
                             const double* __restrict__ I, const double* __restrict__ M, double eps, double tscale,
                             float* g_lt, float* pt_tau) {
  const int64_t grp = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + (threadIdx.x >> 5);
  if (grp >= ngroups) return;
  const int lane = threadIdx.x & 31;
  // group grp = tile grp / kPPT, sub-tile grp % kPPT: the tile's points lane + 32 * sub
  const TileInfo T = tiles[grp / kPPT];
  const int j = lane + 32 * static_cast<int>(grp % kPPT);
  const int64_t i = T.start + j;
  float ts = HUGE_VALF;
  if (j < T.count) {
    const int64_t g = perm[i];
    double tau = HUGE_VAL;
    if (mode == 0) {
      tau = w[g] > 0.0 ? segT[seg_of ? seg_of[g] : 0] / w[g] : HUGE_VAL;
    } else if (mode == 1) {
      tau = M[i] > 0.0 ? segT[0] / M[i] : HUGE_VAL;
    } else if (mode == 2) {
      const double lo = fmax(fabs(I[i]) - M[i], 0.0);
      const double x = eps * lo;
      tau = M[i] > 0.0 ? tscale * x * x / M[i] : HUGE_VAL;
    } else {
      tau = segT[0];
    }
    tau *= kTestScale;
    ts = tau >= 3.0e38 ? HUGE_VALF : static_cast<float>(tau);
    pt_tau[i] = ts;
  }
  if (!g_lt) return;
  float tmin = ts;
  for (int o = 16; o > 0; o >>= 1) tmin = fminf(tmin, __shfl_xor_sync(0xffffffffu, tmin, o));
  if (lane == 0) g_lt[grp] = tmin >= HUGE_VALF ? HUGE_VALF : (tmin > 0.0f ? log2f(tmin) : -HUGE_VALF);
}

// Sub-tiles where the exact threshold fell below the estimate used by the one-pass kernel:
// g_lt = log2 of the smallest exact threshold among those points (else +inf); counts them.
template <int kPPT>
__global__ void k_band(const TileInfo* __restrict__ tiles, int64_t ngroups, const float* __restrict__ pt_tau,
                       const float* __restrict__ pt_tau_est, float* g_lt, unsigned long long* nband) {
  const int64_t grp = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + (threadIdx.x >> 5);
  if (grp >= ngroups) return;
  const int lane = threadIdx.x & 31;
  const TileInfo T = tiles[grp / kPPT];
  const int j = lane + 32 * static_cast<int>(grp % kPPT);
  const int64_t i = T.start + j;
  float t = HUGE_VALF;
  if (j < T.count && pt_tau[i] < pt_tau_est[i]) t = pt_tau[i];
  for (int o = 16; o > 0; o >>= 1) t = fminf(t, __shfl_xor_sync(0xffffffffu, t, o));
  if (lane == 0) {
    g_lt[grp] = t >= HUGE_VALF ? HUGE_VALF : (t > 0.0f ? log2f(t) : -HUGE_VALF);
    if (t < HUGE_VALF) atomicAdd(nband, 1ull);
  }
}

// Sampled estimates, scattered to grid order: I and E at the sampled points, their weights
// (zero elsewhere; the targets are cleared first).
__global__ void k_scatter_sample(int64_t n, const int64_t* __restrict__ perm, const double* __restrict__ I,
                                 const double* __restrict__ M, const double* __restrict__ w, double* Io,
                                 double* Mo, double* wo) {
  const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (j >= n) return;
  const int64_t g = perm[j];
  Io[g] = I[j];
  Mo[g] = M[j];
  if (w) wo[g] = w[g];
}

__global__ void k_absmax2(int64_t n, const double* __restrict__ I, const double* __restrict__ M,
                          unsigned long long* out) {
  double a = 0.0, b = 0.0;
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < n;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    a = fmax(a, fabs(I[g]));
    b = fmax(b, fabs(M[g]));
  }
  for (int o = 16; o > 0; o >>= 1) {
    a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out[0], static_cast<unsigned long long>(__double_as_longlong(a)));
    atomicMax(&out[1], static_cast<unsigned long long>(__double_as_longlong(b)));
  }
}

__global__ void k_scatter(int64_t n, const int64_t* __restrict__ perm, const double* __restrict__ src, double* dst) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < n) dst[perm[i]] = src[i];
}

// Segment sums of w*I, w*M and w over contiguous original-order ranges (fixed-order trees).
__global__ void k_seg_sums(int nseg, const int64_t* __restrict__ off, const double* __restrict__ w,
                           const double* __restrict__ I, const double* __restrict__ M, double* out) {
  __shared__ double s[3][256];
  const int seg = blockIdx.x;
  const int64_t lo = off[seg], hi = off[seg + 1];
  double a = 0, b = 0, c = 0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double wi = w ? w[i] : 1.0;
    a += wi * I[i];
    b += wi * M[i];
    c += wi;
  }
  s[0][threadIdx.x] = a;
  s[1][threadIdx.x] = b;
  s[2][threadIdx.x] = c;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k)
      for (int j = 0; j < 3; ++j) s[j][threadIdx.x] += s[j][threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int j = 0; j < 3; ++j) out[3 * seg + j] = s[j][0];
}

// log2 of the smallest per-point value of each tile (one warp per tile).
template <int kPPT>
__global__ void k_tile_min_log2(const TileInfo* __restrict__ tiles, int64_t nwt, const float* __restrict__ pt,
                                float* lt) {
  const int64_t wt = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + (threadIdx.x >> 5);
  if (wt >= nwt) return;
  const int lane = threadIdx.x & 31;
  const TileInfo T = tiles[wt];
  float t = HUGE_VALF;
  for (int p = 0; p < kPPT; ++p) {
    const int j = lane + 32 * p;
    if (j < T.count) t = fminf(t, pt[T.start + j]);
  }
  for (int o = 16; o > 0; o >>= 1) t = fminf(t, __shfl_xor_sync(0xffffffffu, t, o));
  if (lane == 0) lt[wt] = t >= HUGE_VALF ? HUGE_VALF : (t > 0.0f ? log2f(t) : -HUGE_VALF);
}

// Per-tile values spread to the tile's points, in grid order.
__global__ void k_tile_to_points(const TileInfo* __restrict__ tiles, int64_t nwt, const int64_t* __restrict__ perm,
                                 const double* __restrict__ vt, double* out) {
  const int64_t wt = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + (threadIdx.x >> 5);
  if (wt >= nwt) return;
  const int lane = threadIdx.x & 31;
  const TileInfo T = tiles[wt];
  for (int j = lane; j < T.count; j += 32) out[perm[T.start + j]] = vt[wt];
}

// Sum over the splits of each sorted point (partials laid out per molecule), in split order;
// b (optional) has the same layout and is added after a.
// Sums over the split partials of each point (k_sum_mol) or tile (k_sum_drop) in a fixed
// order, so results are reproducible bit for bit: kSumLanes threads per output each add every
// kSumLanes-th split in increasing order, then the kSumLanes partial sums are added in thread
// order. (A small grid has few points and up to 4096 splits; one thread per output adding them
// one after the other waited on memory latency for milliseconds.) Block: 32 outputs x kSumLanes.
constexpr int kSumLanes = 16;
__global__ void __launch_bounds__(32 * kSumLanes)
k_sum_mol(int64_t n, const MolWork* __restrict__ mw, int nmol, const double* __restrict__ a,
          const double* __restrict__ b, double* out) {
  __shared__ double sh[kSumLanes][33];
  const int64_t i = blockIdx.x * 32LL + threadIdx.x;
  const int y = threadIdx.y;
  double s = 0.0;
  if (i < n) {
    const MolWork W = mw[mol_of_point(mw, nmol, i)];
    const int64_t at = W.poff + (i - W.p0);
    for (int k = y; k < W.nsplit; k += kSumLanes) s += a[at + static_cast<int64_t>(k) * W.np];
    if (b)
      for (int k = y; k < W.nsplit; k += kSumLanes) s += b[at + static_cast<int64_t>(k) * W.np];
  }
  sh[y][threadIdx.x] = s;
  __syncthreads();
  if (y == 0 && i < n) {
    double t = sh[0][threadIdx.x];
#pragma unroll
    for (int r = 1; r < kSumLanes; ++r) t += sh[r][threadIdx.x];
    out[i] = t;
  }
}

// Left-out bound mass of each tile: sum over its molecule's splits.
__global__ void __launch_bounds__(32 * kSumLanes)
k_sum_drop(int64_t ntiles, const MolWork* __restrict__ mw, int nmol, const double* __restrict__ d, double* out) {
  __shared__ double sh[kSumLanes][33];
  const int64_t t = blockIdx.x * 32LL + threadIdx.x;
  const int y = threadIdx.y;
  double s = 0.0;
  if (t < ntiles) {
    const MolWork W = mw[mol_of_tile(mw, nmol, t)];
    for (int k = y; k < W.nsplit; k += kSumLanes)
      s += d[W.doff + static_cast<int64_t>(k) * W.ntiles + (t - W.tile0)];
  }
  sh[y][threadIdx.x] = s;
  __syncthreads();
  if (y == 0 && t < ntiles) {
    double r0 = sh[0][threadIdx.x];
#pragma unroll
    for (int r = 1; r < kSumLanes; ++r) r0 += sh[r][threadIdx.x];
    out[t] = r0;
  }
}
inline unsigned nblk32(int64_t n) { return static_cast<unsigned>((n + 31) / 32); }
const dim3 kSumBlock(32, kSumLanes);

// ---- thresholds of the outputs, on the device (no host round trip between the passes)
// The threshold of an output: 3 sigma of the uncorrected rounding errors within the absolute
// budget B (tolerance times a lower bound of |O|, less the left-out bound mass):
// T = tscale B^2 / E_O.
__device__ __forceinline__ double tau_budget(double B, double M, double tscale) {
  return M > 0.0 ? tscale * B * B / M : HUGE_VAL;
}
__device__ __forceinline__ double ull_to_double(unsigned long long u) { return __longlong_as_double(static_cast<long long>(u)); }

// Estimates, segments of a radial or scan grid: the sampled sums sam[3s..3s+2] = (sum w I~,
// sum w E~, sum w) over the sampled points of segment s, all[3s+2] = sum w over all its points.
__global__ void k_thr_est_seg(int nseg, const double* __restrict__ sam, const double* __restrict__ all,
                              const int64_t* __restrict__ off, double eps, double tscale, double safety,
                              double drop_half, double nq, double* T, double* Theta) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const double wsam = sam[3 * s + 2], wtot = all[3 * s + 2];
  const double f = wsam > 0.0 ? wtot / wsam : 0.0;
  const double O = sam[3 * s] * f, M = sam[3 * s + 1] * f;
  const double lo = fmax(fabs(O) - M, 0.0);
  T[s] = (wsam > 0.0 && M > 0.0) ? safety * tau_budget(eps * lo, M, tscale) : 0.0;
  // drop threshold per point: theta_g = Theta / w_g with sum_g w_g nq theta_g at most
  // drop_frac eps |O| (half of it here, for the sampling error of the estimate)
  const double npts = static_cast<double>(off[s + 1] - off[s]);
  Theta[s] = wsam > 0.0 ? drop_half * eps * lo / (nq * fmax(npts, 1.0)) : 0.0;
}

// Estimates, cube (max-norm): from the sampled max |I~| and max E~.
__global__ void k_thr_est_max(const unsigned long long* __restrict__ mx, double eps, double tscale, double safety,
                              double margin, double drop_half, double nq, double* T, double* Theta) {
  if (threadIdx.x + blockIdx.x != 0) return;
  const double imax = ull_to_double(mx[0]), emax = ull_to_double(mx[1]);
  const double x = eps * imax;
  T[0] = emax > 0.0 ? safety * tscale * x * x / (margin * emax) : 0.0;
  Theta[0] = drop_half * eps * imax / nq;
}

// Exact thresholds, segments: sums ex[3s..] = (sum w I~, sum w E~, .) over all points and, with
// dropping, dd[3s] = sum w D (bound mass left out); *retry set when D took more than half the
// budget (the pass is then repeated without dropping).
__global__ void k_thr_exact_seg(int nseg, const double* __restrict__ ex, const double* __restrict__ dd, int use_drop,
                                double eps, double tscale, double* T, int* retry) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const double D = use_drop ? dd[3 * s] : 0.0;
  const double lo = fmax(fabs(ex[3 * s]) - ex[3 * s + 1] - D, 0.0);
  const double B = eps * lo - D;
  if (use_drop && B < 0.5 * eps * lo) atomicExch(retry, 1);
  T[s] = tau_budget(fmax(B, 0.0), ex[3 * s + 1], tscale);
}

// Exact threshold, cube: from max |I~| and the largest left-out mass of a tile.
__global__ void k_thr_exact_max(const unsigned long long* __restrict__ mx, const unsigned long long* __restrict__ mdrop,
                                int use_drop, double eps, double tscale, double* T, int* retry) {
  if (threadIdx.x + blockIdx.x != 0) return;
  const double imax = ull_to_double(mx[0]);
  const double dmx = use_drop ? ull_to_double(mdrop[0]) : 0.0;
  const double B = eps * imax - dmx;
  if (use_drop && B < 0.5 * eps * imax) atomicExch(retry, 1);
  const double b = fmax(B, 0.0);
  T[0] = tscale * b * b;
}

inline unsigned nblk(int64_t n, int bs = 256) { return static_cast<unsigned>((n + bs - 1) / bs); }

// Bump allocator over a scratch buffer: a dry run (base == nullptr) measures the size.
struct Carve {
  unsigned char* base;
  size_t off = 0;
  template <typename T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += n * sizeof(T);
    return p;
  }
};

// Default stride of the grid sample behind the threshold estimates: about 2 048 sampled points
// (a power of two between 16 and 64). Measured: the CH4 scan (62 390 points) runs fastest at 32,
// the 12-atom ring's radial grid (345 876 points) at 64 (9.96 s at 16, 9.15 s at 64), the CH4
// radial-integral grid (3 050 points) at 16.
int sample_stride_for(int64_t ngrid) {
  int s = static_cast<int>(kSampleStride);
  while (s < 64 && static_cast<int64_t>(s) * 2048 < ngrid) s *= 2;
  return s;
}

// Morton-sorted FP32 copy of the points g = j * stride of the grid (stride 1: all of it), the
// permutation (sorted position -> grid index) and the tile / sub-tile boxes.
int sort_points(inca_ctx* c, int64_t stride, int ppt, DevBuf<float4>& phi,
                DevBuf<float4>& plo, DevBuf<int64_t>& perm, DevBuf<float>& boxes, DevBuf<TileInfo>& tiles,
                int64_t* n_out, int64_t* ntiles_out, std::vector<MolSpan>& spans) {
  const int64_t n = (c->ngrid + stride - 1) / stride;
  const int64_t tile = 32 * static_cast<int64_t>(ppt);
  // tiles of <= 32 ppt consecutive sorted points; in a batch they never straddle two molecules
  std::vector<TileInfo> ht;
  const bool batch = c->batch_molecules > 0;
  const int nmol = batch ? c->batch_molecules : 1;
  int64_t o = 0;
  spans.assign(nmol, MolSpan{0, 0, 0, 0});
  for (int m = 0; m < nmol; ++m) {
    int64_t cnt = n;
    if (batch) {  // sampled points of molecule m: multiples of stride in [off_m, off_m+1)
      const int64_t a = c->h_mol_off[m], b = c->h_mol_off[m + 1];
      cnt = (b + stride - 1) / stride - (a + stride - 1) / stride;
    }
    spans[m] = MolSpan{static_cast<int64_t>(ht.size()), 0, o, cnt};
    for (int64_t t = 0; t < cnt; t += tile)
      ht.push_back(TileInfo{o + t, static_cast<int>(std::min<int64_t>(tile, cnt - t)), m});
    spans[m].ntiles = static_cast<int64_t>(ht.size()) - spans[m].tile0;
    o += cnt;
  }
  const int64_t nwt = static_cast<int64_t>(ht.size());
  if (phi.reserve(n) || plo.reserve(n) || perm.reserve(n) || boxes.reserve(8 * nwt + 8 * nwt * ppt) ||
      tiles.reserve(std::max<int64_t>(nwt, 1)))
    return set_error(c, INCA_E_NOMEM, "sorted grid");
  if (nwt) INCA_CUDA(c, cudaMemcpyAsync(tiles.p, ht.data(), sizeof(TileInfo) * nwt, cudaMemcpyHostToDevice, c->stream));
  // keys, indices and the radix sort's storage in the context's sort scratch (kept between calls)
  size_t tb = 0;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, tb, static_cast<uint64_t*>(nullptr),
                                                  static_cast<uint64_t*>(nullptr), static_cast<int64_t*>(nullptr),
                                                  static_cast<int64_t*>(nullptr), n, 0, 63, c->stream);
  if (e) return cuda_error(c, e, "morton sort");
  uint64_t *k1 = nullptr, *k2 = nullptr;
  int64_t* i1 = nullptr;
  unsigned char* tmp = nullptr;
  auto layout = [&](Carve& cv) {
    k1 = cv.take<uint64_t>(n);
    k2 = cv.take<uint64_t>(n);
    i1 = cv.take<int64_t>(n);
    tmp = cv.take<unsigned char>(tb);
  };
  Carve dry{nullptr};
  layout(dry);
  if (c->d_sscratch.reserve(dry.off + 256)) return set_error(c, INCA_E_NOMEM, "morton sort");
  Carve cv{c->d_sscratch.p};
  layout(cv);
  INCA_LAUNCH(c, k_morton, nblk(n), 256, 0, n, stride, c->d_px.p, c->d_py.p, c->d_pz.p,
              batch ? c->d_pmol.p : nullptr, c->d_bbox.p, k1, i1);
  e = cub::DeviceRadixSort::SortPairs(tmp, tb, k1, k2, i1, perm.p, n, 0, 63, c->stream);
  if (!e) {
    INCA_LAUNCH(c, k_gather_points, nblk(n), 256, 0, n, perm.p, c->d_px.p, c->d_py.p, c->d_pz.p, phi.p, plo.p);
    const unsigned bb = static_cast<unsigned>((nwt + 7) / 8);
    if (ppt == 3)
      INCA_LAUNCH(c, k_boxes<3>, bb, 256, 0, tiles.p, nwt, phi.p, plo.p, boxes.p, boxes.p + 8 * nwt);
    else if (ppt == 5)
      INCA_LAUNCH(c, k_boxes<5>, bb, 256, 0, tiles.p, nwt, phi.p, plo.p, boxes.p, boxes.p + 8 * nwt);
    else
      INCA_LAUNCH(c, k_boxes<4>, bb, 256, 0, tiles.p, nwt, phi.p, plo.p, boxes.p, boxes.p + 8 * nwt);
    e = cudaGetLastError();
  }
  if (e) return cuda_error(c, e, "sorted grid");
  *n_out = n;
  *ntiles_out = nwt;
  return INCA_OK;
}

// The sorted grid (and, for the one-pass form, the sorted sample), rebuilt when the grid changes.
int prepare_sorted_grid(inca_ctx* c, bool sample, int ppt) {
  const int stride = c->tune_sample_stride > 0 ? c->tune_sample_stride : sample_stride_for(c->ngrid);
  const bool main_ok = c->mix_version == c->grid_version && c->mix_ppt == ppt;
  const bool sample_ok = !sample || (c->sample_version == c->grid_version && c->sample_stride_built == stride);
  if (main_ok && sample_ok) return INCA_OK;
  const int64_t n = c->ngrid;
  // bounding box of the grid and the Morton key scale, reduced on the device and read there
  if (c->d_bbox.reserve(7)) return set_error(c, INCA_E_NOMEM, "bounding box");
  INCA_LAUNCH(c, k_bbox, 1, 1024, 0, n, c->d_px.p, c->d_py.p, c->d_pz.p, c->d_bbox.p);
  int64_t nn = 0;
  if (!main_ok) {
    const int st = sort_points(c, 1, ppt, c->d_phi, c->d_plo, c->d_perm, c->d_wtbox, c->d_tiles, &nn,
                               &c->ntiles, c->mol_span);
    if (st) return st;
    c->mix_version = c->grid_version;
    c->mix_ppt = ppt;
  }
  if (!sample_ok) {
    const int st = sort_points(c, stride, kSamplePPT, c->d_phi_s, c->d_plo_s, c->d_perm_s, c->d_wtbox_s,
                               c->d_tiles_s, &c->nsample, &c->ntiles_s, c->mol_span_s);
    if (st) return st;
    c->sample_version = c->grid_version;
    c->sample_stride_built = stride;
  }
  return INCA_OK;
}


struct Events {
  cudaEvent_t e[6] = {};
  ~Events() {
    for (auto& x : e)
      if (x) cudaEventDestroy(x);
  }
};

// 2^(j/256), j = -128..128, as float pairs (host, double precision).
std::vector<float2> exp2_table() {
  std::vector<float2> t(kExpTab + 1);
  for (int j = 0; j <= kExpTab; ++j) {
    const double v = std::exp2(double(j - kExpTab / 2) / kExpTab);
    const float h = static_cast<float>(v);
    t[j] = make_float2(h, static_cast<float>(v - static_cast<double>(h)));
  }
  return t;
}

// Work table of a persistent pass over a sorted grid: each molecule's quartet splits in
// proportion to its tiles x chunks, about kItemsPerCta work items per resident CTA in total
// (an item is then small next to the whole pass, so the CTAs finish together).
std::vector<MolWork> work_table(const std::vector<MolSpan>& sp, const std::vector<ChunkRange>& ch, int num_sms,
                                int items_per_cta, int64_t* nitems, int64_t* npart, int64_t* ndrop,
                                int ctas_per_sm = INCA_PASS_CTAS_PER_SM) {
  const int nmol = static_cast<int>(sp.size());
  const double target = double(num_sms) * ctas_per_sm * items_per_cta;
  double total = 0.0;
  for (int m = 0; m < nmol; ++m) total += double(sp[m].ntiles) * std::max(ch[m].end - ch[m].begin, 0);
  std::vector<MolWork> w(nmol);
  int64_t it = 0, po = 0, dro = 0;
  for (int m = 0; m < nmol; ++m) {
    const int nch = std::max(ch[m].end - ch[m].begin, 0);
    int64_t ns = 1;
    if (sp[m].ntiles > 0 && nch > 0 && total > 0.0) {
      const double items = target * double(sp[m].ntiles) * nch / total;
      ns = std::llround(items / double(sp[m].ntiles));
      ns = std::max<int64_t>(1, std::min<int64_t>(ns, std::min(nch, 4096)));
    }
    w[m] = MolWork{ch[m].begin, ch[m].end, static_cast<int>(ns), 0, sp[m].tile0, sp[m].ntiles, sp[m].p0, sp[m].np,
                   it, po, dro};
    it += sp[m].ntiles * ns;
    po += ns * sp[m].np;
    dro += ns * sp[m].ntiles;
  }
  *nitems = it;
  *npart = po;
  *ndrop = dro;
  return w;
}

// Resident CTAs of a persistent pass launch (one-warp CTAs, ctas_per_sm per SM).
unsigned persistent_ctas(int64_t nitems, int num_sms, int ctas_per_sm = INCA_PASS_CTAS_PER_SM) {
  return static_cast<unsigned>(
      std::max<int64_t>(1, std::min<int64_t>(nitems, static_cast<int64_t>(num_sms) * ctas_per_sm)));
}

// Points per lane of the one-pass kernel when the schedule sets none, from the mean surviving
// records per molecule. Measured at the default schedule otherwise (16 CTAs per SM): CH4
// (1.1e5 records; radial integrals at 3 050 and 30 200 points, I(s) at 31 490 and 62 390)
// and ten small batch molecules ran 1-10% faster at 3 than at 4 and slower at 5; the 12-atom
// ring (5.1e7 records; 89 614 and 345 876 points) ran 5-7% faster at 5 and slower at 3.
int default_ppt(const inca_ctx* c) {
  const double per_mol = static_cast<double>(c->nsurv) / std::max<size_t>(1, c->mol_chunks.size());
  return per_mol <= kFewRecords ? 3 : per_mol >= kManyRecords ? 5 : kDefaultPPT;
}

}  // namespace

// The shapes the one-pass kernel is compiled for: points per lane (tile of 32 ppt points) and
// register budget (resident one-warp CTAs per SM); the schedule (inca_set_tuning,
// inca_autotune) picks one. Five points per lane need the larger budgets, three the smaller.
bool valid_pass_shape(int ppt, int ctas) {
  if (ppt == 4) return ctas == 12 || ctas == 16 || ctas == 20;
  if (ppt == 3) return ctas == 16 || ctas == 20;
  if (ppt == 5) return ctas == 12 || ctas == 16;
  return false;
}

namespace {

double env_knob(const char* name, double dflt, double lo, double hi) {
  if (const char* env = std::getenv(name)) {
    char* end = nullptr;
    const double v = std::strtod(env, &end);
    if (end != env && std::isfinite(v) && v >= lo && v < hi) return v;
  }
  return dflt;
}

// Everything an evaluation needs that the host decides: sizes, knobs, buffers (carved from the
// context's scratch) and uploaded tables. The launch sequence then runs on the device alone.
struct MixedPlan {
  bool fused = false;
  int mode = 2, nseg = 1, emode = 0, nmol = 1, cheap = 1, wait_test = 0;
  int ctas = INCA_PASS_CTAS_PER_SM;  // resident CTAs per SM of the one-pass kernel (its register budget)
  int ppt = kDefaultPPT;             // points per lane of the main grid's tiles
  bool f64 = false;  // the screened FP64 form (k_pass_f64 instead of the FP32 passes)
  const int* seg_of = nullptr;
  int64_t ngrid = 0, nwt = 0, ngroups = 0, nitems = 0, npart = 0, ndrop = 0;
  int64_t ns = 0, nitems_s = 0, npart_s = 0;
  unsigned nctas = 1, nctas_s = 1, gblk = 1, tblk = 1;
  int stage_floats = 0;
  size_t dsmem = 0;
  double eps = 0, tau_scale = 0, safety = 0, drop_frac = 0, nq = 1;
  double *p1, *pabs, *p2, *Is, *Ms, *Io, *Mo, *dsam, *dall, *dex, *ddrop, *dTest, *dTheta, *dT, *dmass, *Dt, *Dpt;
  double *q1 = nullptr, *qabs = nullptr, *Iss = nullptr, *Mss = nullptr, *Ios = nullptr, *Mos = nullptr, *ws = nullptr;
  float *glt, *ptau, *ptau_est, *ptheta, *ltdrop;
  unsigned long long *stats, *dmax, *dmax2, *work;
  MolWork *mwdev, *mws = nullptr;
  int *errw, *retry;
  int64_t* doff;
  const float2* tab;
};

int mixed_plan(inca_ctx* c, double eps, MixedPlan& P) {
  P.ngrid = c->ngrid;
  const int64_t ngrid = P.ngrid;
  const double fuse_min = env_knob("INCA_FUSE_MIN_POINTS", static_cast<double>(kFuseMinPoints), 256.0, HUGE_VAL);
  P.fused = (c->grid_kind == GRID_RADIAL || c->grid_kind == GRID_SCAN || c->grid_kind == GRID_CUBE) &&
            static_cast<double>(ngrid) >= fuse_min;
  // test of the bounded staging waits: the pass-1 kernels start no copy and give up waiting
  // after this many tries (0: off)
  P.wait_test = static_cast<int>(env_knob("INCA_TEST_STAGE_TIMEOUT", 0.0, 0.0, 1e6));
  // the shape of the one-pass kernel (the two-pass form and the wait test use the default)
  int tppt = c->tune_ppt > 0 ? c->tune_ppt : default_ppt(c);
  const int tctas = c->tune_ctas > 0 ? c->tune_ctas : INCA_PASS_CTAS_PER_SM;
  if (c->tune_ppt <= 0 && !valid_pass_shape(tppt, tctas)) tppt = kDefaultPPT;  // the budget asked for
  if (P.fused && P.wait_test == 0 && valid_pass_shape(tppt, tctas)) {
    P.ppt = tppt;
    P.ctas = tctas;
  }
  int st = prepare_sorted_grid(c, P.fused, P.ppt);
  if (st) return st;
  P.eps = eps;
  // knobs (environment, read per evaluation; tuning and test aids)
  P.tau_scale = env_knob("INCA_TAU_SCALE", kTauScale, 1e-300, HUGE_VAL);
  P.drop_frac = env_knob("INCA_DROP_FRACTION", c->tune_drop >= 0.0 ? c->tune_drop : kDropFrac, 0.0, 0.5);
  P.safety = env_knob("INCA_EST_SAFETY", c->tune_safety >= 0.0 ? c->tune_safety : kEstSafety, 0.0, HUGE_VAL);
  // the cheap tier of the one-pass form (0 evaluates every live pair in compensated FP32), and
  // its slack: a pair takes the tier when its error bound is at most 2^slack times the drop
  // threshold (0: within the threshold, so the left-out mass keeps its a-priori bound; larger:
  // checked after the pass like the rest of the left-out mass). Passed to the kernels as
  // 0 (off) or 1 + slack.
  const int slack = static_cast<int>(env_knob("INCA_CHEAP_SLACK", c->tune_cheap_slack >= 0 ? c->tune_cheap_slack
                                                                                           : kCheapSlack,
                                              0.0, 31.0));
  P.cheap = env_knob("INCA_CHEAP_TIER", 1.0, 0.0, 2.0) >= 0.5 ? 1 + slack : 0;
  P.nwt = c->ntiles;
  P.ngroups = P.nwt * P.ppt;
  const int ipc = c->tune_items_per_cta > 0 ? c->tune_items_per_cta : kItemsPerCta;
  const std::vector<MolWork> hmw =
      work_table(c->mol_span, c->mol_chunks, c->num_sms, ipc, &P.nitems, &P.npart, &P.ndrop, P.ctas);
  P.nmol = static_cast<int>(hmw.size());
  P.nctas = persistent_ctas(P.nitems, c->num_sms, P.ctas);
  std::vector<MolWork> hmw_s;
  if (P.fused) {
    P.ns = c->nsample;
    int64_t ndrop_s = 0;
    // the sample has 1/stride of the tiles: with the main pass's item count its items would
    // hold a chunk or two each and their fixed costs (points, box, first stage, partial sums)
    // would rival the work; at most 4 items per CTA measured best
    const int ipc_s = static_cast<int>(env_knob("INCA_SAMPLE_ITEMS_PER_CTA", std::min(ipc, 4), 1, 1e6));
    hmw_s = work_table(c->mol_span_s, c->mol_chunks, c->num_sms, ipc_s, &P.nitems_s, &P.npart_s, &ndrop_s);
    P.nctas_s = persistent_ctas(P.nitems_s, c->num_sms);
  }
  // survivors of the largest molecule: an upper bound on the terms left out at a point
  P.nq = static_cast<double>(std::max<int64_t>(*std::max_element(c->mol_surv.begin(), c->mol_surv.end()), 1));
  // outputs and their segments: radial grid (one integral), scan grid (one I(s) per shell),
  // cube (max-norm), explicit points (each point)
  std::vector<int64_t> off;
  if (c->grid_kind == GRID_RADIAL) {
    P.mode = 0;
    off = {0, ngrid};
  } else if (c->grid_kind == GRID_SCAN) {
    P.mode = 0;
    off.assign(c->nradi + 1, 0);
    for (int s = 0; s < c->nradi; ++s) off[s + 1] = off[s] + c->h_smn[s];
    P.seg_of = c->d_cmap.p;  // shell of each scan point
  } else if (c->grid_kind == GRID_CUBE) {
    P.mode = 1;
  }
  P.emode = P.mode == 0 ? 0 : 3;
  P.nseg = off.empty() ? 1 : static_cast<int>(off.size()) - 1;
  const int nseg = P.nseg;
  auto layout = [&](Carve& cv) {
    P.p1 = cv.take<double>(P.npart);
    P.pabs = cv.take<double>(P.npart);
    P.p2 = cv.take<double>(P.npart);
    P.Is = cv.take<double>(ngrid);
    P.Ms = cv.take<double>(ngrid);
    P.Io = cv.take<double>(ngrid);
    P.Mo = cv.take<double>(ngrid);
    P.glt = cv.take<float>(P.ngroups);
    P.ptau = cv.take<float>(ngrid);
    P.ptau_est = cv.take<float>(P.fused ? ngrid : 1);
    P.ptheta = cv.take<float>(P.fused ? ngrid : 1);
    P.ltdrop = cv.take<float>(P.fused ? P.nwt : 1);
    P.dmass = cv.take<double>(P.fused ? P.ndrop : 1);
    P.Dt = cv.take<double>(P.fused ? P.nwt : 1);
    P.Dpt = cv.take<double>(P.fused ? ngrid : 1);
    P.stats = cv.take<unsigned long long>(16);
    P.work = cv.take<unsigned long long>(4);
    P.mwdev = cv.take<MolWork>(P.nmol);
    P.mws = cv.take<MolWork>(P.nmol);
    P.dmax = cv.take<unsigned long long>(2);
    P.dmax2 = cv.take<unsigned long long>(2);
    P.errw = cv.take<int>(4);
    P.retry = cv.take<int>(4);
    P.dsam = cv.take<double>(3 * nseg);
    P.dall = cv.take<double>(3 * nseg);
    P.dex = cv.take<double>(3 * nseg);
    P.ddrop = cv.take<double>(3 * nseg);
    P.dTest = cv.take<double>(nseg);
    P.dTheta = cv.take<double>(nseg);
    P.dT = cv.take<double>(nseg);
    P.doff = cv.take<int64_t>(nseg + 1);
  };
  Carve dry{nullptr};
  layout(dry);
  if (c->d_scratch.reserve(dry.off + 256)) return set_error(c, INCA_E_NOMEM, "mixed scratch");
  Carve cv{c->d_scratch.p};
  layout(cv);
  if (P.fused) {
    auto layout_s = [&](Carve& cs) {
      P.q1 = cs.take<double>(P.npart_s);
      P.qabs = cs.take<double>(P.npart_s);
      P.Iss = cs.take<double>(P.ns);
      P.Mss = cs.take<double>(P.ns);
      P.Ios = cs.take<double>(ngrid);
      P.Mos = cs.take<double>(ngrid);
      P.ws = cs.take<double>(ngrid);
    };
    Carve dry_s{nullptr};
    layout_s(dry_s);
    if (c->d_scratch_s.reserve(dry_s.off + 256)) return set_error(c, INCA_E_NOMEM, "sample scratch");
    Carve cs{c->d_scratch_s.p};
    layout_s(cs);
  }
  if ((st = ensure_exp_table(c))) return st;
  P.tab = c->d_exptab.p;
  INCA_CUDA(c, cudaMemcpyAsync(P.mwdev, hmw.data(), sizeof(MolWork) * P.nmol, cudaMemcpyHostToDevice, c->stream));
  if (P.fused)
    INCA_CUDA(c, cudaMemcpyAsync(P.mws, hmw_s.data(), sizeof(MolWork) * P.nmol, cudaMemcpyHostToDevice, c->stream));
  if (!off.empty())
    INCA_CUDA(c, cudaMemcpyAsync(P.doff, off.data(), sizeof(int64_t) * (nseg + 1), cudaMemcpyHostToDevice, c->stream));
  INCA_CUDA(c, cudaStreamSynchronize(c->stream));  // the host tables above are stack-owned
  int max_stride = 4;
  for (const ClassSeg& sg : c->classes) max_stride = std::max(max_stride, sg.stride32);
  if (max_stride > kMaxStride32) return set_error(c, INCA_E_LIMIT, "inca_eval: record stride above the maximum");
  P.stage_floats = kChunkMax * max_stride;
  P.dsmem = 128 + 2 * sizeof(float) * P.stage_floats;
  P.gblk = static_cast<unsigned>((P.ngroups + 7) / 8);
  P.tblk = static_cast<unsigned>((P.nwt + 7) / 8);
  return INCA_OK;
}

// The device work of one evaluation (no host synchronisation: it can be captured in a graph).
// ev (optional) gets events around the pass over all terms and the correction pass. kPPT: points
// per lane of the main grid's tiles (the sample's are always kSamplePPT).
template <int kPPT>
int mixed_launch_t(inca_ctx* c, const MixedPlan& P, bool use_drop, Events* ev) {
  const int64_t ngrid = P.ngrid, nwt = P.nwt;
  const int nseg = P.nseg;
  const TileInfo* tiles = c->d_tiles.p;
  const float* wbox = c->d_wtbox.p;
  const float* gbox = c->d_wtbox.p + 8 * nwt;
  INCA_CUDA(c, cudaMemsetAsync(P.stats, 0, 16 * sizeof(unsigned long long), c->stream));
  INCA_CUDA(c, cudaMemsetAsync(P.work, 0, 4 * sizeof(unsigned long long), c->stream));
  INCA_CUDA(c, cudaMemsetAsync(P.errw, 0, 4 * sizeof(int), c->stream));
  INCA_CUDA(c, cudaMemsetAsync(P.retry, 0, 4 * sizeof(int), c->stream));
  if (ev) INCA_CUDA(c, cudaEventRecord(ev->e[0], c->stream));
  const unsigned sblk = static_cast<unsigned>((nseg + 127) / 128);
  // ---- estimates from the grid sample (one-pass form): thresholds and drop thresholds
  if (P.fused) {
    const int64_t ns = P.ns;
#define INCA_PASS1_EST(T)                                                                                         \
  INCA_LAUNCH(c, (k_pass1<false, true, INCA_PASS_CTAS_PER_SM, T, kSamplePPT>), P.nctas_s, 32, P.dsmem, c->d_chunks.p, P.mws,     \
              P.nmol, c->d_classes.p, c->d_rec32.p, c->d_phi_s.p, c->d_plo_s.p, c->d_tiles_s.p, c->d_wtbox_s.p,     \
              P.nitems_s, P.stage_floats, nullptr, nullptr, nullptr, 0, P.q1, P.qabs, nullptr, P.work + 3,          \
              P.stats + 8, P.errw, P.wait_test)
    if (P.wait_test > 0)
      INCA_PASS1_EST(true);
    else
      INCA_PASS1_EST(false);
#undef INCA_PASS1_EST
    INCA_LAUNCH(c, k_sum_mol, nblk32(ns), kSumBlock, 0, ns, P.mws, P.nmol, P.q1, nullptr, P.Iss);
    INCA_LAUNCH(c, k_sum_mol, nblk32(ns), kSumBlock, 0, ns, P.mws, P.nmol, P.qabs, nullptr, P.Mss);
    if (P.mode == 0) {
      INCA_CUDA(c, cudaMemsetAsync(P.Ios, 0, sizeof(double) * ngrid, c->stream));
      INCA_CUDA(c, cudaMemsetAsync(P.Mos, 0, sizeof(double) * ngrid, c->stream));
      INCA_CUDA(c, cudaMemsetAsync(P.ws, 0, sizeof(double) * ngrid, c->stream));
      INCA_LAUNCH(c, k_scatter_sample, nblk(ns), 256, 0, ns, c->d_perm_s.p, P.Iss, P.Mss, c->d_w.p, P.Ios, P.Mos, P.ws);
      INCA_LAUNCH(c, k_seg_sums, nseg, 256, 0, nseg, P.doff, P.ws, P.Ios, P.Mos, P.dsam);
      INCA_LAUNCH(c, k_seg_sums, nseg, 256, 0, nseg, P.doff, c->d_w.p, P.Ios, P.Mos, P.dall);
      INCA_LAUNCH(c, k_thr_est_seg, sblk, 128, 0, nseg, P.dsam, P.dall, P.doff, P.eps, P.tau_scale, P.safety,
                  0.5 * P.drop_frac, P.nq, P.dTest, P.dTheta);
    } else {
      INCA_CUDA(c, cudaMemsetAsync(P.dmax, 0, 2 * sizeof(unsigned long long), c->stream));
      INCA_LAUNCH(c, k_absmax2, static_cast<unsigned>(std::min<int64_t>(nblk(ns), 4096)), 256, 0, ns, P.Iss, P.Mss,
                  P.dmax);
      INCA_LAUNCH(c, k_thr_est_max, 1, 32, 0, P.dmax, P.eps, P.tau_scale, P.safety, kCubeMargin, 0.5 * P.drop_frac,
                  P.nq, P.dTest, P.dTheta);
    }
    INCA_LAUNCH(c, k_thresholds<kPPT>, P.gblk, 256, 0, tiles, P.ngroups, P.emode, c->d_perm.p, P.seg_of, P.dTest, c->d_w.p,
                nullptr, nullptr, P.eps, P.tau_scale, nullptr, P.ptau_est);
    if (use_drop) {
      INCA_LAUNCH(c, k_thresholds<kPPT>, P.gblk, 256, 0, tiles, P.ngroups, P.emode, c->d_perm.p, P.seg_of, P.dTheta,
                  c->d_w.p, nullptr, nullptr, P.eps, P.tau_scale, nullptr, P.ptheta);
      INCA_LAUNCH(c, k_tile_min_log2<kPPT>, P.tblk, 256, 0, tiles, nwt, P.ptheta, P.ltdrop);
    }
  }
  // ---- the pass over all terms (one-pass form: corrections above the estimated thresholds,
  // terms below the drop thresholds left out)
  if (ev) INCA_CUDA(c, cudaEventRecord(ev->e[1], c->stream));
  if (P.f64)
    INCA_LAUNCH(c, k_pass_f64<kPPT>, P.nctas, 32, P.dsmem, c->d_chunks.p, P.mwdev, P.nmol, c->d_classes.p, c->d_rec32.p,
                c->d_phi.p, c->d_plo.p, tiles, wbox, P.nitems, P.stage_floats, use_drop ? P.ltdrop : nullptr, P.p1,
                P.pabs, use_drop ? P.dmass : nullptr, P.work, P.stats, P.errw);
  else if (P.fused) {
#define INCA_PASS1_FUSED(N, T)                                                                                    \
  INCA_LAUNCH(c, (k_pass1<true, false, N, T, kPPT>), P.nctas, 32, P.dsmem, c->d_chunks.p, P.mwdev, P.nmol,          \
              c->d_classes.p, c->d_rec32.p, c->d_phi.p, c->d_plo.p, tiles, wbox, P.nitems, P.stage_floats,         \
              P.ptau_est, P.tab, use_drop ? P.ltdrop : nullptr, P.cheap, P.p1, P.pabs, P.dmass, P.work, P.stats,    \
              P.errw, P.wait_test)
    // the shapes valid_pass_shape admits (the wait test runs at the default shape only)
    if constexpr (kPPT == kDefaultPPT) {
      if (P.wait_test > 0)
        INCA_PASS1_FUSED(INCA_PASS_CTAS_PER_SM, true);
      else if (P.ctas == 12)
        INCA_PASS1_FUSED(12, false);
      else if (P.ctas == 20)
        INCA_PASS1_FUSED(20, false);
      else
        INCA_PASS1_FUSED(16, false);
    } else if constexpr (kPPT == 3) {
      if (P.ctas == 20)
        INCA_PASS1_FUSED(20, false);
      else
        INCA_PASS1_FUSED(16, false);
    } else {
      if (P.ctas == 12)
        INCA_PASS1_FUSED(12, false);
      else
        INCA_PASS1_FUSED(16, false);
    }
#undef INCA_PASS1_FUSED
  } else if constexpr (kPPT == kDefaultPPT) {  // the two-pass form: default shape only
    if (P.wait_test > 0)
      INCA_LAUNCH(c, (k_pass1<false, false, INCA_PASS_CTAS_PER_SM, true>), P.nctas, 32, P.dsmem, c->d_chunks.p,
                  P.mwdev, P.nmol, c->d_classes.p, c->d_rec32.p, c->d_phi.p, c->d_plo.p, tiles, wbox, P.nitems,
                  P.stage_floats, nullptr, nullptr, nullptr, 0, P.p1, P.pabs, nullptr, P.work, P.stats, P.errw,
                  P.wait_test);
    else
      INCA_LAUNCH(c, k_pass1<false>, P.nctas, 32, P.dsmem, c->d_chunks.p, P.mwdev, P.nmol, c->d_classes.p,
                  c->d_rec32.p, c->d_phi.p, c->d_plo.p, tiles, wbox, P.nitems, P.stage_floats, nullptr, nullptr,
                  nullptr, 0, P.p1, P.pabs, nullptr, P.work, P.stats, P.errw, 0);
  } else {
    return set_error(c, INCA_E_STATE, "inca_eval: the two-pass form runs at the default tile shape");
  }
  if (ev) INCA_CUDA(c, cudaEventRecord(ev->e[2], c->stream));
  INCA_LAUNCH(c, k_sum_mol, nblk32(ngrid), kSumBlock, 0, ngrid, P.mwdev, P.nmol, P.p1, nullptr, P.Is);
  INCA_LAUNCH(c, k_sum_mol, nblk32(ngrid), kSumBlock, 0, ngrid, P.mwdev, P.nmol, P.pabs, nullptr, P.Ms);
  INCA_LAUNCH(c, k_scatter, nblk(ngrid), 256, 0, ngrid, c->d_perm.p, P.Is, P.Io);
  if (use_drop) {
    INCA_LAUNCH(c, k_sum_drop, nblk32(nwt), kSumBlock, 0, nwt, P.mwdev, P.nmol, P.dmass, P.Dt);
    INCA_LAUNCH(c, k_tile_to_points, P.tblk, 256, 0, tiles, nwt, c->d_perm.p, P.Dt, P.Dpt);
  }
  // ---- exact thresholds of the outputs
  if (P.mode == 0) {
    INCA_LAUNCH(c, k_scatter, nblk(ngrid), 256, 0, ngrid, c->d_perm.p, P.Ms, P.Mo);
    INCA_LAUNCH(c, k_seg_sums, nseg, 256, 0, nseg, P.doff, c->d_w.p, P.Io, P.Mo, P.dex);
    if (use_drop) INCA_LAUNCH(c, k_seg_sums, nseg, 256, 0, nseg, P.doff, c->d_w.p, P.Dpt, P.Dpt, P.ddrop);
    INCA_LAUNCH(c, k_thr_exact_seg, sblk, 128, 0, nseg, P.dex, P.ddrop, use_drop ? 1 : 0, P.eps, P.tau_scale, P.dT,
                P.retry);
  } else if (P.mode == 1) {
    INCA_CUDA(c, cudaMemsetAsync(P.dmax, 0, 2 * sizeof(unsigned long long), c->stream));
    INCA_LAUNCH(c, k_absmax2, static_cast<unsigned>(std::min<int64_t>(nblk(ngrid), 4096)), 256, 0, ngrid, P.Is, P.Ms,
                P.dmax);
    if (use_drop) {
      INCA_CUDA(c, cudaMemsetAsync(P.dmax2, 0, 2 * sizeof(unsigned long long), c->stream));
      INCA_LAUNCH(c, k_absmax2, static_cast<unsigned>(std::min<int64_t>(nblk(nwt), 4096)), 256, 0, nwt, P.Dt, P.Dt,
                  P.dmax2);
    }
    INCA_LAUNCH(c, k_thr_exact_max, 1, 32, 0, P.dmax, P.dmax2, use_drop ? 1 : 0, P.eps, P.tau_scale, P.dT, P.retry);
  } else {
    INCA_CUDA(c, cudaMemsetAsync(P.dT, 0, sizeof(double), c->stream));
  }
  INCA_LAUNCH(c, k_thresholds<kPPT>, P.gblk, 256, 0, tiles, P.ngroups, P.mode, c->d_perm.p, P.seg_of, P.dT, c->d_w.p, P.Is,
              P.Ms, P.eps, P.tau_scale, P.fused ? nullptr : P.glt, P.ptau);
  // sub-tiles where an exact threshold fell below its estimate (the correction pass skips
  // every item whose tile has none)
  if (P.fused) INCA_LAUNCH(c, k_band<kPPT>, P.gblk, 256, 0, tiles, P.ngroups, P.ptau, P.ptau_est, P.glt, P.stats + 12);
  if (ev) INCA_CUDA(c, cudaEventRecord(ev->e[3], c->stream));
  if (!P.f64) {  // the screened FP64 form has nothing to correct
    INCA_LAUNCH(c, k_pass2<kPPT>, P.nctas, 32, P.dsmem, c->d_chunks.p, P.mwdev, P.nmol, c->d_classes.p, c->d_rec32.p,
                c->d_phi.p, c->d_plo.p, tiles, wbox, gbox, P.glt, P.ptau, P.fused ? P.ptau_est : nullptr,
                use_drop ? P.ltdrop : nullptr, P.cheap, P.tab, P.nitems, P.stage_floats, P.p2, P.work + 1,
                P.stats + 4, P.errw);
  }
  if (ev) INCA_CUDA(c, cudaEventRecord(ev->e[4], c->stream));
  INCA_LAUNCH(c, k_sum_mol, nblk32(ngrid), kSumBlock, 0, ngrid, P.mwdev, P.nmol, P.p1, P.f64 ? nullptr : P.p2,
              P.Is);
  INCA_LAUNCH(c, k_scatter, nblk(ngrid), 256, 0, ngrid, c->d_perm.p, P.Is, c->d_ivec.p);
  if (ev) INCA_CUDA(c, cudaEventRecord(ev->e[5], c->stream));
  INCA_CUDA(c, cudaGetLastError());
  return INCA_OK;
}

int mixed_launch(inca_ctx* c, const MixedPlan& P, bool use_drop, Events* ev) {
  switch (P.ppt) {
    case 3: return mixed_launch_t<3>(c, P, use_drop, ev);
    case 5: return mixed_launch_t<5>(c, P, use_drop, ev);
    default: return mixed_launch_t<kDefaultPPT>(c, P, use_drop, ev);
  }
}

// After the device work: errors, the retry flag, statistics and (with events) timings.
int mixed_finish(inca_ctx* c, const MixedPlan& P, Events* ev, bool* retry) {
  INCA_CUDA(c, cudaStreamSynchronize(c->stream));
  unsigned long long hs[16] = {};
  int herr = 0, hretry = 0;
  INCA_CUDA(c, cudaMemcpy(hs, P.stats, sizeof(hs), cudaMemcpyDeviceToHost));
  INCA_CUDA(c, cudaMemcpy(&herr, P.errw, sizeof(int), cudaMemcpyDeviceToHost));
  INCA_CUDA(c, cudaMemcpy(&hretry, P.retry, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) return set_error(c, INCA_E_TIMEOUT, "inca_eval: a bounded wait for a staged quartet chunk gave up");
  *retry = hretry != 0;
  if (ev) {
    float t12 = 0, t34 = 0, t05 = 0;
    cudaEventElapsedTime(&t12, ev->e[1], ev->e[2]);
    cudaEventElapsedTime(&t34, ev->e[3], ev->e[4]);
    cudaEventElapsedTime(&t05, ev->e[0], ev->e[5]);
    c->t_total_ms = t05;
    c->t_kernel_ms = t12;  // the pass over all terms
    c->t_pass2_ms = t34;   // the correction pass
  }
  c->t_kernel_launches = 1;
  if (P.fused) {
    // one-pass kernel: live pairs, warp rounds of corrections (one corrected term per active
    // lane), exact corrected-term count; correction pass: candidate pairs and corrected terms
    // in warps of 32 points
    c->pairs_fp32 = static_cast<int64_t>(hs[0]);
    c->pairs_fp64 = static_cast<int64_t>(hs[1]) + static_cast<int64_t>(hs[5]);
    c->pairs_skip = static_cast<int64_t>(hs[2]);
    c->corrected_points = static_cast<int64_t>(hs[3]) + static_cast<int64_t>(hs[7]);
    c->pairs_cheap = static_cast<int64_t>(hs[13]);
  } else {
    c->pairs_cheap = 0;
    c->pairs_fp32 = static_cast<int64_t>(hs[4]);
    c->pairs_fp64 = static_cast<int64_t>(hs[5]);
    c->pairs_skip = static_cast<int64_t>(hs[2]);
    c->corrected_points = static_cast<int64_t>(hs[7]);
  }
  return INCA_OK;
}

}  // namespace

// The double-float exp2 table of the context (uploaded once).
int ensure_exp_table(inca_ctx* c) {
  if (c->d_exptab.n != 0) return INCA_OK;
  if (c->d_exptab.reserve(kExpTab + 1)) return set_error(c, INCA_E_NOMEM, "exp table");
  const std::vector<float2> htab = exp2_table();
  INCA_CUDA(c, cudaMemcpy(c->d_exptab.p, htab.data(), sizeof(float2) * htab.size(), cudaMemcpyHostToDevice));
  return INCA_OK;
}

int eval_mixed(inca_ctx* c, double eps) {
  if (cube_separable(c)) return eval_cube_separable(c, eps);  // cube lattices: cube_eval.cu
  if (c->chunks.empty()) {
    INCA_CUDA(c, cudaMemsetAsync(c->d_ivec.p, 0, sizeof(double) * c->ngrid, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    return INCA_OK;
  }
  const int64_t launches0 = c->launches;
  MixedPlan P;
  int st = mixed_plan(c, eps, P);
  if (st) return st;
  Events ev;
  for (auto& e : ev.e) INCA_CUDA(c, cudaEventCreate(&e));
  bool use_drop = P.fused && P.drop_frac > 0.0, retry = false;
  if ((st = mixed_launch(c, P, use_drop, &ev))) return st;
  if ((st = mixed_finish(c, P, &ev, &retry))) return st;
  if (retry && use_drop) {  // too much was left out: once more without leaving terms out
    if ((st = mixed_launch(c, P, false, &ev))) return st;
    if ((st = mixed_finish(c, P, &ev, &retry))) return st;
  }
  c->t_launches = static_cast<int>(c->launches - launches0);
  return INCA_OK;
}

// The screened FP64 form: the one-pass form's plan (estimate pass, drop thresholds, left-out mass
// check and repetition without leaving out) with k_pass_f64 as the pass over all terms. Grids
// below the one-pass size, and cube lattices, have no drop thresholds: there it is the FP64 form.
int eval_fp64_screened(inca_ctx* c, double eps, bool* plain) {
  *plain = false;
  if (c->chunks.empty()) {
    INCA_CUDA(c, cudaMemsetAsync(c->d_ivec.p, 0, sizeof(double) * c->ngrid, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    return INCA_OK;
  }
  const int64_t launches0 = c->launches;
  MixedPlan P;
  int st = mixed_plan(c, eps, P);
  if (st) return st;
  if (!P.fused || P.drop_frac <= 0.0) {
    *plain = true;
    return INCA_OK;
  }
  P.f64 = true;
  P.cheap = 0;
  Events ev;
  for (auto& e : ev.e) INCA_CUDA(c, cudaEventCreate(&e));
  bool retry = false;
  if ((st = mixed_launch(c, P, true, &ev))) return st;
  if ((st = mixed_finish(c, P, &ev, &retry))) return st;
  if (retry) {
    if ((st = mixed_launch(c, P, false, &ev))) return st;
    if ((st = mixed_finish(c, P, &ev, &retry))) return st;
  }
  c->pairs_fp64 = c->pairs_fp32;  // the pairs evaluated (in FP64 here)
  c->pairs_fp32 = 0;
  c->corrected_points = 0;
  c->t_launches = static_cast<int>(c->launches - launches0);
  return INCA_OK;
}

// The same evaluation replayed from a CUDA graph: the first call for a given grid, set of
// records, precision and tolerance plans, runs once eagerly and captures the launch sequence;
// later calls launch the graph (all host decisions made at planning; the one that depends on
// the data -- repeating without dropping -- is taken after the replay, eagerly).
// Schedule tuning by coordinate descent over (items per CTA, sample stride, estimate safety,
// drop fraction): every candidate is a complete mixed evaluation on the current grid and
// records, timed with CUDA events (median of `reps` after one untimed run); a candidate replaces
// the best only when it is at least 1% faster, so timing noise does not move the choice. The
// fastest stays in the context. All candidates meet the tolerance, so the choice changes only
// the time. On an error the context's previous schedule is restored.
int autotune_mixed(inca_ctx* c, double eps, int reps, int* ipc_out, int* stride_out, double* safety_out,
                   double* drop_out, int* ctas_out, int* slack_out, int* ppt_out, double* best_ms,
                   double* default_ms) {
  struct Sched {
    int ipc, stride;
    double safety, drop;
    int ctas, slack, ppt;
  };
  const Sched saved{c->tune_items_per_cta, c->tune_sample_stride, c->tune_safety, c->tune_drop, c->tune_ctas,
                    c->tune_cheap_slack, c->tune_ppt};
  auto apply = [&](const Sched& s) {
    c->tune_items_per_cta = s.ipc;
    c->tune_sample_stride = s.stride;
    c->tune_safety = s.safety;
    c->tune_drop = s.drop;
    c->tune_ctas = s.ctas;
    c->tune_cheap_slack = s.slack;
    c->tune_ppt = s.ppt;
  };
  auto timed = [&](const Sched& s, double* ms) -> int {
    apply(s);
    std::vector<double> t;
    for (int r = 0; r < reps + 1; ++r) {
      const int st = eval_mixed(c, eps);
      if (st) {
        apply(saved);
        return st;
      }
      if (r) t.push_back(c->t_total_ms);
    }
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return INCA_OK;
  };
  Sched cur{kItemsPerCta, sample_stride_for(c->ngrid), kEstSafety, kDropFrac, INCA_PASS_CTAS_PER_SM, kCheapSlack,
            default_ppt(c)};
  double best = 0.0;
  int st = timed(cur, &best);
  if (st) return st;
  *default_ms = best;
  const int ipcs[] = {4, 8, 12, 24, 48};
  const int strides[] = {8, 16, 32, 64};
  const double safeties[] = {0.3, 0.5, 0.7, 1.0, 1.25};
  const double drops[] = {0.02, 0.05, 0.1, 0.2, 0.3};
  // the kernel's shape: (points per lane, resident CTAs per SM), the pairs valid_pass_shape admits
  const int shapes[][2] = {{4, 16}, {4, 12}, {4, 20}, {3, 16}, {3, 20}, {5, 12}, {5, 16}};
  const int slacks[] = {0, 2, 4, 6, 8};
  auto consider = [&](Sched s) -> int {
    double ms;
    const int e = timed(s, &ms);
    if (e) return e;
    if (ms < 0.99 * best) {
      best = ms;
      cur = s;
    }
    return INCA_OK;
  };
  for (int pass = 0; pass < 2; ++pass) {
    for (const auto& v : shapes)
      if ((v[0] != cur.ppt || v[1] != cur.ctas) &&
          (st = consider({cur.ipc, cur.stride, cur.safety, cur.drop, v[1], cur.slack, v[0]})))
        return st;
    for (int v : ipcs)
      if (v != cur.ipc && (st = consider({v, cur.stride, cur.safety, cur.drop, cur.ctas, cur.slack, cur.ppt})))
        return st;
    for (int v : strides)
      if (v != cur.stride && (st = consider({cur.ipc, v, cur.safety, cur.drop, cur.ctas, cur.slack, cur.ppt})))
        return st;
    for (double v : safeties)
      if (v != cur.safety && (st = consider({cur.ipc, cur.stride, v, cur.drop, cur.ctas, cur.slack, cur.ppt})))
        return st;
    for (double v : drops)
      if (v != cur.drop && (st = consider({cur.ipc, cur.stride, cur.safety, v, cur.ctas, cur.slack, cur.ppt})))
        return st;
    for (int v : slacks)
      if (v != cur.slack && (st = consider({cur.ipc, cur.stride, cur.safety, cur.drop, cur.ctas, v, cur.ppt})))
        return st;
  }
  // the estimate safety, the drop share and the cheap slack all spend the same error budget, so
  // one at a time they stop at different optima from run to run: a joint sweep over each one's
  // neighbours in its list (3 x 3 x 3 around the result) settles them together
  auto near = [](const auto& list, auto v) {
    const int n = static_cast<int>(sizeof(list) / sizeof(list[0]));
    int i = 0;
    while (i < n - 1 && list[i] != v) ++i;
    return std::array<int, 2>{std::max(0, i - 1), std::min(n - 1, i + 1)};
  };
  const Sched base = cur;
  const auto rs = near(safeties, base.safety), rd = near(drops, base.drop), rk = near(slacks, base.slack);
  for (int a = rs[0]; a <= rs[1]; ++a)
    for (int b = rd[0]; b <= rd[1]; ++b)
      for (int k = rk[0]; k <= rk[1]; ++k) {
        const Sched s{base.ipc, base.stride, safeties[a], drops[b], base.ctas, slacks[k], base.ppt};
        if (s.safety == base.safety && s.drop == base.drop && s.slack == base.slack) continue;
        if ((st = consider(s))) return st;
      }
  apply(cur);
  *ipc_out = cur.ipc;
  *stride_out = cur.stride;
  *safety_out = cur.safety;
  *drop_out = cur.drop;
  *ctas_out = cur.ctas;
  *slack_out = cur.slack;
  *ppt_out = cur.ppt;
  *best_ms = best;
  return INCA_OK;
}

// Everything a captured launch sequence holds by value: the plan's sizes, knobs and buffer
// addresses, and the addresses of the records, chunks, classes and sorted grid it reads. Two
// evaluations with the same signature run the same graph (the data in those buffers is read when
// the graph runs), so a graph stays valid across inca_prepare calls that give tables of the same
// shape, and a new schedule, tolerance or knob forces a new capture.
static std::vector<double> plan_signature(const inca_ctx* c, const MixedPlan& P) {
  auto a = [](const void* p) { return static_cast<double>(reinterpret_cast<uintptr_t>(p)); };
  std::vector<double> s = {double(P.fused), double(P.mode), double(P.nseg), double(P.emode), double(P.nmol),
                           double(P.cheap), double(P.wait_test), double(P.ctas), double(P.ppt),
                           a(P.seg_of), double(P.ngrid), double(P.nwt), double(P.ngroups), double(P.nitems),
                           double(P.npart), double(P.ndrop), double(P.ns), double(P.nitems_s), double(P.npart_s),
                           double(P.nctas), double(P.nctas_s), double(P.gblk), double(P.tblk),
                           double(P.stage_floats), double(P.dsmem), P.eps, P.tau_scale, P.safety, P.drop_frac,
                           P.nq, a(P.p1), a(P.q1), a(P.mwdev), a(P.mws), a(P.tab), a(c->d_scratch.p),
                           a(c->d_scratch_s.p), a(c->d_ivec.p), a(c->d_chunks.p), a(c->d_classes.p),
                           a(c->d_rec32.p), a(c->d_phi.p), a(c->d_plo.p), a(c->d_tiles.p), a(c->d_wtbox.p),
                           a(c->d_perm.p), a(c->d_phi_s.p), a(c->d_plo_s.p), a(c->d_tiles_s.p),
                           a(c->d_wtbox_s.p), a(c->d_perm_s.p), a(c->d_w.p)};
  return s;
}

int eval_mixed_graph(inca_ctx* c, double eps) {
  if (cube_separable(c)) return eval_cube_separable(c, eps);  // a few launches: run directly
  if (c->chunks.empty()) return eval_mixed(c, eps);
  bool fresh = false;
  MixedPlan P;
  int st = 0;
  if (c->graph_exec && c->graph_grid == c->grid_version) {
    if ((st = mixed_plan(c, eps, P))) return st;
    fresh = plan_signature(c, P) == c->graph_sig;
  }
  if (!fresh) {
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
    st = eval_mixed(c, eps);  // sizes every buffer and fills every cache first
    if (st) return st;
    if ((st = mixed_plan(c, eps, P))) return st;
    cudaGraph_t g = nullptr;
    INCA_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = c->launches;
    const int sl = mixed_launch(c, P, P.fused && P.drop_frac > 0.0, nullptr);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    c->graph_launches = c->launches - l0;
    if (sl) {
      if (g) cudaGraphDestroy(g);
      return sl;
    }
    if (e) return cuda_error(c, e, "graph capture");
    e = cudaGraphInstantiate(&c->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e) return cuda_error(c, e, "graph instantiate");
    c->graph_grid = c->grid_version;
    c->graph_sig = plan_signature(c, P);
    c->graph_fused = P.fused;
    c->graph_drop = P.fused && P.drop_frac > 0.0;
    return INCA_OK;  // this call's result came from the eager run
  }
  // the plan of this call (same signature) has uploaded its tables; the graph runs the passes
  INCA_CUDA(c, cudaGraphLaunch(c->graph_exec, c->stream));
  c->launches += c->graph_launches;
  bool retry = false;
  if ((st = mixed_finish(c, P, nullptr, &retry))) return st;
  if (retry && c->graph_drop) {
    if ((st = mixed_launch(c, P, false, nullptr))) return st;
    if ((st = mixed_finish(c, P, nullptr, &retry))) return st;
  }
  c->t_launches = static_cast<int>(c->graph_launches);
  return INCA_OK;
}

}  // namespace inca
