// K2 (mixed): FP32 evaluation with exact accumulation, plus a double-float correction of the
// terms whose FP32 error could exceed the requested tolerance. Everything runs on the FP32
// pipe (GB300's FP64 rate is ~1/64 of it); accumulation per point is exact (TwoSum in FP32
// within a chunk of <= 32 quartets, then FP64 across chunks).
//
// Why a correction. A term evaluated in FP32 carries ~2^-24 relative rounding; on a grid those
// errors average only over the few terms that dominate each output, and symmetry-equivalent
// quartets at symmetry-equivalent points round identically, so pure FP32 stalls near 1e-8
// relative on the CH4 radial integral. The large terms are therefore re-evaluated in
// double-float arithmetic (~2^-44) and the difference is added.
//
// Points are evaluated in Morton order (a sorted copy of the grid), so the 128 points a warp
// owns (32 lanes x 4) form a compact tile with a tight bounding box.
//
// Pass 1 (k_pass1): every (quartet, point) term in FP32 (compensated: hi/lo splits of the
//   scale, the shift and the point), accumulated exactly; also sum |t| per point. Pairs whose
//   bound is below 2^-120 (under FP32's normal range) are skipped.
// Thresholds: for an output O = sum_g w_g I_g (radial integral: TFVC weights; I(s): angular
//   weights of the shell; cube: max-norm; explicit points: each point) with tolerance eps,
//   FP32 errors behave as independent kappa*u*|t| (u = 2^-24, kappa = 8), so keeping every
//   uncorrected term below tau_g = (eps |O| / (3 kappa u))^2 / (w_g M_O) bounds the 3-sigma
//   error by eps |O| / 3 (M_O = sum_g w_g sum_q |t_qg|). |O| is replaced by the lower bound
//   |O~| - 3 kappa u M_O of the estimate.
// Pass 2 (k_pass2): per (quartet, warp tile) the log2 upper bound
//   lb = log2(|A'| prod_d sum_k |Cn_dk|) + sum_d [L_d log2 max(1, M_d) - m_d^2]
//   (m_d/M_d: min/max |u_d| over the tile's box, u = c_u r', e^-r'^2 = 2^-u^2) selects the
//   pairs with lb > log2 tau_T; for those every point gets t_df - t_32, with t_32 recomputed by
//   the same instruction sequence as in pass 1.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cub/cub.cuh>

#include "inca_internal.h"

namespace inca {

int choose_splits(int64_t tiles, int64_t nchunks, int num_sms, int ctas_per_sm);

namespace {

constexpr int kWarps = 4;
constexpr int kThreadsM = 32 * kWarps;
constexpr int kPPT = 4;                        // points per lane
constexpr int kWarpTile = 32 * kPPT;           // 128 points
constexpr int kCtaTile = kWarps * kWarpTile;   // 512 points
constexpr int kMaxStride32 = (12 + 2 * 3 * kMaxCoef + 3) & ~3;
constexpr int kChunkMax = 32;
constexpr double kKappaU = 8.0 * 5.9604644775390625e-08;  // kappa * 2^-24
constexpr float kSkipLog2 = -120.0f;                      // pass-1 skip: bound below 2^-120
constexpr int kExpTab = 256;                              // 2^(j/256), j = -128..128

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// ---------------------------------------------------------------- FP32 term (both passes)
template <int L>
__device__ __forceinline__ void horner_pts(const float* __restrict__ C, const float (&u)[kPPT], float (&v)[kPPT]) {
#pragma unroll
  for (int p = 0; p < kPPT; ++p) v[p] = C[0];
#pragma unroll
  for (int m = 1; m <= L; ++m) {
    const float c = C[m];
#pragma unroll
    for (int p = 0; p < kPPT; ++p) v[p] = __fmaf_rn(v[p], u[p], c);
  }
}

__device__ __forceinline__ void poly_pts(int L, const float* __restrict__ C, const float (&u)[kPPT], float (&v)[kPPT]) {
  switch (L) {
    case 0: horner_pts<0>(C, u, v); break;
    case 1: horner_pts<1>(C, u, v); break;
    case 2: horner_pts<2>(C, u, v); break;
    case 3: horner_pts<3>(C, u, v); break;
    case 4: horner_pts<4>(C, u, v); break;
    case 5: horner_pts<5>(C, u, v); break;
    case 6: horner_pts<6>(C, u, v); break;
    case 7: horner_pts<7>(C, u, v); break;
    case 8: horner_pts<8>(C, u, v); break;
    case 9: horner_pts<9>(C, u, v); break;
    case 10: horner_pts<10>(C, u, v); break;
    case 11: horner_pts<11>(C, u, v); break;
    case 12: horner_pts<12>(C, u, v); break;
    case 13: horner_pts<13>(C, u, v); break;
    case 14: horner_pts<14>(C, u, v); break;
    case 15: horner_pts<15>(C, u, v); break;
    default: horner_pts<16>(C, u, v); break;
  }
}

// The FP32 term of quartet record R at kPPT points. Explicit round-to-nearest intrinsics only,
// so both passes produce the same bits.
__device__ __forceinline__ void terms32(const float* __restrict__ R, const int L[3], const float (&rh)[3][kPPT],
                                        const float (&rl)[3][kPPT], float (&t)[kPPT]) {
  const float s_hi = R[0], s_lo = R[1], A_hi = R[8], A_lo = R[9];
  float u[3][kPPT];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float b_hi = R[2 + d], b_lo = R[5 + d];
#pragma unroll
    for (int p = 0; p < kPPT; ++p) {
      float t1 = __fmaf_rn(s_lo, rh[d][p], b_lo);
      t1 = __fmaf_rn(s_hi, rl[d][p], t1);
      u[d][p] = __fmaf_rn(s_hi, rh[d][p], __fadd_rn(b_hi, t1));
    }
  }
  float E[kPPT];
#pragma unroll
  for (int p = 0; p < kPPT; ++p) {
    float y = __fmul_rn(-u[0][p], u[0][p]);
    y = __fmaf_rn(-u[1][p], u[1][p], y);
    y = __fmaf_rn(-u[2][p], u[2][p], y);
    E[p] = ex2_approx(y);
  }
  const float* Cx = R + 12;
  const float* Cy = Cx + L[0] + 1;
  const float* Cz = Cy + L[1] + 1;
  float vx[kPPT], vy[kPPT], vz[kPPT];
  poly_pts(L[0], Cx, u[0], vx);
  poly_pts(L[1], Cy, u[1], vy);
  poly_pts(L[2], Cz, u[2], vz);
#pragma unroll
  for (int p = 0; p < kPPT; ++p) {
    const float P = __fmul_rn(__fmul_rn(__fmul_rn(E[p], vx[p]), vy[p]), vz[p]);
    t[p] = __fmaf_rn(P, A_hi, __fmul_rn(P, A_lo));
  }
}

// ---------------------------------------------------------------- double-float arithmetic
struct f2 {
  float hi, lo;
};
__device__ __forceinline__ f2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ f2 fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ f2 df_add(f2 x, f2 y) {
  const f2 s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ f2 df_mul(f2 x, f2 y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ f2 df_sqr(f2 x) {
  const float p = __fmul_rn(x.hi, x.hi);
  float e = __fmaf_rn(x.hi, x.hi, -p);
  e = __fmaf_rn(__fadd_rn(x.hi, x.hi), x.lo, e);
  return {p, e};
}

// 2^y in double-float for y <= 0: y = n + j/256 + g, |g| <= 1/512;
// 2^g = e^x, x = g ln2 (double-float), e^x = 1 + x + x^2/2 + x^3/6 + x^4/24 (tail in FP32).
__device__ __forceinline__ f2 df_exp2(f2 y, const float2* __restrict__ tab) {
  if (y.hi < -125.0f) return {0.0f, 0.0f};
  const float n = rintf(y.hi);
  const float f = __fsub_rn(y.hi, n);           // exact
  const float j = rintf(__fmul_rn(f, 256.0f));
  const float g = __fsub_rn(f, __fmul_rn(j, 0.00390625f));  // exact
  const float kLn2Hi = 0.693147182464599609375f, kLn2Lo = -1.904654323148236e-09f;
  const float xh = __fmul_rn(g, kLn2Hi);
  float xl = __fmaf_rn(g, kLn2Hi, -xh);
  xl = __fmaf_rn(g, kLn2Lo, xl);
  xl = __fmaf_rn(y.lo, kLn2Hi, xl);
  const f2 x = fast_two_sum(xh, xl);
  float q = __fmaf_rn(x.hi, 0.041666666666666664f, 0.16666666666666666f);
  q = __fmaf_rn(x.hi, q, 0.5f);
  q = __fmul_rn(__fmul_rn(x.hi, x.hi), q);
  q = __fmaf_rn(x.hi, x.lo, q);
  const f2 s = two_sum(1.0f, x.hi);
  const f2 ex = fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, q)));
  const float2 T = tab[static_cast<int>(j) + kExpTab / 2];
  const f2 r = df_mul({T.x, T.y}, ex);
  const float sc = __int_as_float((static_cast<int>(n) + 127) << 23);  // 2^n, n >= -125
  return {__fmul_rn(r.hi, sc), __fmul_rn(r.lo, sc)};
}

// The double-float term of record R at one point (r_hi + r_lo per dimension).
__device__ f2 term_df(const float* __restrict__ R, const int L[3], int nc, const float rh[3], const float rl[3],
                      const float2* __restrict__ tab) {
  const float s_hi = R[0], s_lo = R[1];
  f2 u[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float p = __fmul_rn(s_hi, rh[d]);
    float e = __fmaf_rn(s_hi, rh[d], -p);
    const f2 t = two_sum(p, R[2 + d]);
    e = __fadd_rn(e, t.lo);
    e = __fmaf_rn(s_hi, rl[d], e);
    e = __fmaf_rn(s_lo, rh[d], e);
    e = __fadd_rn(e, R[5 + d]);
    u[d] = two_sum(t.hi, e);
  }
  f2 y = df_add(df_add(df_sqr(u[0]), df_sqr(u[1])), df_sqr(u[2]));
  y.hi = -y.hi;
  y.lo = -y.lo;
  f2 t = df_exp2(y, tab);
  const float* C = R + 12;
  int o = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    f2 v = {C[o], C[o + nc]};
    for (int m = 1; m <= L[d]; ++m) v = df_add(df_mul(v, u[d]), f2{C[o + m], C[o + m + nc]});
    o += L[d] + 1;
    t = df_mul(t, v);
  }
  return df_mul(t, f2{R[8], R[9]});
}

// log2 upper bound of |term| over a tile's box (see the file comment).
__device__ __forceinline__ float log2_bound(const float* __restrict__ R, const int L[3], const float box[6]) {
  float lb = R[10] + 0.02f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float s = R[0], b = R[2 + d];
    const float a0 = fmaf(s, box[d], b), a1 = fmaf(s, box[3 + d], b);
    float m = (a0 <= 0.0f && a1 >= 0.0f) ? 0.0f : fminf(fabsf(a0), fabsf(a1));
    float M = fmaxf(fabsf(a0), fabsf(a1));
    m = fmaxf(0.0f, m * (1.0f - 1e-5f) - 1e-5f);
    M = M * (1.0f + 1e-5f) + 1e-5f;
    lb += static_cast<float>(L[d]) * __log2f(fmaxf(M, 1.0f)) - m * m;
  }
  return lb;
}

__device__ __forceinline__ void load_points(const float4* __restrict__ phi, const float4* __restrict__ plo,
                                            int64_t base, int lane, int64_t ngrid, float (&rh)[3][kPPT],
                                            float (&rl)[3][kPPT]) {
#pragma unroll
  for (int p = 0; p < kPPT; ++p) {
    const int64_t i = base + lane + 32 * p;
    float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
    if (i < ngrid) {
      h = phi[i];
      l = plo[i];
    }
    rh[0][p] = h.x; rh[1][p] = h.y; rh[2][p] = h.z;
    rl[0][p] = l.x; rl[1][p] = l.y; rl[2][p] = l.z;
  }
}

__device__ __forceinline__ void stage_chunk(float* st, const float* __restrict__ rec32, const ClassSeg& sg,
                                            const WorkChunk& w) {
  const float4* src = reinterpret_cast<const float4*>(rec32 + sg.off32 + (w.rec - sg.first) * sg.stride32);
  const int nvec = w.count * sg.stride32 / 4;
  for (int i = threadIdx.x; i < nvec; i += kThreadsM) reinterpret_cast<float4*>(st)[i] = src[i];
}

// ---------------------------------------------------------------- pass 1
__global__ void __launch_bounds__(kThreadsM)
k_pass1(const WorkChunk* __restrict__ chunks, int nchunks, const ClassSeg* __restrict__ segs,
        const float* __restrict__ rec32, const float4* __restrict__ phi, const float4* __restrict__ plo,
        const float* __restrict__ wtbox, int64_t ngrid, int nsplit, double* __restrict__ part,
        double* __restrict__ part_abs, unsigned long long* __restrict__ stats) {
  __shared__ __align__(16) float st[kChunkMax * kMaxStride32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t wtile = static_cast<int64_t>(blockIdx.x) * kWarps + warp;
  const int64_t base = wtile * kWarpTile;
  float rh[3][kPPT], rl[3][kPPT];
  load_points(phi, plo, base, lane, ngrid, rh, rl);
  float box[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) box[k] = wtbox[wtile * 8 + k];
  double acc[kPPT], acc_abs[kPPT];
#pragma unroll
  for (int p = 0; p < kPPT; ++p) acc[p] = acc_abs[p] = 0.0;
  unsigned long long nskip = 0;
  for (int ch = blockIdx.y; ch < nchunks; ch += nsplit) {
    const WorkChunk w = chunks[ch];
    const ClassSeg sg = segs[w.cls];
    __syncthreads();
    stage_chunk(st, rec32, sg, w);
    __syncthreads();
    const int L[3] = {sg.L[0], sg.L[1], sg.L[2]};
    const float lb = lane < w.count ? log2_bound(st + lane * sg.stride32, L, box) : -HUGE_VALF;
    uint32_t m = __ballot_sync(0xffffffffu, lane < w.count && lb > kSkipLog2);
    if (lane == 0) nskip += w.count - __popc(m);
    float sh[kPPT], sl[kPPT], sa[kPPT];
#pragma unroll
    for (int p = 0; p < kPPT; ++p) sh[p] = sl[p] = sa[p] = 0.0f;
    while (m) {
      const int q = __ffs(m) - 1;
      m &= m - 1;
      float t[kPPT];
      terms32(st + q * sg.stride32, L, rh, rl, t);
#pragma unroll
      for (int p = 0; p < kPPT; ++p) {
        const f2 s = two_sum(sh[p], t[p]);
        sh[p] = s.hi;
        sl[p] = __fadd_rn(sl[p], s.lo);
        sa[p] = __fadd_rn(sa[p], fabsf(t[p]));
      }
    }
#pragma unroll
    for (int p = 0; p < kPPT; ++p) {
      acc[p] += static_cast<double>(sh[p]) + static_cast<double>(sl[p]);
      acc_abs[p] += static_cast<double>(sa[p]);
    }
  }
#pragma unroll
  for (int p = 0; p < kPPT; ++p) {
    const int64_t i = base + lane + 32 * p;
    if (i < ngrid) {
      part[static_cast<int64_t>(blockIdx.y) * ngrid + i] = acc[p];
      part_abs[static_cast<int64_t>(blockIdx.y) * ngrid + i] = acc_abs[p];
    }
  }
  if (lane == 0) atomicAdd(&stats[2], nskip);
}

// ---------------------------------------------------------------- pass 2 (corrections)
__global__ void __launch_bounds__(kThreadsM)
k_pass2(const WorkChunk* __restrict__ chunks, int nchunks, const ClassSeg* __restrict__ segs,
        const float* __restrict__ rec32, const float4* __restrict__ phi, const float4* __restrict__ plo,
        const float* __restrict__ wtbox, const float* __restrict__ wt_lt, const float2* __restrict__ exp_tab,
        int64_t ngrid, int nsplit, double* __restrict__ part, unsigned long long* __restrict__ stats) {
  __shared__ __align__(16) float st[kChunkMax * kMaxStride32];
  __shared__ float2 tab[kExpTab + 1];
  for (int i = threadIdx.x; i <= kExpTab; i += kThreadsM) tab[i] = exp_tab[i];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t wtile = static_cast<int64_t>(blockIdx.x) * kWarps + warp;
  const int64_t base = wtile * kWarpTile;
  float rh[3][kPPT], rl[3][kPPT];
  load_points(phi, plo, base, lane, ngrid, rh, rl);
  float box[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) box[k] = wtbox[wtile * 8 + k];
  const float lt = wt_lt[wtile];
  double acc[kPPT];
#pragma unroll
  for (int p = 0; p < kPPT; ++p) acc[p] = 0.0;
  unsigned long long n32 = 0, ndf = 0;
  for (int ch = blockIdx.y; ch < nchunks; ch += nsplit) {
    const WorkChunk w = chunks[ch];
    const ClassSeg sg = segs[w.cls];
    __syncthreads();
    stage_chunk(st, rec32, sg, w);
    __syncthreads();
    const int L[3] = {sg.L[0], sg.L[1], sg.L[2]};
    const int nc = L[0] + L[1] + L[2] + 3;
    const float lb = lane < w.count ? log2_bound(st + lane * sg.stride32, L, box) : -HUGE_VALF;
    const uint32_t live = __ballot_sync(0xffffffffu, lane < w.count && lb > kSkipLog2);
    uint32_t m = __ballot_sync(0xffffffffu, lane < w.count && lb > lt);
    if (lane == 0) {
      ndf += __popc(m);
      n32 += __popc(live & ~m);
    }
    if (!m) continue;
    f2 corr[kPPT];
#pragma unroll
    for (int p = 0; p < kPPT; ++p) corr[p] = {0.0f, 0.0f};
    while (m) {
      const int q = __ffs(m) - 1;
      m &= m - 1;
      const float* R = st + q * sg.stride32;
      float t32[kPPT];
      terms32(R, L, rh, rl, t32);
      const bool was_live = (live >> q) & 1u;
#pragma unroll
      for (int p = 0; p < kPPT; ++p) {
        const float ph[3] = {rh[0][p], rh[1][p], rh[2][p]};
        const float pl[3] = {rl[0][p], rl[1][p], rl[2][p]};
        f2 tdf = term_df(R, L, nc, ph, pl, tab);
        if (was_live) tdf = df_add(tdf, f2{-t32[p], 0.0f});
        corr[p] = df_add(corr[p], tdf);
      }
    }
#pragma unroll
    for (int p = 0; p < kPPT; ++p) acc[p] += static_cast<double>(corr[p].hi) + static_cast<double>(corr[p].lo);
  }
#pragma unroll
  for (int p = 0; p < kPPT; ++p) {
    const int64_t i = base + lane + 32 * p;
    if (i < ngrid) part[static_cast<int64_t>(blockIdx.y) * ngrid + i] = acc[p];
  }
  if (lane == 0) {
    atomicAdd(&stats[0], n32);
    atomicAdd(&stats[1], ndf);
  }
}

// ---------------------------------------------------------------- grid preparation
__global__ void k_morton(int64_t n, const double* __restrict__ px, const double* __restrict__ py,
                         const double* __restrict__ pz, double lo0, double lo1, double lo2, double inv,
                         uint64_t* key, int64_t* idx) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= n) return;
  const double c[3] = {(px[g] - lo0) * inv, (py[g] - lo1) * inv, (pz[g] - lo2) * inv};
  uint64_t k = 0;
  uint32_t q[3];
  for (int d = 0; d < 3; ++d) q[d] = static_cast<uint32_t>(fmin(fmax(c[d], 0.0), 2097151.0));
  for (int b = 20; b >= 0; --b)
    for (int d = 0; d < 3; ++d) k = (k << 1) | ((q[d] >> b) & 1u);
  key[g] = k;
  idx[g] = g;
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
    l[d] = static_cast<float>(x[d] - static_cast<double>(h[d]));
  }
  phi[i] = make_float4(h[0], h[1], h[2], 0.0f);
  plo[i] = make_float4(l[0], l[1], l[2], 0.0f);
}

// Bounding box of each 128-point warp tile (FP32, rounded outwards).
__global__ void k_warp_boxes(int64_t n, int64_t nwt, const float4* __restrict__ phi, const float4* __restrict__ plo,
                             float* box) {
  const int64_t wt = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + (threadIdx.x >> 5);
  if (wt >= nwt) return;
  const int lane = threadIdx.x & 31;
  float lo[3] = {HUGE_VALF, HUGE_VALF, HUGE_VALF}, hi[3] = {-HUGE_VALF, -HUGE_VALF, -HUGE_VALF};
  for (int p = 0; p < kPPT; ++p) {
    const int64_t i = wt * kWarpTile + lane + 32 * p;
    if (i >= n) break;
    const float4 h = phi[i], l = plo[i];
    const float x[3] = {h.x + l.x, h.y + l.y, h.z + l.z};
    for (int d = 0; d < 3; ++d) {
      lo[d] = fminf(lo[d], x[d]);
      hi[d] = fmaxf(hi[d], x[d]);
    }
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int d = 0; d < 3; ++d) {
      lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
  if (lane == 0)
    for (int d = 0; d < 3; ++d) {
      box[wt * 8 + d] = lo[d] - (fabsf(lo[d]) * 1e-6f + 1e-6f);
      box[wt * 8 + 3 + d] = hi[d] + (fabsf(hi[d]) * 1e-6f + 1e-6f);
    }
}

// Per-point thresholds (sorted order) reduced to per-warp-tile log2 minima.
// mode 0: tau = T_o / w_g; mode 1 (max-norm): tau = T_o / M_g; mode 2 (per point).
__global__ void k_warp_thresholds(int64_t n, int64_t nwt, int mode, const int64_t* __restrict__ perm,
                                  const int* __restrict__ seg_of, const double* __restrict__ segT,
                                  const double* __restrict__ w, const double* __restrict__ I,
                                  const double* __restrict__ M, double eps, float* lt) {
  const int64_t wt = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + (threadIdx.x >> 5);
  if (wt >= nwt) return;
  const int lane = threadIdx.x & 31;
  double tmin = HUGE_VAL;
  for (int p = 0; p < kPPT; ++p) {
    const int64_t i = wt * kWarpTile + lane + 32 * p;
    if (i >= n) break;
    const int64_t g = perm[i];
    double tau;
    if (mode == 0) {
      tau = w[g] > 0.0 ? segT[seg_of ? seg_of[g] : 0] / w[g] : HUGE_VAL;
    } else if (mode == 1) {
      tau = M[i] > 0.0 ? segT[0] / M[i] : HUGE_VAL;
    } else {
      const double lo = fmax(fabs(I[i]) - 3.0 * kKappaU * M[i], 0.0);
      const double x = eps * lo / (3.0 * kKappaU);
      tau = M[i] > 0.0 ? x * x / M[i] : HUGE_VAL;
    }
    tmin = fmin(tmin, tau);
  }
  for (int o = 16; o > 0; o >>= 1) tmin = fmin(tmin, __shfl_xor_sync(0xffffffffu, tmin, o));
  if (lane == 0) lt[wt] = tmin >= HUGE_VAL ? HUGE_VALF : (tmin > 0.0 ? static_cast<float>(log2(tmin)) : -HUGE_VALF);
}

// Sum the split partials of the passes (sorted order) in a fixed order.
__global__ void k_sum_splits(int64_t n, int nsplit, const double* __restrict__ a, const double* __restrict__ b,
                             double* out) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int k = 0; k < nsplit; ++k) s += a[static_cast<int64_t>(k) * n + i];
  if (b)
    for (int k = 0; k < nsplit; ++k) s += b[static_cast<int64_t>(k) * n + i];
  out[i] = s;
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

__global__ void k_absmax(int64_t n, const double* __restrict__ I, unsigned long long* out) {
  double m = 0.0;
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < n;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x)
    m = fmax(m, fabs(I[g]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, static_cast<unsigned long long>(__double_as_longlong(m)));
}

inline unsigned nblk(int64_t n, int bs = 256) { return static_cast<unsigned>((n + bs - 1) / bs); }

// Morton-sorted FP32 copy of the grid, the permutation and the warp-tile boxes.
int prepare_sorted_grid(inca_ctx* c) {
  if (c->mix_version == c->grid_version) return INCA_OK;
  const int64_t n = c->ngrid;
  const int64_t ctas = (n + kCtaTile - 1) / kCtaTile;
  const int64_t nwt = ctas * kWarps;
  if (c->d_phi.reserve(n) || c->d_plo.reserve(n) || c->d_perm.reserve(n) || c->d_wtbox.reserve(8 * nwt))
    return set_error(c, INCA_E_NOMEM, "sorted grid");
  // bounding box of the grid (one host copy of the coordinates; cheap next to evaluation)
  std::vector<double> hx(n), hy(n), hz(n);
  INCA_CUDA(c, cudaMemcpy(hx.data(), c->d_px.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  INCA_CUDA(c, cudaMemcpy(hy.data(), c->d_py.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  INCA_CUDA(c, cudaMemcpy(hz.data(), c->d_pz.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
  for (int64_t g = 0; g < n; ++g) {
    lo[0] = std::min(lo[0], hx[g]); hi[0] = std::max(hi[0], hx[g]);
    lo[1] = std::min(lo[1], hy[g]); hi[1] = std::max(hi[1], hy[g]);
    lo[2] = std::min(lo[2], hz[g]); hi[2] = std::max(hi[2], hz[g]);
  }
  const double ext = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), std::max(hi[2] - lo[2], 1e-12));
  const double inv = 2097151.0 / ext;
  DevBuf<uint64_t> k1, k2;
  DevBuf<int64_t> i1;
  DevBuf<unsigned char> tmp;
  auto rel = [&]() { k1.release(); k2.release(); i1.release(); tmp.release(); };
  if (k1.reserve(n) || k2.reserve(n) || i1.reserve(n)) {
    rel();
    return set_error(c, INCA_E_NOMEM, "morton sort");
  }
  INCA_LAUNCH(c, k_morton, nblk(n), 256, 0, n, c->d_px.p, c->d_py.p, c->d_pz.p, lo[0], lo[1], lo[2], inv, k1.p, i1.p);
  size_t tb = 0;
  cudaError_t e = cub::DeviceRadixSort::SortPairs(nullptr, tb, k1.p, k2.p, i1.p, c->d_perm.p, n, 0, 63, c->stream);
  if (!e) e = tmp.reserve(tb);
  if (!e) e = cub::DeviceRadixSort::SortPairs(tmp.p, tb, k1.p, k2.p, i1.p, c->d_perm.p, n, 0, 63, c->stream);
  if (!e) {
    INCA_LAUNCH(c, k_gather_points, nblk(n), 256, 0, n, c->d_perm.p, c->d_px.p, c->d_py.p, c->d_pz.p, c->d_phi.p,
                c->d_plo.p);
    e = cudaMemsetAsync(c->d_wtbox.p, 0, sizeof(float) * 8 * nwt, c->stream);
  }
  if (!e) {
    INCA_LAUNCH(c, k_warp_boxes, static_cast<unsigned>((nwt + 7) / 8), 256, 0, n, nwt, c->d_phi.p, c->d_plo.p,
                c->d_wtbox.p);
    e = cudaStreamSynchronize(c->stream);
  }
  rel();
  if (e) return cuda_error(c, e, "sorted grid");
  c->mix_version = c->grid_version;
  return INCA_OK;
}

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

}  // namespace

int eval_mixed(inca_ctx* c, double eps) {
  const int64_t ngrid = c->ngrid;
  const int nchunks = static_cast<int>(c->chunks.size());
  if (nchunks == 0) {
    INCA_CUDA(c, cudaMemsetAsync(c->d_ivec.p, 0, sizeof(double) * ngrid, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    return INCA_OK;
  }
  cudaEvent_t ev[6];
  for (auto& e : ev) INCA_CUDA(c, cudaEventCreate(&e));
  INCA_CUDA(c, cudaEventRecord(ev[0], c->stream));
  int st = prepare_sorted_grid(c);
  if (st) return st;
  const int64_t ctas = (ngrid + kCtaTile - 1) / kCtaTile;
  const int64_t nwt = ctas * kWarps;
  const int nsplit = choose_splits(ctas, nchunks, c->num_sms, 4);
  // scratch: pass-1 sums and |t| sums, pass-2 corrections (nsplit x n each), I~, M~ (sorted),
  // I~ (grid order), warp-tile thresholds, stats, exp table
  const size_t nd = 3 * static_cast<size_t>(nsplit) * ngrid + 3 * static_cast<size_t>(ngrid);
  const size_t need = sizeof(double) * nd + sizeof(float) * nwt + 64 + sizeof(float2) * (kExpTab + 1) + 256;
  if (c->d_scratch.reserve(need)) return set_error(c, INCA_E_NOMEM, "mixed scratch");
  double* p1 = reinterpret_cast<double*>(c->d_scratch.p);
  double* pabs = p1 + static_cast<size_t>(nsplit) * ngrid;
  double* p2 = pabs + static_cast<size_t>(nsplit) * ngrid;
  double* Is = p2 + static_cast<size_t>(nsplit) * ngrid;  // I~ in sorted order
  double* Ms = Is + ngrid;                                 // M~ in sorted order
  double* Io = Ms + ngrid;                                 // I~ in grid order (thresholds)
  float* wlt = reinterpret_cast<float*>(Io + ngrid);
  unsigned long long* stats =
      reinterpret_cast<unsigned long long*>((reinterpret_cast<uintptr_t>(wlt + nwt) + 15) & ~uintptr_t(15));
  float2* tab = reinterpret_cast<float2*>(stats + 4);
  const std::vector<float2> htab = exp2_table();
  INCA_CUDA(c, cudaMemcpyAsync(tab, htab.data(), sizeof(float2) * htab.size(), cudaMemcpyHostToDevice, c->stream));
  INCA_CUDA(c, cudaMemsetAsync(stats, 0, 4 * sizeof(unsigned long long), c->stream));
  INCA_CUDA(c, cudaEventRecord(ev[1], c->stream));
  dim3 grid(static_cast<unsigned>(ctas), static_cast<unsigned>(nsplit));
  INCA_LAUNCH(c, k_pass1, grid, kThreadsM, 0, c->d_chunks.p, nchunks, c->d_classes.p, c->d_rec32.p, c->d_phi.p,
              c->d_plo.p, c->d_wtbox.p, ngrid, nsplit, p1, pabs, stats);
  INCA_CUDA(c, cudaGetLastError());
  INCA_CUDA(c, cudaEventRecord(ev[2], c->stream));
  INCA_LAUNCH(c, k_sum_splits, nblk(ngrid), 256, 0, ngrid, nsplit, p1, nullptr, Is);
  INCA_LAUNCH(c, k_sum_splits, nblk(ngrid), 256, 0, ngrid, nsplit, pabs, nullptr, Ms);
  INCA_LAUNCH(c, k_scatter, nblk(ngrid), 256, 0, ngrid, c->d_perm.p, Is, Io);
  // per-output scales
  int mode = 2;
  std::vector<double> segT;
  const int* seg_of = nullptr;
  DevBuf<double> dT, dout, Mo;
  DevBuf<int64_t> doff;
  DevBuf<unsigned long long> dmax;
  auto rel = [&]() { dT.release(); dout.release(); doff.release(); dmax.release(); Mo.release(); };
  if (c->grid_kind == GRID_RADIAL || c->grid_kind == GRID_SCAN) {
    mode = 0;
    std::vector<int64_t> off;
    if (c->grid_kind == GRID_RADIAL) {
      off = {0, ngrid};
    } else {
      off.assign(c->nradi + 1, 0);
      for (int s = 0; s < c->nradi; ++s) off[s + 1] = off[s] + c->h_smn[s];
      seg_of = c->d_cmap.p;  // shell of each scan point
    }
    const int nseg = static_cast<int>(off.size()) - 1;
    if (doff.reserve(nseg + 1) || dout.reserve(3 * nseg) || Mo.reserve(ngrid)) {
      rel();
      return set_error(c, INCA_E_NOMEM, "thresholds");
    }
    INCA_LAUNCH(c, k_scatter, nblk(ngrid), 256, 0, ngrid, c->d_perm.p, Ms, Mo.p);
    INCA_CUDA(c, cudaMemcpyAsync(doff.p, off.data(), sizeof(int64_t) * (nseg + 1), cudaMemcpyHostToDevice, c->stream));
    INCA_LAUNCH(c, k_seg_sums, nseg, 256, 0, nseg, doff.p, c->d_w.p, Io, Mo.p, dout.p);
    std::vector<double> h(3 * nseg);
    INCA_CUDA(c, cudaMemcpyAsync(h.data(), dout.p, sizeof(double) * 3 * nseg, cudaMemcpyDeviceToHost, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    segT.resize(nseg);
    for (int s = 0; s < nseg; ++s) {
      const double O = h[3 * s], M = h[3 * s + 1];
      const double lo = std::max(std::fabs(O) - 3.0 * kKappaU * M, 0.0);
      const double x = eps * lo / (3.0 * kKappaU);
      segT[s] = M > 0.0 ? x * x / M : HUGE_VAL;
    }
  } else if (c->grid_kind == GRID_CUBE) {
    mode = 1;
    if (dmax.reserve(1)) {
      rel();
      return set_error(c, INCA_E_NOMEM, "thresholds");
    }
    INCA_CUDA(c, cudaMemsetAsync(dmax.p, 0, sizeof(unsigned long long), c->stream));
    const unsigned nb = static_cast<unsigned>(std::min<int64_t>(nblk(ngrid), 4096));
    INCA_LAUNCH(c, k_absmax, nb, 256, 0, ngrid, Is, dmax.p);
    unsigned long long hm = 0;
    INCA_CUDA(c, cudaMemcpyAsync(&hm, dmax.p, sizeof(hm), cudaMemcpyDeviceToHost, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    double Imax;
    std::memcpy(&Imax, &hm, sizeof(double));
    const double x = eps * Imax / (3.0 * kKappaU);
    segT = {x * x};
  } else {
    segT = {0.0};
  }
  if (dT.reserve(segT.size())) {
    rel();
    return set_error(c, INCA_E_NOMEM, "thresholds");
  }
  INCA_CUDA(c, cudaMemcpyAsync(dT.p, segT.data(), sizeof(double) * segT.size(), cudaMemcpyHostToDevice, c->stream));
  INCA_LAUNCH(c, k_warp_thresholds, static_cast<unsigned>((nwt + 7) / 8), 256, 0, ngrid, nwt, mode, c->d_perm.p,
              seg_of, dT.p, c->d_w.p, Is, Ms, eps, wlt);
  INCA_CUDA(c, cudaGetLastError());
  INCA_CUDA(c, cudaEventRecord(ev[3], c->stream));
  INCA_LAUNCH(c, k_pass2, grid, kThreadsM, 0, c->d_chunks.p, nchunks, c->d_classes.p, c->d_rec32.p, c->d_phi.p,
              c->d_plo.p, c->d_wtbox.p, wlt, tab, ngrid, nsplit, p2, stats);
  INCA_CUDA(c, cudaGetLastError());
  INCA_CUDA(c, cudaEventRecord(ev[4], c->stream));
  INCA_LAUNCH(c, k_sum_splits, nblk(ngrid), 256, 0, ngrid, nsplit, p1, p2, Is);
  INCA_LAUNCH(c, k_scatter, nblk(ngrid), 256, 0, ngrid, c->d_perm.p, Is, c->d_ivec.p);
  INCA_CUDA(c, cudaGetLastError());
  INCA_CUDA(c, cudaEventRecord(ev[5], c->stream));
  INCA_CUDA(c, cudaEventSynchronize(ev[5]));
  rel();
  float t12 = 0, t34 = 0, t05 = 0;
  cudaEventElapsedTime(&t12, ev[1], ev[2]);
  cudaEventElapsedTime(&t34, ev[3], ev[4]);
  cudaEventElapsedTime(&t05, ev[0], ev[5]);
  for (auto& e : ev) cudaEventDestroy(e);
  unsigned long long hs[3] = {0, 0, 0};
  INCA_CUDA(c, cudaMemcpy(hs, stats, sizeof(hs), cudaMemcpyDeviceToHost));
  c->t_total_ms = t05;
  c->t_kernel_ms = t12;  // the dominant kernel (pass 1)
  c->t_pass2_ms = t34;
  c->t_kernel_launches = 1;
  c->t_launches = 9;
  c->pairs_fp32 = static_cast<int64_t>(hs[0]);
  c->pairs_fp64 = static_cast<int64_t>(hs[1]);
  c->pairs_skip = static_cast<int64_t>(hs[2]);
  return INCA_OK;
}

}  // namespace inca
