// K2 (mixed): FP32 evaluation with FP64 accumulation and an FP64 precise tier.
//
// Why a precise tier. A term evaluated in FP32 carries ~2^-24 relative rounding; on a grid
// those errors average only over the few terms that dominate each output, and symmetry-
// equivalent quartets at symmetry-equivalent points round identically, so pure FP32 stalls
// near 1e-8 relative on the CH4 radial integral. Terms large enough to matter at the requested
// tolerance are therefore evaluated in FP64; the rest (the overwhelming majority) in FP32.
//
// Pass 1 (estimate): every term in FP32 -> I~(g) and M~(g) = sum_q |t_qg| per point.
// Thresholds: for an output O = sum_g w_g I_g (radial integral: TFVC weights; I(s): angular
//   weights of the shell; cube: max-norm; explicit points: each point) with tolerance eps,
//   FP32 errors behave as independent kappa*u*|t| (u = 2^-24, kappa = 8), so keeping every
//   FP32 term below tau_g = (eps |O| / (3 kappa u))^2 / (w_g M_O) bounds the 3-sigma error by
//   eps |O| / 3. Terms below sigma = eps |O| / (3 N W) (N survivors, W = sum w) are skipped:
//   their total cannot exceed eps |O| / 3. |O| is replaced by the lower bound
//   |O~| - 3 kappa u M_O of the estimate.
// Pass 2: per (quartet, point tile) the log2 upper bound
//   lb = log2(|A'| prod_d sum_k |Cn_dk|) + sum_d [L_d log2 max(1, M_d) - m_d^2]
//   (m_d/M_d: min/max |u_d| over the tile's bounding box, u = c_u r', e^-r'^2 = 2^-u^2)
//   selects skip (lb <= log2 sigma_T), FP32 (<= log2 tau_T) or FP64.
//
// FP32 term: u_d = s (r_d + d_d) from hi/lo splits of s, s d_d and r_d (4 FMA/add per
// dimension), y = -|u|^2 (3), E = ex2.approx(y) (1 MUFU), V_d by Horner on the normalised
// coefficients (L ops), E Vx Vy Vz (3), accumulate with A'_hi and A'_lo (2). The partial sum
// of a chunk (<= 32 quartets) is added into the FP64 accumulator of the point.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "inca_internal.h"

namespace inca {

__global__ void k_reduce_splits(const double* __restrict__ partial, int nsplit, int64_t ngrid,
                                double* __restrict__ out);
int choose_splits(int64_t tiles, int64_t nchunks, int num_sms, int ctas_per_sm);

namespace {

constexpr int kThreadsM = 128;
constexpr int kPPTM = 4;
constexpr int kTileM = kThreadsM * kPPTM;
constexpr int kMaxStride32 = (12 + 3 * kMaxCoef + 3) & ~3;
constexpr int kChunkMax = 32;
constexpr double kKappaU = 8.0 * 5.9604644775390625e-08;  // kappa * 2^-24

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <int L>
__device__ __forceinline__ void horner_pts(const float* __restrict__ C, const float (&u)[kPPTM],
                                           float (&v)[kPPTM]) {
#pragma unroll
  for (int p = 0; p < kPPTM; ++p) v[p] = C[0];
#pragma unroll
  for (int m = 1; m <= L; ++m) {
    const float c = C[m];
#pragma unroll
    for (int p = 0; p < kPPTM; ++p) v[p] = fmaf(v[p], u[p], c);
  }
}

// Polynomial of a class-uniform (warp-uniform) degree: one indirect branch per quartet.
__device__ __forceinline__ void poly_pts(int L, const float* __restrict__ C, const float (&u)[kPPTM],
                                         float (&v)[kPPTM]) {
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

// log2 upper bound of |term| over a tile's bounding box (see the file comment).
__device__ __forceinline__ float log2_bound(const float* __restrict__ R, const int L[3], const float box[6]) {
  float lb = R[10] + 0.02f;  // slack for the FP32 evaluation of the bound itself
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

template <bool kPass1>
__global__ void __launch_bounds__(kThreadsM)
k_mixed(const WorkChunk* __restrict__ chunks, int nchunks, const ClassSeg* __restrict__ segs,
        const float* __restrict__ rec32, const double* __restrict__ rec64, const double* __restrict__ px,
        const double* __restrict__ py, const double* __restrict__ pz, int64_t ngrid, int nsplit,
        const float* __restrict__ tile_box, const float* __restrict__ tile_lt,
        const float* __restrict__ tile_ls, double* __restrict__ partial, double* __restrict__ partial_abs,
        unsigned long long* __restrict__ stats) {
  __shared__ __align__(16) float st[kChunkMax * kMaxStride32];
  __shared__ uint32_t s_m32, s_m64;
  const int tid = threadIdx.x;
  const int tile = blockIdx.x;
  const int64_t base = static_cast<int64_t>(tile) * kTileM;
  float rh[3][kPPTM], rl[3][kPPTM];
  double acc[kPPTM], acc_abs[kPPTM];
#pragma unroll
  for (int p = 0; p < kPPTM; ++p) {
    const int64_t g = base + tid + p * kThreadsM;
    const bool ok = g < ngrid;
    const double x[3] = {ok ? px[g] : 0.0, ok ? py[g] : 0.0, ok ? pz[g] : 0.0};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      rh[d][p] = static_cast<float>(x[d]);
      rl[d][p] = static_cast<float>(x[d] - static_cast<double>(rh[d][p]));
    }
    acc[p] = 0.0;
    acc_abs[p] = 0.0;
  }
  float box[6] = {0, 0, 0, 0, 0, 0};
  float lt = 0.0f, ls = 0.0f;
  if (!kPass1) {
#pragma unroll
    for (int k = 0; k < 6; ++k) box[k] = tile_box[tile * 8 + k];
    lt = tile_lt[tile];
    ls = tile_ls[tile];
  }
  unsigned long long n32 = 0, n64 = 0, nskip = 0;
  for (int ch = blockIdx.y; ch < nchunks; ch += nsplit) {
    const WorkChunk w = chunks[ch];
    const ClassSeg sg = segs[w.cls];
    const int stride = sg.stride32;
    const float4* src = reinterpret_cast<const float4*>(rec32 + sg.off32 + (w.rec - sg.first) * stride);
    const int nvec = w.count * stride / 4;
    __syncthreads();
    for (int i = tid; i < nvec; i += kThreadsM) reinterpret_cast<float4*>(st)[i] = src[i];
    __syncthreads();
    const int L[3] = {sg.L[0], sg.L[1], sg.L[2]};
    uint32_t m32, m64 = 0;
    if (kPass1) {
      m32 = (w.count >= 32) ? 0xffffffffu : ((1u << w.count) - 1u);
    } else {
      if (tid < 32) {
        int tier = 0;
        if (tid < w.count) {
          const float lb = log2_bound(st + tid * stride, L, box);
          tier = lb > lt ? 2 : (lb > ls ? 1 : 0);
        }
        const uint32_t b32 = __ballot_sync(0xffffffffu, tier == 1);
        const uint32_t b64 = __ballot_sync(0xffffffffu, tier == 2);
        if (tid == 0) {
          s_m32 = b32;
          s_m64 = b64;
        }
      }
      __syncthreads();
      m32 = s_m32;
      m64 = s_m64;
      if (tid == 0) {
        n32 += __popc(m32);
        n64 += __popc(m64);
        nskip += w.count - __popc(m32) - __popc(m64);
      }
    }
    float a32[kPPTM], aabs[kPPTM];
#pragma unroll
    for (int p = 0; p < kPPTM; ++p) {
      a32[p] = 0.0f;
      aabs[p] = 0.0f;
    }
    while (m32) {
      const int q = __ffs(m32) - 1;
      m32 &= m32 - 1;
      const float* R = st + q * stride;
      const float s_hi = R[0], s_lo = R[1], A_hi = R[8], A_lo = R[9];
      float u[3][kPPTM];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float b_hi = R[2 + d], b_lo = R[5 + d];
#pragma unroll
        for (int p = 0; p < kPPTM; ++p) {
          float t1 = fmaf(s_lo, rh[d][p], b_lo);
          t1 = fmaf(s_hi, rl[d][p], t1);
          const float t2 = b_hi + t1;
          u[d][p] = fmaf(s_hi, rh[d][p], t2);
        }
      }
      float E[kPPTM];
#pragma unroll
      for (int p = 0; p < kPPTM; ++p) {
        float y = -u[0][p] * u[0][p];
        y = fmaf(-u[1][p], u[1][p], y);
        y = fmaf(-u[2][p], u[2][p], y);
        E[p] = ex2_approx(y);
      }
      const float* Cx = R + 12;
      const float* Cy = Cx + L[0] + 1;
      const float* Cz = Cy + L[1] + 1;
      float vx[kPPTM], vy[kPPTM], vz[kPPTM];
      poly_pts(L[0], Cx, u[0], vx);
      poly_pts(L[1], Cy, u[1], vy);
      poly_pts(L[2], Cz, u[2], vz);
#pragma unroll
      for (int p = 0; p < kPPTM; ++p) {
        const float P = ((E[p] * vx[p]) * vy[p]) * vz[p];
        if (kPass1) {
          const float t = fmaf(P, A_hi, P * A_lo);
          a32[p] += t;
          aabs[p] += fabsf(t);
        } else {
          a32[p] = fmaf(P, A_hi, fmaf(P, A_lo, a32[p]));
        }
      }
    }
#pragma unroll
    for (int p = 0; p < kPPTM; ++p) {
      acc[p] += static_cast<double>(a32[p]);
      if (kPass1) acc_abs[p] += static_cast<double>(aabs[p]);
    }
    if (!kPass1) {
      while (m64) {  // precise tier: the FP64 record, same arithmetic as the FP64 form
        const int q = __ffs(m64) - 1;
        m64 &= m64 - 1;
        const double* R = rec64 + sg.off64 + (w.rec - sg.first + q) * sg.stride;
        const double A = R[0], s = R[1], d0 = R[2], d1 = R[3], d2 = R[4];
        const double* Cx = R + kRecHeader;
        const double* Cy = Cx + L[0] + 1;
        const double* Cz = Cy + L[1] + 1;
#pragma unroll
        for (int p = 0; p < kPPTM; ++p) {
          const int64_t g = base + tid + p * kThreadsM;
          if (g >= ngrid) continue;
          const double rx = s * (px[g] + d0), ry = s * (py[g] + d1), rz = s * (pz[g] + d2);
          double vx = Cx[0], vy = Cy[0], vz = Cz[0];
          for (int m = 1; m <= L[0]; ++m) vx = fma(vx, rx, Cx[m]);
          for (int m = 1; m <= L[1]; ++m) vy = fma(vy, ry, Cy[m]);
          for (int m = 1; m <= L[2]; ++m) vz = fma(vz, rz, Cz[m]);
          const double e = exp(-(rx * rx + ry * ry + rz * rz));
          acc[p] += A * e * vx * vy * vz;
        }
      }
    }
  }
#pragma unroll
  for (int p = 0; p < kPPTM; ++p) {
    const int64_t g = base + tid + p * kThreadsM;
    if (g < ngrid) {
      partial[static_cast<int64_t>(blockIdx.y) * ngrid + g] = acc[p];
      if (kPass1) partial_abs[static_cast<int64_t>(blockIdx.y) * ngrid + g] = acc_abs[p];
    }
  }
  if (!kPass1 && tid == 0) {
    atomicAdd(&stats[0], n32);
    atomicAdd(&stats[1], n64);
    atomicAdd(&stats[2], nskip);
  }
}

// Bounding boxes of the point tiles (FP32, rounded outwards).
__global__ void k_tile_boxes(int64_t ngrid, const double* __restrict__ px, const double* __restrict__ py,
                             const double* __restrict__ pz, float* box) {
  const int tile = blockIdx.x;
  __shared__ double red[6][kThreadsM];
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int i = threadIdx.x; i < kTileM; i += blockDim.x) {
    const int64_t g = static_cast<int64_t>(tile) * kTileM + i;
    if (g >= ngrid) break;
    const double x[3] = {px[g], py[g], pz[g]};
    for (int d = 0; d < 3; ++d) {
      lo[d] = fmin(lo[d], x[d]);
      hi[d] = fmax(hi[d], x[d]);
    }
  }
  for (int d = 0; d < 3; ++d) {
    red[d][threadIdx.x] = lo[d];
    red[3 + d][threadIdx.x] = hi[d];
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int d = 0; d < 3; ++d) {
        red[d][threadIdx.x] = fmin(red[d][threadIdx.x], red[d][threadIdx.x + w]);
        red[3 + d][threadIdx.x] = fmax(red[3 + d][threadIdx.x], red[3 + d][threadIdx.x + w]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int d = 0; d < 3; ++d) {
      const double l = red[d][0], h = red[3 + d][0];
      box[tile * 8 + d] = static_cast<float>(l - (fabs(l) * 1e-6 + 1e-6));
      box[tile * 8 + 3 + d] = static_cast<float>(h + (fabs(h) * 1e-6 + 1e-6));
    }
}

// Per-point FP32 threshold tau_g and skip threshold sigma_g from per-segment scales, then the
// per-tile minima (log2). seg_of: segment of each point (nullptr: segment 0);
// mode 0: tau_g = T_o / w_g; mode 1 (max-norm): tau_g = T_o / M~_g; mode 2 (per point):
// tau_g = (eps max(|I~|-3 k u M~, 0) / (3 k u))^2 / M~_g.
__global__ void k_tile_thresholds(int64_t ngrid, int mode, const int* __restrict__ seg_of,
                                  const double* __restrict__ segT, const double* __restrict__ segS,
                                  const double* __restrict__ w, const double* __restrict__ I,
                                  const double* __restrict__ Mabs, double eps, double nsurv, float* lt,
                                  float* ls) {
  const int tile = blockIdx.x;
  __shared__ double r1[kThreadsM], r2[kThreadsM];
  double tmin = HUGE_VAL, smin = HUGE_VAL;
  for (int i = threadIdx.x; i < kTileM; i += blockDim.x) {
    const int64_t g = static_cast<int64_t>(tile) * kTileM + i;
    if (g >= ngrid) break;
    const int o = seg_of ? seg_of[g] : 0;
    double tau, sig;
    if (mode == 0) {
      tau = w[g] > 0.0 ? segT[o] / w[g] : HUGE_VAL;
      sig = segS[o];
    } else if (mode == 1) {
      tau = Mabs[g] > 0.0 ? segT[o] / Mabs[g] : HUGE_VAL;
      sig = segS[o];
    } else {
      const double lo = fmax(fabs(I[g]) - 3.0 * kKappaU * Mabs[g], 0.0);
      const double x = eps * lo / (3.0 * kKappaU);
      tau = Mabs[g] > 0.0 ? x * x / Mabs[g] : HUGE_VAL;
      sig = eps * lo / (3.0 * nsurv);
    }
    tmin = fmin(tmin, tau);
    smin = fmin(smin, sig);
  }
  r1[threadIdx.x] = tmin;
  r2[threadIdx.x] = smin;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      r1[threadIdx.x] = fmin(r1[threadIdx.x], r1[threadIdx.x + s]);
      r2[threadIdx.x] = fmin(r2[threadIdx.x], r2[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double t = r1[0], s = fmin(r2[0], t);
    lt[tile] = t >= HUGE_VAL ? HUGE_VALF : (t > 0.0 ? static_cast<float>(log2(t)) : -HUGE_VALF);
    ls[tile] = s >= HUGE_VAL ? HUGE_VALF : (s > 0.0 ? static_cast<float>(log2(s)) : -HUGE_VALF);
  }
}

// Segment sums of w*I, w*M and w (fixed-order block trees).
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

}  // namespace

int eval_mixed(inca_ctx* c, double eps) {
  const int64_t ngrid = c->ngrid;
  const int nchunks = static_cast<int>(c->chunks.size());
  if (nchunks == 0) {
    INCA_CUDA(c, cudaMemsetAsync(c->d_ivec.p, 0, sizeof(double) * ngrid, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    return INCA_OK;
  }
  const int64_t tiles = (ngrid + kTileM - 1) / kTileM;
  const int nsplit = choose_splits(tiles, nchunks, c->num_sms, 4);
  // scratch: partials (2 x nsplit x ngrid), M~ (ngrid), tile data, stats
  const size_t need = sizeof(double) * (2 * static_cast<size_t>(nsplit) * ngrid + ngrid) +
                      sizeof(float) * 10 * tiles + 64;
  if (c->d_scratch.reserve(need + 1024)) return set_error(c, INCA_E_NOMEM, "mixed scratch");
  double* part = reinterpret_cast<double*>(c->d_scratch.p);
  double* part_abs = part + static_cast<size_t>(nsplit) * ngrid;
  double* Mabs = part_abs + static_cast<size_t>(nsplit) * ngrid;
  float* tbox = reinterpret_cast<float*>(Mabs + ngrid);
  float* tlt = tbox + 8 * tiles;
  float* tls = tlt + tiles;
  unsigned long long* stats = reinterpret_cast<unsigned long long*>(
      (reinterpret_cast<uintptr_t>(tls + tiles) + 15) & ~uintptr_t(15));
  cudaEvent_t ev[5];
  for (auto& e : ev) INCA_CUDA(c, cudaEventCreate(&e));
  INCA_CUDA(c, cudaEventRecord(ev[0], c->stream));
  INCA_CUDA(c, cudaMemsetAsync(stats, 0, 3 * sizeof(unsigned long long), c->stream));
  dim3 grid(static_cast<unsigned>(tiles), static_cast<unsigned>(nsplit));
  // pass 1: estimate
  INCA_LAUNCH(c, k_mixed<true>, grid, kThreadsM, 0, c->d_chunks.p, nchunks, c->d_classes.p, c->d_rec32.p,
                                                   c->d_rec64.p, c->d_px.p, c->d_py.p, c->d_pz.p, ngrid, nsplit,
                                                   nullptr, nullptr, nullptr, part, part_abs, stats);
  INCA_CUDA(c, cudaGetLastError());
  INCA_CUDA(c, cudaEventRecord(ev[1], c->stream));
  INCA_LAUNCH(c, k_reduce_splits, nblk(ngrid), 256, 0, part, nsplit, ngrid, c->d_ivec.p);
  INCA_LAUNCH(c, k_reduce_splits, nblk(ngrid), 256, 0, part_abs, nsplit, ngrid, Mabs);
  INCA_LAUNCH(c, k_tile_boxes, static_cast<unsigned>(tiles), kThreadsM, 0, ngrid, c->d_px.p, c->d_py.p, c->d_pz.p, tbox);
  INCA_CUDA(c, cudaGetLastError());
  // thresholds per output kind
  const double N = static_cast<double>(c->nsurv);
  int mode = 2;
  std::vector<double> segT, segS;
  const int* seg_of = nullptr;
  const double* wptr = nullptr;
  DevBuf<double> dT, dS, dout;
  DevBuf<int64_t> doff;
  DevBuf<unsigned long long> dmax;
  auto rel = [&]() { dT.release(); dS.release(); dout.release(); doff.release(); dmax.release(); };
  if (c->grid_kind == GRID_RADIAL || c->grid_kind == GRID_SCAN) {
    mode = 0;
    wptr = c->d_w.p;
    std::vector<int64_t> off;
    if (c->grid_kind == GRID_RADIAL) {
      off = {0, ngrid};
    } else {
      off.assign(c->nradi + 1, 0);
      for (int s = 0; s < c->nradi; ++s) off[s + 1] = off[s] + c->h_smn[s];
      seg_of = c->d_cmap.p;  // shell index of each scan point
    }
    const int nseg = static_cast<int>(off.size()) - 1;
    if (doff.reserve(nseg + 1) || dout.reserve(3 * nseg)) {
      rel();
      return set_error(c, INCA_E_NOMEM, "thresholds");
    }
    INCA_CUDA(c, cudaMemcpyAsync(doff.p, off.data(), sizeof(int64_t) * (nseg + 1), cudaMemcpyHostToDevice, c->stream));
    INCA_LAUNCH(c, k_seg_sums, nseg, 256, 0, nseg, doff.p, c->d_w.p, c->d_ivec.p, Mabs, dout.p);
    std::vector<double> h(3 * nseg);
    INCA_CUDA(c, cudaMemcpyAsync(h.data(), dout.p, sizeof(double) * 3 * nseg, cudaMemcpyDeviceToHost, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    segT.resize(nseg);
    segS.resize(nseg);
    for (int s = 0; s < nseg; ++s) {
      const double O = h[3 * s], M = h[3 * s + 1], W = h[3 * s + 2];
      const double lo = std::max(std::fabs(O) - 3.0 * kKappaU * M, 0.0);
      const double x = eps * lo / (3.0 * kKappaU);
      segT[s] = M > 0.0 ? x * x / M : HUGE_VAL;
      segS[s] = (N > 0 && W > 0) ? eps * lo / (3.0 * N * W) : 0.0;
    }
  } else if (c->grid_kind == GRID_CUBE) {
    mode = 1;
    if (dmax.reserve(1)) {
      rel();
      return set_error(c, INCA_E_NOMEM, "thresholds");
    }
    INCA_CUDA(c, cudaMemsetAsync(dmax.p, 0, sizeof(unsigned long long), c->stream));
    const unsigned nb = static_cast<unsigned>(std::min<int64_t>(nblk(ngrid), 4096));
    INCA_LAUNCH(c, k_absmax, nb, 256, 0, ngrid, c->d_ivec.p, dmax.p);
    unsigned long long hm = 0;
    INCA_CUDA(c, cudaMemcpyAsync(&hm, dmax.p, sizeof(hm), cudaMemcpyDeviceToHost, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    double Imax;
    std::memcpy(&Imax, &hm, sizeof(double));
    const double x = eps * Imax / (3.0 * kKappaU);
    segT = {x * x};
    segS = {N > 0 ? eps * Imax / (3.0 * N) : 0.0};
  } else {
    segT = {0.0};
    segS = {0.0};
  }
  if (dT.reserve(segT.size()) || dS.reserve(segS.size())) {
    rel();
    return set_error(c, INCA_E_NOMEM, "thresholds");
  }
  INCA_CUDA(c, cudaMemcpyAsync(dT.p, segT.data(), sizeof(double) * segT.size(), cudaMemcpyHostToDevice, c->stream));
  INCA_CUDA(c, cudaMemcpyAsync(dS.p, segS.data(), sizeof(double) * segS.size(), cudaMemcpyHostToDevice, c->stream));
  INCA_LAUNCH(c, k_tile_thresholds, static_cast<unsigned>(tiles), kThreadsM, 0, 
      ngrid, mode, seg_of, dT.p, dS.p, wptr, c->d_ivec.p, Mabs, eps, N, tlt, tls);
  INCA_CUDA(c, cudaGetLastError());
  INCA_CUDA(c, cudaEventRecord(ev[2], c->stream));
  // pass 2: tiered evaluation
  INCA_LAUNCH(c, k_mixed<false>, grid, kThreadsM, 0, c->d_chunks.p, nchunks, c->d_classes.p, c->d_rec32.p,
                                                    c->d_rec64.p, c->d_px.p, c->d_py.p, c->d_pz.p, ngrid, nsplit,
                                                    tbox, tlt, tls, part, nullptr, stats);
  INCA_CUDA(c, cudaGetLastError());
  INCA_CUDA(c, cudaEventRecord(ev[3], c->stream));
  INCA_LAUNCH(c, k_reduce_splits, nblk(ngrid), 256, 0, part, nsplit, ngrid, c->d_ivec.p);
  INCA_CUDA(c, cudaGetLastError());
  INCA_CUDA(c, cudaEventRecord(ev[4], c->stream));
  INCA_CUDA(c, cudaEventSynchronize(ev[4]));
  rel();
  float t01 = 0, t23 = 0, t04 = 0;
  cudaEventElapsedTime(&t01, ev[0], ev[1]);
  cudaEventElapsedTime(&t23, ev[2], ev[3]);
  cudaEventElapsedTime(&t04, ev[0], ev[4]);
  for (auto& e : ev) cudaEventDestroy(e);
  unsigned long long hs[3] = {0, 0, 0};
  INCA_CUDA(c, cudaMemcpy(hs, stats, sizeof(hs), cudaMemcpyDeviceToHost));
  c->t_total_ms = t04;
  c->t_kernel_ms = t01 + t23;
  c->t_kernel_launches = 2;
  c->t_launches = 10;
  c->pairs_fp32 = static_cast<int64_t>(hs[0]);
  c->pairs_fp64 = static_cast<int64_t>(hs[1]);
  c->pairs_skip = static_cast<int64_t>(hs[2]);
  return INCA_OK;
}

}  // namespace inca
