// K2 for cube lattices (cubeintra, INCA_MIXED): separable double-float evaluation.
//
// The cube grid (src/mod_build_grid.f90:412-440) is a lattice x_i = x0 + i hx, y_j, z_k, and the
// point loop (src/mod_intracule.f90:345-358) evaluates at each point
//   A' 2^(-|u|^2 + ks) prod_d Vn_d(u_d),   u = s (r + d)   (FP32 record, see mixed_eval.cu).
// Every factor depends on one coordinate only, so on the lattice the term is a product
//   A' F_x(i) F_y(j) F_z(k),   F_d = 2^(-u_d^2 + k_d) Vn_d(u_d),   k_x + k_y + k_z = ks,
// and a tile of kTX x kTY x kTZ points needs kTX + kTY + kTZ = 32 factor evaluations per quartet
// instead of 1024 terms: one factor per lane. Factors are evaluated in double-float (~2^-44),
// the products A' F_y F_z (per lane and z) and F_x (A' F_y F_z) are compensated and accumulated
// in double-float, folded into FP64 every few chunks. Every term is then accurate to ~2^-44
// relative: no error model, thresholds, estimate pass or corrections (the result agrees with the
// FP64 form to ~1e-13 whatever the tolerance asked for).
//
// Work: one-warp CTAs take (split, tile) items from a device counter (items of one split run
// side by side, so they read the same chunks while those are in L2); a split walks every
// nsplit-th quartet chunk, staged by double-buffered TMA bulk copies, skipping records whose
// bound over the tile is below a floor (2^-120, or the tolerance-budgeted floor of
// eval_cube_separable). Each item writes its partial sums in the grid's own
// order; a second kernel adds the splits in a fixed order (bit-reproducible results). Within a
// live record, an x slab (the 128 points of one i) whose terms all stay below the same floor is
// left out too: a record contributes at most one left-out term per point either way, so the
// budget of the floor holds. (With the 2^-120 floor alone the slab test cost 1-4 %; with the
// tolerance-budgeted floor it saves 3 % on CH4 cubes and 9-10 % on a 20-atom molecule.)
// Lane l evaluates factor l (x for l < 8, y for l < 16, z otherwise) and owns the 32 points
// (i, j0 + l/4, k0 + 4 (l%4) + e), i < 8, e < 4.
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "inca_internal.h"
#include "stage_df.cuh"

namespace inca {
namespace {

constexpr int kTX = 8, kTY = 8, kTZ = 16;  // lattice tile: 1024 points, 32 factors
constexpr int kZPL = 4;                    // z points per lane
constexpr int kCubeFold = 8;               // chunks between FP64 folds
constexpr float kCubeSkipLog2 = -120.0f;   // records whose tile bound is below 2^-120 are skipped
#ifndef INCA_CUBE_SLAB_SKIP
#define INCA_CUBE_SLAB_SKIP 1
#endif
#ifndef INCA_CUBE_CTAS_PER_SM
#define INCA_CUBE_CTAS_PER_SM 12
#endif
static_assert(kTX + kTY + kTZ == 32 && kTY * (kTZ / kZPL) == 32, "one factor and 32 points per lane");

struct CubeDims {
  int n[3];   // lattice points per axis
  int nt[3];  // tiles per axis
};

// Axis coordinates of the lattice points with indices 0, st, 2 st, ... (st = 1: every point),
// read back from the lattice itself (both forms then see the same bits): the x run, then y, z.
__global__ void k_cube_axes(const double* __restrict__ px, const double* __restrict__ py,
                            const double* __restrict__ pz, int nx, int ny, int nz, int st, double* __restrict__ ax) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int mx = (nx + st - 1) / st, my = (ny + st - 1) / st, mz = (nz + st - 1) / st;
  if (t < mx)
    ax[t] = px[static_cast<int64_t>(t) * st * ny * nz];
  else if (t < mx + my)
    ax[t] = py[static_cast<int64_t>(t - mx) * st * nz];
  else if (t < mx + my + mz)
    ax[t] = pz[static_cast<int64_t>(t - mx - my) * st];
}

// max |x_i| over n values into *M (one block)
__global__ void k_absmax(int64_t n, const double* __restrict__ x, double* M) {
  __shared__ double sh[256];
  double m = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(x[i]));
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *M = sh[0];
}

// The share of the tolerance given to left-out terms: INCA_DROP_FRACTION, else the context's
// schedule (inca_set_tuning), else 0.05.
double drop_fraction(const inca_ctx* c) {
  if (const char* e = std::getenv("INCA_DROP_FRACTION")) {
    char* end = nullptr;
    const double v = std::strtod(e, &end);
    if (end != e && v >= 0.0 && v < 0.5) return v;
  }
  return c->tune_drop >= 0.0 ? c->tune_drop : 0.05;
}

// Compensated product x y of double-float values, added to the double-float accumulator (h, l):
// p + pe = x y to ~2^-46, then TwoSum(h, p) with its rounding error and pe going to l.
__device__ __forceinline__ void acc_prod(float& h, float& l, float xh, float xl, f2 g) {
  const float p = __fmul_rn(xh, g.hi);
  float pe = __fmaf_rn(xh, g.hi, -p);
  pe = __fmaf_rn(xh, g.lo, pe);
  pe = __fmaf_rn(xl, g.hi, pe);
  const float s = __fadd_rn(h, p);
  const float bb = __fsub_rn(s, h);
  const float er = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  h = s;
  l = __fadd_rn(l, __fadd_rn(er, pe));
}

__global__ void __launch_bounds__(32, INCA_CUBE_CTAS_PER_SM)
k_cube_sep(const WorkChunk* __restrict__ chunks, int nchunks, const ClassSeg* __restrict__ segs,
           const float* __restrict__ rec32, const double* __restrict__ axes, CubeDims D, int nsplit,
           int64_t nitems, int stage_floats, float floor_log2, const float2* __restrict__ exp_tab,
           double* __restrict__ part,
           unsigned long long* __restrict__ work, unsigned long long* __restrict__ stats, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char dsm[];
  const Stage S = stage_view(dsm, stage_floats);
  __shared__ float2 tab[kExpTab + 1];
  __shared__ float2 fac[32];
  __shared__ double acc64[kTX][kZPL][32];
  const int lane = threadIdx.x;
  for (int i = lane; i <= kExpTab; i += 32) tab[i] = exp_tab[i];
  stage_init(S);
  const int64_t ngrid = static_cast<int64_t>(D.n[0]) * D.n[1] * D.n[2];
  const int64_t ntiles = static_cast<int64_t>(D.nt[0]) * D.nt[1] * D.nt[2];
  // this lane's factor (dimension fd, offset fo within the tile) and points (y jl, z kl + e)
  const int fd = lane < kTX ? 0 : (lane < kTX + kTY ? 1 : 2);
  const int fo = fd == 0 ? lane : (fd == 1 ? lane - kTX : lane - kTX - kTY);
  const int ao = fd == 0 ? 0 : (fd == 1 ? D.n[0] : D.n[0] + D.n[1]);
  const int nfd = fd == 0 ? D.n[0] : (fd == 1 ? D.n[1] : D.n[2]);
  const int jl = lane >> 2, kl = (lane & 3) * kZPL;
  const float floor_v = exp2f(floor_log2);
  unsigned long long nlive = 0, nskip = 0;
  int k = 0;  // chunks taken by this CTA so far: selects buffer and barrier phase
  for (;;) {
    const int64_t item = next_item(work);
    if (item >= nitems) break;
    const int split = static_cast<int>(item / ntiles);
    const int64_t tile = item - static_cast<int64_t>(split) * ntiles;
    const int tz = static_cast<int>(tile % D.nt[2]);
    const int64_t rest = tile / D.nt[2];
    const int ty = static_cast<int>(rest % D.nt[1]);
    const int tx = static_cast<int>(rest / D.nt[1]);
    const int b0[3] = {tx * kTX, ty * kTY, tz * kTZ};
    if (split < nchunks) stage_first(S, chunks, segs, rec32, k, split);
    const int bfd = fd == 0 ? b0[0] : (fd == 1 ? b0[1] : b0[2]);
    const double xc = axes[ao + min(bfd + fo, nfd - 1)];
    const float xh = static_cast<float>(xc), xl = static_cast<float>(xc - static_cast<double>(xh));
    // bounding box of the tile's lattice points (widened by a few FP32 ulps)
    float box[6];
    {
      const int o[3] = {0, D.n[0], D.n[0] + D.n[1]};
      const int ext[3] = {kTX, kTY, kTZ};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const double a = axes[o[d] + b0[d]], b = axes[o[d] + min(b0[d] + ext[d], D.n[d]) - 1];
        const double lo = fmin(a, b), hi = fmax(a, b), pad = 1e-6 * fmax(fabs(lo), fabs(hi)) + 1e-30;
        box[d] = static_cast<float>(lo - pad);
        box[3 + d] = static_cast<float>(hi + pad);
      }
    }
#pragma unroll
    for (int i = 0; i < kTX; ++i)
#pragma unroll
      for (int e = 0; e < kZPL; ++e) acc64[i][e][lane] = 0.0;
    float h[kTX][kZPL], l[kTX][kZPL];
#pragma unroll
    for (int i = 0; i < kTX; ++i)
#pragma unroll
      for (int e = 0; e < kZPL; ++e) h[i][e] = l[i][e] = 0.0f;
    __syncwarp();
    int nfold = 0;
    bool ok = true;
    for (int ch = split; ch < nchunks; ch += nsplit, ++k) {
      ok = __all_sync(0xffffffffu, stage_next(S, chunks, segs, rec32, k, ch + nsplit, nchunks));
      if (!ok) break;
      const WorkChunk w = chunks[ch];
      const ClassSeg sg = segs[w.cls];
      const float* st = S.buf(k);
      const int L[3] = {sg.L[0], sg.L[1], sg.L[2]};
      const float lb = lane < w.count ? log2_bound(st + lane * sg.stride32, L, box) : -HUGE_VALF;
      uint32_t live = __ballot_sync(0xffffffffu, lane < w.count && lb > floor_log2);
      if (lane == 0) {
        nlive += __popc(live);
        nskip += w.count - __popc(live);
      }
      const int nc = L[0] + L[1] + L[2] + 3;
      const int Ld = fd == 0 ? L[0] : (fd == 1 ? L[1] : L[2]);
      const int co = 12 + (fd > 0 ? L[0] + 1 : 0) + (fd > 1 ? L[1] + 1 : 0);
      while (live) {
        const int q = __ffs(live) - 1;
        live &= live - 1;
        const float* R = st + q * sg.stride32;
        // factor fd of record q at this lane's coordinate, in double-float
        const int ks = static_cast<int>(R[11]);
        const int kx = ks / 3, ky = (ks - kx) / 2;
        const int kd = fd == 0 ? kx : (fd == 1 ? ky : ks - kx - ky);
        f2 u;
        {
          const float s_hi = R[0], s_lo = R[1];
          const float p = __fmul_rn(s_hi, xh);
          float e = __fmaf_rn(s_hi, xh, -p);
          const f2 t = two_sum(p, R[2 + fd]);
          e = __fadd_rn(e, t.lo);
          e = __fmaf_rn(s_hi, xl, e);
          e = __fmaf_rn(s_lo, xh, e);
          e = __fadd_rn(e, R[5 + fd]);
          u = fast_two_sum(t.hi, e);
        }
        f2 y = df_sqr(u);
        y.hi = -y.hi;
        y.lo = -y.lo;
        f2 F = df_exp2(y, kd, tab);
        if (fabsf(u.hi) > kUClamp) u = {copysignf(kUClamp, u.hi), 0.0f};
        f2 v = {R[co], R[co + nc]};  // Ld = 0: the normalised constant +-1
        for (int m = 1; m <= Ld; ++m) v = df_add(df_mul(v, u), f2{R[co + m], R[co + m + nc]});
        F = df_mul(F, v);
        __syncwarp();
        fac[lane] = make_float2(F.hi, F.lo);
        __syncwarp();
        // G_e = A' F_y(jl) F_z(kl + e), then the 32 terms F_x(i) G_e
        const float2 fy = fac[kTX + jl];
        const f2 AY = df_mul(f2{R[8], R[9]}, f2{fy.x, fy.y});
        f2 G[kZPL];
#pragma unroll
        for (int e = 0; e < kZPL; ++e) {
          const float2 fz = fac[kTX + kTY + kl + e];
          G[e] = df_mul(AY, f2{fz.x, fz.y});
        }
#if INCA_CUBE_SLAB_SKIP
        // an x slab whose 128 terms all stay below the floor is left out (warp-uniform test with
        // the warp's largest |A' F_y F_z|; hi parts, so the bound carries a 2^-20 margin)
        unsigned gbits = 0;
#pragma unroll
        for (int e = 0; e < kZPL; ++e) gbits = max(gbits, __float_as_uint(fabsf(G[e].hi)));
        const float gmax = __uint_as_float(__reduce_max_sync(0xffffffffu, gbits)) * (1.0f + 0x1p-20f);
#endif
#pragma unroll
        for (int i = 0; i < kTX; ++i) {
          const float2 fx = fac[i];
#if INCA_CUBE_SLAB_SKIP
          if (fabsf(fx.x) * gmax < floor_v) continue;
#endif
#pragma unroll
          for (int e = 0; e < kZPL; ++e) acc_prod(h[i][e], l[i][e], fx.x, fx.y, G[e]);
        }
      }
      if (++nfold == kCubeFold) {
        nfold = 0;
#pragma unroll
        for (int i = 0; i < kTX; ++i)
#pragma unroll
          for (int e = 0; e < kZPL; ++e) {
            acc64[i][e][lane] += static_cast<double>(h[i][e]) + static_cast<double>(l[i][e]);
            h[i][e] = l[i][e] = 0.0f;
          }
      }
      __syncwarp();
    }
    if (!ok) {
      if (lane == 0) atomicExch(err, 1);
      break;
    }
    const int j = b0[1] + jl;
#pragma unroll
    for (int i = 0; i < kTX; ++i)
#pragma unroll
      for (int e = 0; e < kZPL; ++e) {
        const int ii = b0[0] + i, kk = b0[2] + kl + e;
        const double a = acc64[i][e][lane] + (static_cast<double>(h[i][e]) + static_cast<double>(l[i][e]));
        if (ii < D.n[0] && j < D.n[1] && kk < D.n[2])
          part[static_cast<int64_t>(split) * ngrid + (static_cast<int64_t>(ii) * D.n[1] + j) * D.n[2] + kk] = a;
      }
    __syncwarp();
  }
  if (lane == 0) {
    atomicAdd(&stats[0], nlive);
    atomicAdd(&stats[1], nskip);
  }
}

// out[g] = sum over splits s of part[s n + g], 16 threads per point each adding every 16th split
// in increasing order, then the 16 sums in thread order (a fixed order: reproducible bits).
constexpr int kSumLanes = 16;
__global__ void __launch_bounds__(32 * kSumLanes)
k_sum_split_major(int64_t n, int nsplit, const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double sh[kSumLanes][33];
  const int64_t g = blockIdx.x * 32LL + threadIdx.x;
  const int y = threadIdx.y;
  double s = 0.0;
  if (g < n)
    for (int k = y; k < nsplit; k += kSumLanes) s += part[static_cast<int64_t>(k) * n + g];
  sh[y][threadIdx.x] = s;
  __syncthreads();
  if (y == 0 && g < n) {
    double t = sh[0][threadIdx.x];
#pragma unroll
    for (int r = 1; r < kSumLanes; ++r) t += sh[r][threadIdx.x];
    out[g] = t;
  }
}

}  // namespace

// The separable form serves INCA_MIXED on cube lattices of a single molecule; the environment
// variable INCA_CUBE_SEPARABLE=0 selects the general mixed form instead (for comparisons).
bool cube_separable(const inca_ctx* c) {
  if (c->grid_kind != GRID_CUBE || c->batch_molecules > 0) return false;
  const char* env = std::getenv("INCA_CUBE_SEPARABLE");
  return !(env && env[0] == '0');
}

namespace {

// One pass of k_cube_sep + the split sums over a lattice (axes: x run, y run, z run) into out.
// Records whose bound over a tile is below 2^floor_log2 are left out.
struct CubeRun {
  unsigned long long live = 0, skip = 0;
};
int cube_pass(inca_ctx* c, const double* axes, const int n[3], float floor_log2, double* out, CubeRun* run) {
  const int nchunks = static_cast<int>(c->chunks.size());
  CubeDims D;
  const int ext[3] = {kTX, kTY, kTZ};
  for (int d = 0; d < 3; ++d) {
    D.n[d] = n[d];
    D.nt[d] = (n[d] + ext[d] - 1) / ext[d];
  }
  const int64_t ngrid = static_cast<int64_t>(n[0]) * n[1] * n[2];
  int max_stride = 4;
  for (const ClassSeg& sg : c->classes) max_stride = std::max(max_stride, sg.stride32);
  const int stage_floats = kChunkMax * max_stride;
  const size_t dsmem = 128 + 2 * sizeof(float) * stage_floats;
  INCA_CUDA(c, cudaFuncSetAttribute(k_cube_sep, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(dsmem)));
  int occ = 0;
  INCA_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cube_sep, 32, dsmem));
  occ = std::max(occ, 1);
  const int64_t ntiles = static_cast<int64_t>(D.nt[0]) * D.nt[1] * D.nt[2];
  // splits: about four items per resident CTA; at most one per chunk, 4096 in all, and 2^27
  // partial sums
  const int64_t target = static_cast<int64_t>(c->num_sms) * occ * 4;
  int64_t nsplit = (target + ntiles - 1) / ntiles;
  nsplit = std::min<int64_t>(nsplit, std::min<int64_t>(nchunks, 4096));
  nsplit = std::min<int64_t>(nsplit, std::max<int64_t>(1, (int64_t(1) << 27) / ngrid));
  nsplit = std::max<int64_t>(nsplit, 1);
  const int64_t nitems = ntiles * nsplit;
  if (c->d_partial.reserve(static_cast<size_t>(nsplit * ngrid))) return set_error(c, INCA_E_NOMEM, "cube partials");
  unsigned long long* work = reinterpret_cast<unsigned long long*>(c->d_scratch.p);
  unsigned long long* stats = work + 1;
  int* errw = reinterpret_cast<int*>(work + 4);
  INCA_CUDA(c, cudaMemsetAsync(work, 0, 64, c->stream));
  const unsigned nctas = static_cast<unsigned>(std::min<int64_t>(nitems, static_cast<int64_t>(c->num_sms) * occ));
  INCA_LAUNCH(c, k_cube_sep, nctas, 32, dsmem, c->d_chunks.p, nchunks, c->d_classes.p, c->d_rec32.p, axes, D,
              static_cast<int>(nsplit), nitems, stage_floats, floor_log2, c->d_exptab.p, c->d_partial.p, work, stats,
              errw);
  INCA_CUDA(c, cudaGetLastError());
  INCA_LAUNCH(c, k_sum_split_major, static_cast<unsigned>((ngrid + 31) / 32), dim3(32, kSumLanes), 0, ngrid,
              static_cast<int>(nsplit), c->d_partial.p, out);
  INCA_CUDA(c, cudaGetLastError());
  unsigned long long hs[2] = {};
  int herr = 0;
  INCA_CUDA(c, cudaMemcpyAsync(hs, stats, sizeof(hs), cudaMemcpyDeviceToHost, c->stream));
  INCA_CUDA(c, cudaMemcpyAsync(&herr, errw, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  INCA_CUDA(c, cudaStreamSynchronize(c->stream));
  if (herr) return set_error(c, INCA_E_TIMEOUT, "inca_eval: a bounded wait for a staged quartet chunk gave up");
  run->live += hs[0];
  run->skip += hs[1];
  return INCA_OK;
}

}  // namespace

// Tolerance-budgeted dropping: a coarse pre-pass on every kCoarse-th lattice point (itself a
// lattice, evaluated the same way) gives M = max |I| over those points, a lower bound of the
// cube's max |I| (every 4th point from 32 points per axis, every 2nd from 16). The main pass
// then leaves out every record whose bound over a tile is below
// theta = f eps M / N (N survivors, f = INCA_DROP_FRACTION, 0.05 by default): at any point the
// left-out terms sum to at most f eps max |I|, the cube's max-norm tolerance share. Lattices with
// an axis below 16 points skip the pre-pass (floor 2^-120 only).
int eval_cube_separable(inca_ctx* c, double eps) {
  const int64_t ngrid = c->ngrid;
  const int nchunks = static_cast<int>(c->chunks.size());
  c->t_total_ms = c->t_kernel_ms = c->t_pass2_ms = 0;
  if (nchunks == 0) {
    INCA_CUDA(c, cudaMemsetAsync(c->d_ivec.p, 0, sizeof(double) * ngrid, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    return INCA_OK;
  }
  const int64_t l0 = c->launches;
  const int* n = c->cube_np;
  const int nmin = std::min(n[0], std::min(n[1], n[2]));
  const int coarse = nmin >= 32 ? 4 : (nmin >= 16 ? 2 : 0);
  int m[3] = {0, 0, 0};
  if (coarse)
    for (int d = 0; d < 3; ++d) m[d] = (n[d] + coarse - 1) / coarse;
  const int naxes = n[0] + n[1] + n[2], maxes = m[0] + m[1] + m[2];
  if (c->cube_axes_version != c->grid_version || c->d_cube_axes.n < static_cast<size_t>(naxes + maxes)) {
    if (c->d_cube_axes.reserve(naxes + maxes)) return set_error(c, INCA_E_NOMEM, "cube axes");
    INCA_LAUNCH(c, k_cube_axes, static_cast<unsigned>((naxes + 127) / 128), 128, 0, c->d_px.p, c->d_py.p, c->d_pz.p,
                n[0], n[1], n[2], 1, c->d_cube_axes.p);
    INCA_CUDA(c, cudaGetLastError());
    c->cube_axes_version = c->grid_version;
  }
  int st = ensure_exp_table(c);
  if (st) return st;
  const int64_t ncoarse = static_cast<int64_t>(m[0]) * m[1] * m[2];
  if (c->d_scratch.reserve(256 + 8 * ncoarse + 64)) return set_error(c, INCA_E_NOMEM, "cube counters");
  double* Icoarse = reinterpret_cast<double*>(c->d_scratch.p + 256);
  cudaEvent_t ev[2] = {};
  for (auto& e : ev) INCA_CUDA(c, cudaEventCreate(&e));
  struct Guard {
    cudaEvent_t* e;
    ~Guard() {
      for (int i = 0; i < 2; ++i) cudaEventDestroy(e[i]);
    }
  } guard{ev};
  INCA_CUDA(c, cudaEventRecord(ev[0], c->stream));
  CubeRun run;
  float floor_log2 = kCubeSkipLog2;
  const double frac = drop_fraction(c);
  if (coarse && frac > 0.0 && eps > 0.0) {
    double* sub = c->d_cube_axes.p + naxes;
    INCA_LAUNCH(c, k_cube_axes, static_cast<unsigned>((maxes + 127) / 128), 128, 0, c->d_px.p, c->d_py.p, c->d_pz.p,
                n[0], n[1], n[2], coarse, sub);
    INCA_CUDA(c, cudaGetLastError());
    if ((st = cube_pass(c, sub, m, kCubeSkipLog2, Icoarse, &run))) return st;
    double* M = Icoarse + ncoarse;
    INCA_CUDA(c, cudaMemsetAsync(M, 0, sizeof(double), c->stream));
    INCA_LAUNCH(c, k_absmax, 1, 256, 0, ncoarse, Icoarse, M);
    double hM = 0.0;
    INCA_CUDA(c, cudaMemcpyAsync(&hM, M, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    const double nsurv = static_cast<double>(std::max<int64_t>(c->nsurv, 1));
    const double theta = frac * eps * hM / nsurv;
    if (theta > 0.0 && std::isfinite(theta))
      floor_log2 = std::max(kCubeSkipLog2, static_cast<float>(std::floor(std::log2(theta))));
  }
  c->cube_floor_log2 = floor_log2;
  if ((st = cube_pass(c, c->d_cube_axes.p, n, floor_log2, c->d_ivec.p, &run))) return st;
  INCA_CUDA(c, cudaEventRecord(ev[1], c->stream));
  INCA_CUDA(c, cudaEventSynchronize(ev[1]));
  float t01 = 0;
  cudaEventElapsedTime(&t01, ev[0], ev[1]);
  c->t_kernel_ms = t01;
  c->t_total_ms = t01;
  c->t_kernel_launches = 1;
  c->t_launches = static_cast<int>(c->launches - l0);
  c->pairs_fp32 = 0;
  c->pairs_fp64 = static_cast<int64_t>(run.live);  // (record, tile) pairs evaluated in double-float
  c->pairs_skip = static_cast<int64_t>(run.skip);
  c->corrected_points = 0;
  c->pairs_cheap = 0;
  return INCA_OK;
}

}  // namespace inca
