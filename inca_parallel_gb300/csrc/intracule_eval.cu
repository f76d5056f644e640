// K2: evaluation of the intracule at every grid point (src/mod_intracule.f90:345-358):
//   I(r_g) = sum over surviving quartets q of A_q exp(-|r'|^2) Vx(r'_x) Vy(r'_y) Vz(r'_z),
//   r' = sqe_q (r_g + P_ik - P_jl), V_d a Horner polynomial of degree L_d.
//
// Work decomposition (both precisions): a CTA owns a tile of grid points (registers) and a
// strided subset of the class-uniform work chunks (<= 32 survivor records of one angular
// class, staged in shared memory). Each (tile, split) writes its FP64 partial sums; a second
// kernel adds the splits in a fixed order, so results are bit-reproducible run to run.
//
// INCA_FP64: every term in FP64 (the "plain FP64 GPU form").
// INCA_MIXED: see mixed_eval.cu.
#include <algorithm>
#include <cmath>

#include "inca_internal.h"

namespace inca {

int eval_mixed(inca_ctx* c, double tol);        // mixed_eval.cu
int eval_mixed_graph(inca_ctx* c, double tol);  // mixed_eval.cu

namespace {

constexpr int kThreads64 = 128;
constexpr int kPPT64 = 2;  // points per thread
constexpr int kTile64 = kThreads64 * kPPT64;
constexpr int kMaxStride64 = (kRecHeader + 3 * kMaxCoef + 1) & ~1;

__global__ void __launch_bounds__(kThreads64)
k_eval_fp64(const WorkChunk* __restrict__ chunks, int nchunks, const ClassSeg* __restrict__ segs,
            const double* __restrict__ rec64, const double* __restrict__ px,
            const double* __restrict__ py, const double* __restrict__ pz, int64_t ngrid, int nsplit,
            double* __restrict__ partial) {
  __shared__ double sh[32 * kMaxStride64];
  const int tid = threadIdx.x;
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kTile64;
  double x[kPPT64], y[kPPT64], z[kPPT64], acc[kPPT64];
#pragma unroll
  for (int p = 0; p < kPPT64; ++p) {
    const int64_t g = base + tid + p * kThreads64;
    const bool ok = g < ngrid;
    x[p] = ok ? px[g] : 0.0;
    y[p] = ok ? py[g] : 0.0;
    z[p] = ok ? pz[g] : 0.0;
    acc[p] = 0.0;
  }
  for (int ch = blockIdx.y; ch < nchunks; ch += nsplit) {
    const WorkChunk w = chunks[ch];
    const ClassSeg sg = segs[w.cls];
    const double* src = rec64 + sg.off64 + (w.rec - sg.first) * sg.stride;
    const int nd = w.count * sg.stride;
    __syncthreads();
    for (int i = tid; i < nd; i += kThreads64) sh[i] = src[i];
    __syncthreads();
    const int Lx = sg.L[0], Ly = sg.L[1], Lz = sg.L[2];
    for (int q = 0; q < w.count; ++q) {
      const double* R = sh + q * sg.stride;
      const double A = R[0], s = R[1], d0 = R[2], d1 = R[3], d2 = R[4];
      const double* Cx = R + kRecHeader;
      const double* Cy = Cx + Lx + 1;
      const double* Cz = Cy + Ly + 1;
#pragma unroll
      for (int p = 0; p < kPPT64; ++p) {
        const double rx = s * (x[p] + d0), ry = s * (y[p] + d1), rz = s * (z[p] + d2);
        double vx = Cx[0], vy = Cy[0], vz = Cz[0];
        for (int m = 1; m <= Lx; ++m) vx = fma(vx, rx, Cx[m]);
        for (int m = 1; m <= Ly; ++m) vy = fma(vy, ry, Cy[m]);
        for (int m = 1; m <= Lz; ++m) vz = fma(vz, rz, Cz[m]);
        const double e = exp(-(rx * rx + ry * ry + rz * rz));
        acc[p] += A * e * vx * vy * vz;
      }
    }
  }
#pragma unroll
  for (int p = 0; p < kPPT64; ++p) {
    const int64_t g = base + tid + p * kThreads64;
    if (g < ngrid) partial[static_cast<int64_t>(blockIdx.y) * ngrid + g] = acc[p];
  }
}

}  // namespace

// Sum the split partials in split order (deterministic).
__global__ void k_reduce_splits(const double* __restrict__ partial, int nsplit, int64_t ngrid,
                                double* __restrict__ out) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= ngrid) return;
  double s = 0.0;
  for (int k = 0; k < nsplit; ++k) s += partial[static_cast<int64_t>(k) * ngrid + g];
  out[g] = s;
}

// Number of quartet splits so that tiles x splits fill the GPU a few times over.
int choose_splits(int64_t tiles, int64_t nchunks, int num_sms, int ctas_per_sm) {
  const int64_t target = static_cast<int64_t>(num_sms) * ctas_per_sm * 4;
  int64_t s = (target + tiles - 1) / std::max<int64_t>(tiles, 1);
  s = std::max<int64_t>(1, std::min<int64_t>(s, nchunks));
  s = std::min<int64_t>(s, 4096);
  return static_cast<int>(s);
}

int eval_device(inca_ctx* c, int mode, double tol, bool graph) {
  if (!c->prepared) return set_error(c, INCA_E_STATE, "inca_eval: call inca_prepare first");
  if (c->grid_kind == GRID_NONE || c->ngrid <= 0) return set_error(c, INCA_E_STATE, "inca_eval: no grid");
  if (c->batch_molecules > 0 && c->batch_grid_version != c->grid_version)
    return set_error(c, INCA_E_STATE, "inca_eval: the batch's grid was replaced; prepare the batch again");
  if (c->d_ivec.reserve(c->ngrid)) return set_error(c, INCA_E_NOMEM, "ivec");
  c->t_total_ms = c->t_kernel_ms = c->t_pass2_ms = 0;
  c->t_kernel_launches = c->t_launches = 0;
  c->pairs_fp32 = c->pairs_fp64 = c->pairs_skip = c->corrected_points = c->pairs_cheap = 0;
  if (mode == INCA_MIXED) {
    const int st = graph ? eval_mixed_graph(c, tol > 0 ? tol : 1e-10) : eval_mixed(c, tol > 0 ? tol : 1e-10);
    if (st == INCA_OK) c->evaluated = true;
    return st;
  }
  if (mode == INCA_FP64_SCREENED && !cube_separable(c)) {
    bool plain = false;
    const int st = eval_fp64_screened(c, tol > 0 ? tol : 1e-10, &plain);
    if (st != INCA_OK) return st;
    if (!plain) {
      c->evaluated = true;
      return INCA_OK;
    }
  } else if (mode != INCA_FP64 && mode != INCA_FP64_SCREENED) {
    return set_error(c, INCA_E_ARG, "inca_eval: unknown mode");
  }
  const int64_t ngrid = c->ngrid;
  const int nchunks = static_cast<int>(c->chunks.size());
  cudaEvent_t e0, e1, e2;
  INCA_CUDA(c, cudaEventCreate(&e0));
  INCA_CUDA(c, cudaEventCreate(&e1));
  INCA_CUDA(c, cudaEventCreate(&e2));
  if (nchunks == 0) {
    INCA_CUDA(c, cudaMemsetAsync(c->d_ivec.p, 0, sizeof(double) * ngrid, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
    c->evaluated = true;
    return INCA_OK;
  }
  // one launch pair per molecule of a batch (each molecule's points against its own chunks)
  const int nmol = c->batch_molecules > 0 ? c->batch_molecules : 1;
  INCA_CUDA(c, cudaEventRecord(e0, c->stream));
  int launches = 0;
  for (int m = 0; m < nmol; ++m) {
    const int64_t p0 = c->batch_molecules > 0 ? c->h_mol_off[m] : 0;
    const int64_t np = c->batch_molecules > 0 ? c->h_mol_off[m + 1] - p0 : ngrid;
    const int cb = c->mol_chunks[m].begin, nch = c->mol_chunks[m].end - c->mol_chunks[m].begin;
    if (np == 0) continue;
    if (nch <= 0) {
      INCA_CUDA(c, cudaMemsetAsync(c->d_ivec.p + p0, 0, sizeof(double) * np, c->stream));
      continue;
    }
    const int64_t tiles = (np + kTile64 - 1) / kTile64;
    const int nsplit = choose_splits(tiles, nch, c->num_sms, 4);
    if (c->d_partial.reserve(static_cast<size_t>(nsplit) * np)) return set_error(c, INCA_E_NOMEM, "partials");
    dim3 grid(static_cast<unsigned>(tiles), static_cast<unsigned>(nsplit));
    INCA_LAUNCH(c, k_eval_fp64, grid, kThreads64, 0, c->d_chunks.p + cb, nch, c->d_classes.p, c->d_rec64.p,
                c->d_px.p + p0, c->d_py.p + p0, c->d_pz.p + p0, np, nsplit, c->d_partial.p);
    INCA_CUDA(c, cudaGetLastError());
    INCA_LAUNCH(c, k_reduce_splits, static_cast<unsigned>((np + 255) / 256), 256, 0, c->d_partial.p, nsplit, np,
                c->d_ivec.p + p0);
    INCA_CUDA(c, cudaGetLastError());
    launches += 2;
  }
  INCA_CUDA(c, cudaEventRecord(e1, c->stream));
  INCA_CUDA(c, cudaEventRecord(e2, c->stream));
  INCA_CUDA(c, cudaEventSynchronize(e2));
  float a = 0, b = 0;
  cudaEventElapsedTime(&a, e0, e1);
  cudaEventElapsedTime(&b, e0, e2);
  c->t_kernel_ms = a;
  c->t_total_ms = b;
  c->t_kernel_launches = launches / 2;
  c->t_launches = launches;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  c->evaluated = true;
  return INCA_OK;
}

}  // namespace inca
