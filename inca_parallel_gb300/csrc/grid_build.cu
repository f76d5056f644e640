// K3: grids on the device (src/mod_build_grid.f90) and K4: the post-reductions of
// calculate_intracule (src/mod_intracule.f90:441-455, 522-530, 576-649). FP64 throughout.
//
// This translation unit is compiled with -fmad=false: grid points and weights are then the
// same bits as the CPU oracle's (an FMA-contracted x0 + s*i differs in the last place, which
// can move a point across the 1e-106 weight cut or a z >= -tol test).
//
// Grids are stored as FP64 structure-of-arrays (x, y, z, weight, Vee weight, centre) in the
// reference's point order: centre-major, then radial node, then Lebedev point; shells in
// order for the radial scan; x outer / z inner for the cube. Reductions are deterministic
// (fixed-order block trees over contiguous segments).
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

#include "inca_internal.h"

namespace inca {
namespace {

// Candidate points of a multicentre grid: one thread per (centre, radial node, Lebedev point).
struct RadialCentre {
  double cx, cy, cz;
  int nrad, nang;
  int64_t first;     // first candidate index of this centre
  int rad_off;       // offset into the radial tables
  int ang_off;       // offset into the angular tables
};

__global__ void k_radial_candidates(int64_t ncand, const RadialCentre* __restrict__ cen, int nquad,
                                    const double* __restrict__ radius, const double* __restrict__ wrad,
                                    const double* __restrict__ lx, const double* __restrict__ ly,
                                    const double* __restrict__ lz, const double* __restrict__ lw, int nosym,
                                    double* ox, double* oy, double* oz, double* ow, int* oc,
                                    uint8_t* keep) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= ncand) return;
  int c = 0;
  while (c + 1 < nquad && cen[c + 1].first <= g) ++c;
  const RadialCentre C = cen[c];
  const int64_t local = g - C.first;
  const int ir = static_cast<int>(local / C.nang), ia = static_cast<int>(local % C.nang);
  const double r = radius[C.rad_off + ir];
  const double x = r * lx[C.ang_off + ia] + C.cx;
  const double y = r * ly[C.ang_off + ia] + C.cy;
  const double z = r * lz[C.ang_off + ia] + C.cz;
  const double tol = 1e-100;
  double w = lw[C.ang_off + ia] * wrad[C.rad_off + ir];
  bool k = true;
  if (!nosym) {
    k = z >= -tol;
    if (fabs(z) >= tol) w = 2.0 * lw[C.ang_off + ia] * wrad[C.rad_off + ir];
  }
  ox[g] = x;
  oy[g] = y;
  oz[g] = z;
  ow[g] = w;
  oc[g] = c;
  keep[g] = k ? 1 : 0;
}

// TFVC partition (becke, mod_build_grid.f90:474-575): P_i = prod_{j != i} s(nu_ij),
// nu = (1 + mu - chi(1 - mu)) / (1 + mu + chi(1 - mu)), s = (1 - p(p(p(p(nu))))) / 2,
// p(x) = 1.5 x - 0.5 x^3; weight of a point of centre c multiplied by P_c / sum_i P_i.
__global__ void k_tfvc(int64_t n, const double* __restrict__ px, const double* __restrict__ py,
                       const double* __restrict__ pz, const int* __restrict__ cmap, int nquad,
                       const double* __restrict__ cent, const double* __restrict__ Rij,
                       const double* __restrict__ chi, double* w) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= n) return;
  const double x = px[g], y = py[g], z = pz[g];
  const int own = cmap[g];
  double ptot = 0.0, pown = 0.0;
  for (int i = 0; i < nquad; ++i) {
    const double dxi = x - cent[3 * i], dyi = y - cent[3 * i + 1], dzi = z - cent[3 * i + 2];
    const double ri = sqrt(dxi * dxi + dyi * dyi + dzi * dzi);
    double P = 1.0;
    for (int j = 0; j < nquad; ++j) {
      if (j == i) continue;
      const double dxj = x - cent[3 * j], dyj = y - cent[3 * j + 1], dzj = z - cent[3 * j + 2];
      const double rj = sqrt(dxj * dxj + dyj * dyj + dzj * dzj);
      const double R = Rij[i * nquad + j];
      const double mu = R > 1e-12 ? (ri - rj) * (1.0 / R) : 0.0;
      const double term = chi[i * nquad + j] * (1.0 - mu);
      double v = (1.0 + mu - term) / (1.0 + mu + term);
#pragma unroll
      for (int k = 0; k < 4; ++k) v = 1.5 * v - 0.5 * ((v * v) * v);
      P *= 0.5 * (1.0 - v);
    }
    ptot += P;
    if (i == own) pown = P;
  }
  double wb = pown;
  if (ptot > 1e-15) wb = wb * (1.0 / ptot);
  w[g] = w[g] * wb;
}

__global__ void k_weight_keep(int64_t n, const double* __restrict__ w, uint8_t* keep) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g < n) keep[g] = w[g] > 1e-106 ? 1 : 0;
}

__global__ void k_vee(int64_t n, const double* __restrict__ px, const double* __restrict__ py,
                      const double* __restrict__ pz, const double* __restrict__ w, double* wvee) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= n) return;
  const double d = sqrt(px[g] * px[g] + py[g] * py[g] + pz[g] * pz[g]);
  wvee[g] = w[g] * (1.0 / d);
}

// Radial-scan candidates (gridpoints2, mod_build_grid.f90:281-408).
struct ScanShell {
  double s;
  int ang_off, nang;
  int64_t first;  // first candidate index
};

__global__ void k_scan_candidates(int64_t ncand, const ScanShell* __restrict__ sh, int nsh,
                                  const double* __restrict__ lx, const double* __restrict__ ly,
                                  const double* __restrict__ lz, const double* __restrict__ lw, int nosym,
                                  double* ox, double* oy, double* oz, double* ow, int* oshell,
                                  uint8_t* keep) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= ncand) return;
  int lo = 0, hi = nsh - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (sh[mid].first <= g) lo = mid; else hi = mid - 1;
  }
  const ScanShell S = sh[lo];
  const int ia = static_cast<int>(g - S.first);
  const double tol = 1.4901161193847656e-08;  // sqrt(epsilon(1d0))
  const double z = S.s * lz[S.ang_off + ia];
  const bool k = nosym || z >= -tol;
  ox[g] = S.s * lx[S.ang_off + ia];
  oy[g] = S.s * ly[S.ang_off + ia];
  oz[g] = z;
  ow[g] = (nosym || fabs(z) < tol) ? lw[S.ang_off + ia] : 2.0 * lw[S.ang_off + ia];
  oshell[g] = lo;
  keep[g] = k ? 1 : 0;
}

// Points kept on each shell of a scan grid (its candidates' keep flags summed): one warp per shell.
__global__ void k_shell_counts(int nsh, const ScanShell* __restrict__ sh, const uint8_t* __restrict__ keep,
                               int* counts) {
  const int s = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (s >= nsh) return;
  const int lane = threadIdx.x & 31;
  const ScanShell S = sh[s];
  int k = 0;
  for (int i = lane; i < S.nang; i += 32) k += keep[S.first + i];
  for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
  if (lane == 0) counts[s] = k;
}

// Cube lattice (gridpoints3): x outer, y middle, z inner.
__global__ void k_cube(int64_t n, double x0, double y0, double z0, double sx, double sy, double sz,
                       int ny, int nz, double* ox, double* oy, double* oz) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= n) return;
  const int64_t k = g % nz, j = (g / nz) % ny, i = g / (static_cast<int64_t>(ny) * nz);
  ox[g] = x0 + sx * static_cast<double>(i);
  oy[g] = y0 + sy * static_cast<double>(j);
  oz[g] = z0 + sz * static_cast<double>(k);
}

// Segmented dot products sum_{i in [off_s, off_s+len_s)} a_i b_i, one block per segment,
// fixed-order block tree (deterministic). b may be null (then plain sums of a).
__global__ void k_seg_dot(int nseg, const int64_t* __restrict__ off, const double* __restrict__ a,
                          const double* __restrict__ b, const double* __restrict__ b2, double* out,
                          double* out2) {
  __shared__ double s1[256], s2[256];
  const int seg = blockIdx.x;
  if (seg >= nseg) return;
  const int64_t lo = off[seg], hi = off[seg + 1];
  double t1 = 0.0, t2 = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    t1 += a[i] * (b ? b[i] : 1.0);
    if (b2) t2 += a[i] * b2[i];
  }
  s1[threadIdx.x] = t1;
  s2[threadIdx.x] = t2;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[seg] = s1[0];
    if (out2) out2[seg] = s2[0];
  }
}

// Radial smearing, bin-parallel over points sorted by |r| (deterministic): bin j (0-based)
// receives the points whose reference window int((u-4s)/bw)+1 .. int((u+4s)/bw)+1 holds j+1.
__global__ void k_smear(int nbins, double bw, double sigma, int64_t n, const double* __restrict__ u,
                        const double* __restrict__ val, double* P) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nbins) return;
  const double uj = double(j) * bw;
  const double pref = 1.0 / (sigma * sqrt(2.0 * 3.141592653589793));
  const double lo_u = uj - 4.0 * sigma - 2.0 * bw, hi_u = uj + 4.0 * sigma + 2.0 * bw;
  int64_t lo = 0, hi = n;
  while (lo < hi) {  // first point with u >= lo_u
    const int64_t mid = (lo + hi) / 2;
    if (u[mid] < lo_u) lo = mid + 1; else hi = mid;
  }
  double acc = 0.0;
  for (int64_t i = lo; i < n && u[i] <= hi_u; ++i) {
    const int jmin = max(1, static_cast<int>((u[i] - 4.0 * sigma) / bw) + 1);
    const int jmax = min(nbins, static_cast<int>((u[i] + 4.0 * sigma) / bw) + 1);
    if (j + 1 < jmin || j + 1 > jmax) continue;
    const double dist = uj - u[i];
    acc += val[i] * (pref * exp(-(dist * dist) / (2.0 * sigma * sigma)));
  }
  P[j] = acc;
}

__global__ void k_smear_prep(int64_t n, const double* px, const double* py, const double* pz, const double* w,
                             const double* ivec, double* u, double* val) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= n) return;
  u[g] = sqrt(px[g] * px[g] + py[g] * py[g] + pz[g] * pz[g]);
  val[g] = w[g] * ivec[g];
}

inline unsigned nblk(int64_t n, int bs = 256) { return static_cast<unsigned>((n + bs - 1) / bs); }

// Stable compaction of (x, y, z, w, tag) by keep flags, into the context's grid arrays.
// Bump allocation over a context-owned device buffer: a dry run (base == nullptr) measures
// the bytes, the buffer grows to that (never shrinks), and the same sequence of take() calls
// carves it. The grid builders' temporaries live there, so rebuilding a grid allocates and
// frees nothing once the buffer is large enough.
struct Slab {
  unsigned char* base = nullptr;
  size_t off = 0;
  template <typename T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += n * sizeof(T);
    return p;
  }
};

// Temporaries of a grid build: candidate points, weights, tags, keep flags, the selected count
// and the stream-compaction's temporary storage.
struct Candidates {
  double *x, *y, *z, *w;
  int* tag;
  uint8_t* keep;
  int* nsel;
  unsigned char* tmp;
  size_t tmp_bytes;
};

// Carve the candidate arrays for ncand points (plus `extra`, which carves the caller's own
// tables from the same slab) out of the context's grid scratch.
template <typename Extra>
int carve_candidates(inca_ctx* c, int64_t ncand, Candidates& cd, Extra&& extra) {
  size_t tb = 0;
  cudaError_t e = cub::DeviceSelect::Flagged(nullptr, tb, static_cast<const double*>(nullptr),
                                             static_cast<const uint8_t*>(nullptr), static_cast<double*>(nullptr),
                                             static_cast<int*>(nullptr), ncand, c->stream);
  if (e) return cuda_error(c, e, "grid compaction");
  auto layout = [&](Slab& sl) {
    cd.x = sl.take<double>(ncand);
    cd.y = sl.take<double>(ncand);
    cd.z = sl.take<double>(ncand);
    cd.w = sl.take<double>(ncand);
    cd.tag = sl.take<int>(ncand);
    cd.keep = sl.take<uint8_t>(ncand);
    cd.nsel = sl.take<int>(1);
    cd.tmp = sl.take<unsigned char>(tb);
    cd.tmp_bytes = tb;
    extra(sl);
  };
  Slab dry;
  layout(dry);
  if (c->d_gscratch.reserve(dry.off + 256)) return set_error(c, INCA_E_NOMEM, "grid scratch");
  Slab sl{c->d_gscratch.p};
  layout(sl);
  return INCA_OK;
}

// Keep the flagged candidates (in order) as the context's grid arrays; *nout gets their count.
int compact_into(inca_ctx* c, int64_t ncand, const Candidates& cd, int64_t* nout) {
  if (c->d_px.reserve(ncand) || c->d_py.reserve(ncand) || c->d_pz.reserve(ncand) || c->d_w.reserve(ncand) ||
      c->d_wvee.reserve(ncand) || c->d_cmap.reserve(ncand))
    return set_error(c, INCA_E_NOMEM, "grid arrays");
  size_t tb = cd.tmp_bytes;
  cudaError_t e = cudaSuccess;
  double* outs[4] = {c->d_px.p, c->d_py.p, c->d_pz.p, c->d_w.p};
  const double* ins[4] = {cd.x, cd.y, cd.z, cd.w};
  for (int k = 0; k < 4 && e == cudaSuccess; ++k)
    e = cub::DeviceSelect::Flagged(cd.tmp, tb, ins[k], cd.keep, outs[k], cd.nsel, ncand, c->stream);
  if (e == cudaSuccess)
    e = cub::DeviceSelect::Flagged(cd.tmp, tb, cd.tag, cd.keep, c->d_cmap.p, cd.nsel, ncand, c->stream);
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, cd.nsel, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_error(c, e, "grid compaction");
  *nout = h;
  return INCA_OK;
}

}  // namespace

int grid_radial_device(inca_ctx* c, int nquad, const int* nradc, const int* nangc, const double* sfalpha,
                       const double* cent, const double* Ps, int nosym) {
  const double pi = 4.0 * std::atan(1.0);
  std::vector<RadialCentre> cen(nquad);
  std::vector<double> radius, wrad, lx, ly, lz, lw;
  int64_t ncand = 0;
  for (int q = 0; q < nquad; ++q) {
    if (nradc[q] < 1 || nangc[q] < 1) return set_error(c, INCA_E_ARG, "inca_grid_radial: nrad/nang must be >= 1");
    std::vector<double> x, y, z, w;
    if (lebedev_rule(nangc[q], x, y, z, w))
      return set_error(c, INCA_E_ARG, "inca_grid_radial: no Lebedev rule with " + std::to_string(nangc[q]) + " points");
    std::vector<double> t(nradc[q]), wl(nradc[q]);
    gauss_legendre(nradc[q], t.data(), wl.data());
    cen[q].cx = cent[3 * q];
    cen[q].cy = cent[3 * q + 1];
    cen[q].cz = cent[3 * q + 2];
    cen[q].nrad = nradc[q];
    cen[q].nang = nangc[q];
    cen[q].first = ncand;
    cen[q].rad_off = static_cast<int>(radius.size());
    cen[q].ang_off = static_cast<int>(lx.size());
    for (int ir = 0; ir < nradc[q]; ++ir) {
      const double r = (1.0 + t[ir]) / (1.0 - t[ir]) * sfalpha[q];
      double wr;
      if (nquad > 1 && r > 15.0)
        wr = 0.0;  // points beyond 15 bohr are dropped for multicentre grids (line 127)
      else
        wr = 2 * pi * (2.0 * sfalpha[q] / std::pow(1.0 - t[ir], 2.0)) * wl[ir] * r * r;
      radius.push_back(r);
      wrad.push_back(wr);
    }
    lx.insert(lx.end(), x.begin(), x.end());
    ly.insert(ly.end(), y.begin(), y.end());
    lz.insert(lz.end(), z.begin(), z.end());
    lw.insert(lw.end(), w.begin(), w.end());
    ncand += static_cast<int64_t>(nradc[q]) * nangc[q];
  }
  const size_t nlx = lx.size(), nrr = radius.size();
  RadialCentre* dcen = nullptr;
  double *drad = nullptr, *dwr = nullptr, *dlx = nullptr, *dly = nullptr, *dlz = nullptr, *dlw = nullptr;
  double *dR = nullptr, *dchi = nullptr, *dcent = nullptr;
  Candidates cd;
  int st = carve_candidates(c, ncand, cd, [&](Slab& sl) {
    dcen = sl.take<RadialCentre>(nquad);
    drad = sl.take<double>(nrr);
    dwr = sl.take<double>(nrr);
    dlx = sl.take<double>(nlx);
    dly = sl.take<double>(nlx);
    dlz = sl.take<double>(nlx);
    dlw = sl.take<double>(nlx);
    dR = sl.take<double>(static_cast<size_t>(nquad) * nquad);
    dchi = sl.take<double>(static_cast<size_t>(nquad) * nquad);
    dcent = sl.take<double>(3 * static_cast<size_t>(nquad));
  });
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(dcen, cen.data(), sizeof(RadialCentre) * nquad, cudaMemcpyHostToDevice, c->stream);
  if (!e) e = cudaMemcpyAsync(drad, radius.data(), sizeof(double) * nrr, cudaMemcpyHostToDevice, c->stream);
  if (!e) e = cudaMemcpyAsync(dwr, wrad.data(), sizeof(double) * nrr, cudaMemcpyHostToDevice, c->stream);
  if (!e) e = cudaMemcpyAsync(dlx, lx.data(), sizeof(double) * nlx, cudaMemcpyHostToDevice, c->stream);
  if (!e) e = cudaMemcpyAsync(dly, ly.data(), sizeof(double) * nlx, cudaMemcpyHostToDevice, c->stream);
  if (!e) e = cudaMemcpyAsync(dlz, lz.data(), sizeof(double) * nlx, cudaMemcpyHostToDevice, c->stream);
  if (!e) e = cudaMemcpyAsync(dlw, lw.data(), sizeof(double) * nlx, cudaMemcpyHostToDevice, c->stream);
  if (!e) {
    INCA_LAUNCH(c, k_radial_candidates, nblk(ncand), 256, 0, ncand, dcen, nquad, drad, dwr, dlx, dly, dlz, dlw,
                nosym, cd.x, cd.y, cd.z, cd.w, cd.tag, cd.keep);
    e = cudaGetLastError();
  }
  if (e) return cuda_error(c, e, "inca_grid_radial (candidates)");
  int64_t rgrid = 0;
  st = compact_into(c, ncand, cd, &rgrid);
  if (st) return st;
  int64_t ngrid = rgrid;
  if (nquad > 1) {
    std::vector<double> Rij(nquad * nquad), chi(nquad * nquad);
    for (int i = 0; i < nquad; ++i)
      for (int j = 0; j < nquad; ++j) {
        double s = 0;
        for (int d = 0; d < 3; ++d) s += std::pow(cent[3 * i + d] - cent[3 * j + d], 2.0);
        Rij[i * nquad + j] = std::sqrt(s);
        chi[i * nquad + j] = Ps[j] > 1e-12 ? std::pow(Ps[i] / Ps[j], 1.0 / 3.0) : 1.0;
      }
    e = cudaMemcpyAsync(dR, Rij.data(), sizeof(double) * Rij.size(), cudaMemcpyHostToDevice, c->stream);
    if (!e) e = cudaMemcpyAsync(dchi, chi.data(), sizeof(double) * chi.size(), cudaMemcpyHostToDevice, c->stream);
    if (!e) e = cudaMemcpyAsync(dcent, cent, sizeof(double) * 3 * nquad, cudaMemcpyHostToDevice, c->stream);
    if (!e) {
      const unsigned tb = nblk(rgrid, 128);
      INCA_LAUNCH(c, k_tfvc, tb, 128, 0, rgrid, c->d_px.p, c->d_py.p, c->d_pz.p, c->d_cmap.p, nquad, dcent, dR, dchi,
                  c->d_w.p);
      e = cudaGetLastError();
    }
    if (!e) {
      // copy the weighted grid back to candidates and drop weights <= 1e-106
      e = cudaMemcpyAsync(cd.x, c->d_px.p, sizeof(double) * rgrid, cudaMemcpyDeviceToDevice, c->stream);
      if (!e) e = cudaMemcpyAsync(cd.y, c->d_py.p, sizeof(double) * rgrid, cudaMemcpyDeviceToDevice, c->stream);
      if (!e) e = cudaMemcpyAsync(cd.z, c->d_pz.p, sizeof(double) * rgrid, cudaMemcpyDeviceToDevice, c->stream);
      if (!e) e = cudaMemcpyAsync(cd.w, c->d_w.p, sizeof(double) * rgrid, cudaMemcpyDeviceToDevice, c->stream);
      if (!e) e = cudaMemcpyAsync(cd.tag, c->d_cmap.p, sizeof(int) * rgrid, cudaMemcpyDeviceToDevice, c->stream);
      if (!e) {
        INCA_LAUNCH(c, k_weight_keep, nblk(rgrid), 256, 0, rgrid, cd.w, cd.keep);
        e = cudaGetLastError();
      }
    }
    if (e) return cuda_error(c, e, "inca_grid_radial (tfvc)");
    st = compact_into(c, rgrid, cd, &ngrid);
    if (st) return st;
  }
  INCA_LAUNCH(c, k_vee, nblk(ngrid), 256, 0, ngrid, c->d_px.p, c->d_py.p, c->d_pz.p, c->d_w.p, c->d_wvee.p);
  INCA_CUDA(c, cudaGetLastError());
  INCA_CUDA(c, cudaStreamSynchronize(c->stream));
  c->grid_kind = GRID_RADIAL;
  c->ngrid = ngrid;
  c->rgrid = rgrid;
  c->maxgrid = ncand;
  c->nquad = nquad;
  c->h_cent.assign(cent, cent + 3 * nquad);
  c->evaluated = false;
  ++c->grid_version;
  return INCA_OK;
}

int grid_scan_device(inca_ctx* c, int nblock, const double* start, const double* end, const double* step,
                     const int* nang, int nosym) {
  std::vector<ScanShell> sh;
  std::vector<double> lx, ly, lz, lw;
  std::vector<double> radi;
  int64_t ncand = 0;
  for (int b = 0; b < nblock; ++b) {
    if (!(step[b] > 0.0)) return set_error(c, INCA_E_ARG, "inca_grid_scan: step must be > 0");
    std::vector<double> x, y, z, w;
    if (lebedev_rule(nang[b], x, y, z, w))
      return set_error(c, INCA_E_ARG, "inca_grid_scan: no Lebedev rule with " + std::to_string(nang[b]) + " points");
    const int ang_off = static_cast<int>(lx.size());
    lx.insert(lx.end(), x.begin(), x.end());
    ly.insert(ly.end(), y.begin(), y.end());
    lz.insert(lz.end(), z.begin(), z.end());
    lw.insert(lw.end(), w.begin(), w.end());
    const int npb = static_cast<int>((end[b] - start[b]) / step[b]) + 1;
    for (int j = 0; j < npb; ++j) {
      ScanShell s;
      s.s = start[b] + step[b] * double(j);
      s.ang_off = ang_off;
      s.nang = nang[b];
      s.first = ncand;
      ncand += nang[b];
      sh.push_back(s);
      radi.push_back(s.s);
    }
  }
  const int nsh = static_cast<int>(sh.size());
  if (nsh == 0) return set_error(c, INCA_E_ARG, "inca_grid_scan: no shells");
  const size_t nlx = lx.size();
  ScanShell* dsh = nullptr;
  int* dcnt = nullptr;
  double *dlx = nullptr, *dly = nullptr, *dlz = nullptr, *dlw = nullptr;
  Candidates cd;
  int st = carve_candidates(c, ncand, cd, [&](Slab& sl) {
    dsh = sl.take<ScanShell>(nsh);
    dcnt = sl.take<int>(nsh);
    dlx = sl.take<double>(nlx);
    dly = sl.take<double>(nlx);
    dlz = sl.take<double>(nlx);
    dlw = sl.take<double>(nlx);
  });
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(dsh, sh.data(), sizeof(ScanShell) * nsh, cudaMemcpyHostToDevice, c->stream);
  if (!e) e = cudaMemcpyAsync(dlx, lx.data(), sizeof(double) * nlx, cudaMemcpyHostToDevice, c->stream);
  if (!e) e = cudaMemcpyAsync(dly, ly.data(), sizeof(double) * nlx, cudaMemcpyHostToDevice, c->stream);
  if (!e) e = cudaMemcpyAsync(dlz, lz.data(), sizeof(double) * nlx, cudaMemcpyHostToDevice, c->stream);
  if (!e) e = cudaMemcpyAsync(dlw, lw.data(), sizeof(double) * nlx, cudaMemcpyHostToDevice, c->stream);
  if (!e) {
    INCA_LAUNCH(c, k_scan_candidates, nblk(ncand), 256, 0, ncand, dsh, nsh, dlx, dly, dlz, dlw, nosym, cd.x, cd.y,
                cd.z, cd.w, cd.tag, cd.keep);
    INCA_LAUNCH(c, k_shell_counts, static_cast<unsigned>((nsh + 7) / 8), 256, 0, nsh, dsh, cd.keep, dcnt);
    e = cudaGetLastError();
  }
  if (e) return cuda_error(c, e, "inca_grid_scan");
  int64_t n = 0;
  st = compact_into(c, ncand, cd, &n);
  if (st) return st;
  // points per shell (counted on the device; the compaction above has synchronised the stream)
  c->h_smn.assign(nsh, 0);
  INCA_CUDA(c, cudaMemcpy(c->h_smn.data(), dcnt, sizeof(int) * nsh, cudaMemcpyDeviceToHost));
  c->h_radi = radi;
  c->nradi = nsh;
  c->grid_kind = GRID_SCAN;
  c->ngrid = n;
  c->rgrid = n;
  c->maxgrid = ncand;
  c->evaluated = false;
  ++c->grid_version;
  return INCA_OK;
}

int grid_cube_device(inca_ctx* c, const double* center, const double* step, const int* np) {
  double xm[3];
  for (int i = 0; i < 3; ++i) {
    if (np[i] < 1) return set_error(c, INCA_E_ARG, "inca_grid_cube: np must be >= 1");
    if (std::fmod(double(np[i]), 2.0) == 0.0)
      xm[i] = center[i] - (step[i] / 2.0) - ((double(np[i]) - 2.0) / 2.0) * step[i];
    else
      xm[i] = center[i] - ((double(np[i]) - 1.0) / 2.0) * step[i];
  }
  const int64_t n = static_cast<int64_t>(np[0]) * np[1] * np[2];
  if (c->d_px.reserve(n) || c->d_py.reserve(n) || c->d_pz.reserve(n))
    return set_error(c, INCA_E_NOMEM, "inca_grid_cube");
  INCA_LAUNCH(c, k_cube, nblk(n), 256, 0, n, xm[0], xm[1], xm[2], step[0], step[1], step[2], np[1], np[2], c->d_px.p,
                                         c->d_py.p, c->d_pz.p);
  INCA_CUDA(c, cudaGetLastError());
  INCA_CUDA(c, cudaStreamSynchronize(c->stream));
  c->grid_kind = GRID_CUBE;
  for (int i = 0; i < 3; ++i) c->cube_np[i] = np[i];
  c->ngrid = n;
  c->rgrid = n;
  c->maxgrid = n;
  c->evaluated = false;
  ++c->grid_version;
  return INCA_OK;
}

int radial_integral_device(inca_ctx* c, double* total, double* vee, double* per_c, double* vee_c) {
  if (c->grid_kind != GRID_RADIAL) return set_error(c, INCA_E_STATE, "inca_radial_integral: not a radial grid");
  if (!c->evaluated) return set_error(c, INCA_E_STATE, "inca_radial_integral: evaluate first");
  // points are centre-major: segment offsets from the centre tags
  std::vector<int> tags(c->ngrid);
  INCA_CUDA(c, cudaMemcpy(tags.data(), c->d_cmap.p, sizeof(int) * c->ngrid, cudaMemcpyDeviceToHost));
  std::vector<int64_t> off(c->nquad + 1, 0);
  for (int64_t i = 0; i < c->ngrid; ++i) off[tags[i] + 1]++;
  for (int q = 0; q < c->nquad; ++q) off[q + 1] += off[q];
  if (c->d_roff.reserve(c->nquad + 1) || c->d_rsum.reserve(2 * static_cast<size_t>(c->nquad)))
    return set_error(c, INCA_E_NOMEM, "radial integral");
  int64_t* doff = c->d_roff.p;
  double* o1 = c->d_rsum.p;
  double* o2 = c->d_rsum.p + c->nquad;
  cudaError_t e = cudaMemcpyAsync(doff, off.data(), sizeof(int64_t) * (c->nquad + 1), cudaMemcpyHostToDevice, c->stream);
  if (!e) {
    INCA_LAUNCH(c, k_seg_dot, c->nquad, 256, 0, c->nquad, doff, c->d_ivec.p, c->d_w.p, c->d_wvee.p, o1, o2);
    e = cudaGetLastError();
  }
  std::vector<double> h1(c->nquad), h2(c->nquad);
  if (!e) e = cudaMemcpyAsync(h1.data(), o1, sizeof(double) * c->nquad, cudaMemcpyDeviceToHost, c->stream);
  if (!e) e = cudaMemcpyAsync(h2.data(), o2, sizeof(double) * c->nquad, cudaMemcpyDeviceToHost, c->stream);
  if (!e) e = cudaStreamSynchronize(c->stream);
  if (e) return cuda_error(c, e, "radial integral");
  double t = 0, v = 0;
  for (int q = 0; q < c->nquad; ++q) {
    t += h1[q];
    v += h2[q];
    if (per_c) per_c[q] = h1[q];
    if (vee_c) vee_c[q] = h2[q];
  }
  if (total) *total = t;
  if (vee) *vee = v;
  return INCA_OK;
}

int radial_plot_device(inca_ctx* c, double* rintra) {
  if (c->grid_kind != GRID_SCAN) return set_error(c, INCA_E_STATE, "inca_radial_plot: not a scan grid");
  if (!c->evaluated) return set_error(c, INCA_E_STATE, "inca_radial_plot: evaluate first");
  const int ns = c->nradi;
  std::vector<int64_t> off(ns + 1, 0);
  for (int s = 0; s < ns; ++s) off[s + 1] = off[s] + c->h_smn[s];
  if (c->d_roff.reserve(ns + 1) || c->d_rsum.reserve(ns)) return set_error(c, INCA_E_NOMEM, "radial plot");
  cudaError_t e = cudaMemcpyAsync(c->d_roff.p, off.data(), sizeof(int64_t) * (ns + 1), cudaMemcpyHostToDevice, c->stream);
  if (!e) {
    INCA_LAUNCH(c, k_seg_dot, ns, 256, 0, ns, c->d_roff.p, c->d_ivec.p, c->d_w.p, nullptr, c->d_rsum.p, nullptr);
    e = cudaGetLastError();
  }
  if (!e) e = cudaMemcpyAsync(rintra, c->d_rsum.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, c->stream);
  if (!e) e = cudaStreamSynchronize(c->stream);
  if (e) return cuda_error(c, e, "radial plot");
  return INCA_OK;
}

int smearing_device(inca_ctx* c, double u_max, int n_bins, double sigma, double* u_axis, double* P_u, double* I_avg) {
  if (c->grid_kind != GRID_RADIAL) return set_error(c, INCA_E_STATE, "inca_radial_smearing: not a radial grid");
  if (!c->evaluated) return set_error(c, INCA_E_STATE, "inca_radial_smearing: evaluate first");
  if (n_bins < 2 || !(sigma > 0) || !(u_max > 0)) return set_error(c, INCA_E_ARG, "inca_radial_smearing: bad bins");
  const int64_t n = c->ngrid;
  DevBuf<double> u, val, u2, val2, P;
  DevBuf<unsigned char> tmp;
  auto rel = [&]() { u.release(); val.release(); u2.release(); val2.release(); P.release(); tmp.release(); };
  if (u.reserve(n) || val.reserve(n) || u2.reserve(n) || val2.reserve(n) || P.reserve(n_bins)) {
    rel();
    return set_error(c, INCA_E_NOMEM, "smearing");
  }
  INCA_LAUNCH(c, k_smear_prep, nblk(n), 256, 0, n, c->d_px.p, c->d_py.p, c->d_pz.p, c->d_w.p, c->d_ivec.p, u.p, val.p);
  cudaError_t e = cudaGetLastError();
  size_t tb = 0;
  if (!e) e = cub::DeviceRadixSort::SortPairs(nullptr, tb, u.p, u2.p, val.p, val2.p, n, 0, 64, c->stream);
  if (!e) e = tmp.reserve(tb);
  if (!e) e = cub::DeviceRadixSort::SortPairs(tmp.p, tb, u.p, u2.p, val.p, val2.p, n, 0, 64, c->stream);
  const double bw = u_max / double(n_bins - 1);
  if (!e) {
    INCA_LAUNCH(c, k_smear, (n_bins + 127) / 128, 128, 0, n_bins, bw, sigma, n, u2.p, val2.p, P.p);
    e = cudaGetLastError();
  }
  if (!e) e = cudaMemcpyAsync(P_u, P.p, sizeof(double) * n_bins, cudaMemcpyDeviceToHost, c->stream);
  if (!e) e = cudaStreamSynchronize(c->stream);
  rel();
  if (e) return cuda_error(c, e, "smearing");
  const double pi = 4.0 * std::atan(1.0);
  for (int j = 0; j < n_bins; ++j) {
    const double uj = double(j) * bw;
    if (u_axis) u_axis[j] = uj;
    if (I_avg) I_avg[j] = uj > 1e-6 ? P_u[j] * (1.0 / (4.0 * pi * uj * uj)) : 0.0;
  }
  return INCA_OK;
}

}  // namespace inca
