// C ABI of libinca_gpu.so (include/inca_gpu.h): context management, host<->device
// transfers, argument checking and dispatch to the kernels of the other translation units.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "inca_internal.h"

namespace inca {

int set_error(inca_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_error(inca_ctx* c, cudaError_t e, const char* what) {
  const int code = (e == cudaErrorMemoryAllocation) ? INCA_E_NOMEM : INCA_E_CUDA;
  return set_error(c, code, std::string(what) + ": " + cudaGetErrorString(e));
}

// dfact (src/mod_numbers.f90:14-28)
static long long dfact(int a) {
  long long r = 1;
  if (a % 2 == 0) {
    for (int i = 1; i <= a / 2; ++i) r *= 2 * i;
  } else {
    for (int i = 1; i <= (a + 1) / 2; ++i) r *= 2 * i - 1;
  }
  return r;
}

PrimD make_prim(double alpha, const int t[3], double x, double y, double z, int nprim_mol, int mol) {
  PrimD q;
  q.alpha = alpha;
  q.x = x;
  q.y = y;
  q.z = z;
  for (int d = 0; d < 3; ++d) q.t[d] = t[d];
  q.mol = mol;
  q.lim_scale = 1.0 / (double(nprim_mol) * (double(nprim_mol) + 1.0) * 0.5);
  // normprim (src/mod_intracule.f90:145-152)
  const double pi = 4.0 * std::atan(1.0);
  const int L = t[0] + t[1] + t[2];
  const double df = double(dfact(2 * t[0] - 1) * dfact(2 * t[1] - 1) * dfact(2 * t[2] - 1));
  q.norm = std::pow(2.0 * alpha / pi, 0.75) * std::sqrt(std::pow(4.0 * alpha, double(L)) * (1.0 / df));
  return q;
}

}  // namespace inca

using namespace inca;

extern "C" {

int inca_abi_version(void) { return INCA_ABI_VERSION; }

int inca_ctx_create(inca_ctx** out, int device) {
  if (!out) return INCA_E_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return INCA_E_CUDA;
  if (device < 0 || device >= ndev) return INCA_E_ARG;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return INCA_E_CUDA;
  if (prop.major != 10 || prop.minor != 3) return INCA_E_CUDA;  // built for sm_103a only
  if (cudaSetDevice(device) != cudaSuccess) return INCA_E_CUDA;
  inca_ctx* c = new inca_ctx();
  c->device = device;
  c->num_sms = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return INCA_E_CUDA;
  }
  *out = c;
  return INCA_OK;
}

int inca_ctx_destroy(inca_ctx* c) {
  if (!c) return INCA_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  c->d_prims.release();
  c->d_ijkl.release();
  c->d_v.release();
  c->d_flags.release();
  c->d_ja8.release();
  c->d_s1.release();
  c->d_s2.release();
  c->d_pkey.release();
  c->d_pkey2.release();
  c->d_pukeys.release();
  c->d_pidx.release();
  c->d_pidx2.release();
  c->d_pucounts.release();
  c->d_ptmp.release();
  c->d_pbad.release();
  c->d_pnruns.release();
  c->d_pn1.release();
  c->d_pqrec.release();
  c->d_roff.release();
  c->d_rsum.release();
  c->d_classes.release();
  c->d_chunks.release();
  c->d_rec64.release();
  c->d_rec32.release();
  c->d_surv_src.release();
  c->d_px.release();
  c->d_py.release();
  c->d_pz.release();
  c->d_w.release();
  c->d_wvee.release();
  c->d_cmap.release();
  c->d_ivec.release();
  c->d_partial.release();
  c->d_scratch.release();
  c->d_phi.release();
  c->d_plo.release();
  c->d_perm.release();
  c->d_wtbox.release();
  c->d_phi_s.release();
  c->d_plo_s.release();
  c->d_perm_s.release();
  c->d_wtbox_s.release();
  c->d_scratch_s.release();
  c->d_tiles.release();
  c->d_tiles_s.release();
  c->d_exptab.release();
  c->d_pmol.release();
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  c->graph_exec = nullptr;
  cudaStreamDestroy(c->stream);
  delete c;
  return INCA_OK;
}

const char* inca_last_error(const inca_ctx* c) { return c ? c->err.c_str() : "null context"; }

#define CTX_CHECK(c)                   \
  do {                                 \
    if (!(c)) return INCA_E_ARG;       \
    cudaSetDevice((c)->device);        \
  } while (0)

int inca_set_primitives(inca_ctx* c, int32_t nprim, const double* alpha, const int32_t* tmn, const double* xn,
                        const double* yn, const double* zn) {
  CTX_CHECK(c);
  if (nprim <= 0 || !alpha || !tmn || !xn || !yn || !zn)
    return set_error(c, INCA_E_ARG, "inca_set_primitives: bad arguments");
  std::vector<PrimD> h(nprim);
  c->h_alpha.assign(alpha, alpha + nprim);
  c->h_x.assign(xn, xn + nprim);
  c->h_y.assign(yn, yn + nprim);
  c->h_z.assign(zn, zn + nprim);
  c->h_tmn.assign(3 * static_cast<size_t>(nprim), 0);
  for (int p = 0; p < nprim; ++p) {
    if (!(alpha[p] > 0.0)) return set_error(c, INCA_E_ARG, "inca_set_primitives: exponent <= 0 or NaN at primitive " + std::to_string(p + 1));
    int t[3];
    for (int d = 0; d < 3; ++d) {
      t[d] = tmn[p + static_cast<size_t>(nprim) * d];  // TMN(nprim,3), column-major
      if (t[d] < 0) return set_error(c, INCA_E_ARG, "inca_set_primitives: negative Cartesian power");
      c->h_tmn[3 * p + d] = t[d];
    }
    h[p] = make_prim(alpha[p], t, xn[p], yn[p], zn[p], nprim, 0);
  }
  if (c->d_prims.reserve(nprim)) return set_error(c, INCA_E_NOMEM, "primitives");
  INCA_CUDA(c, cudaMemcpyAsync(c->d_prims.p, h.data(), sizeof(PrimD) * nprim, cudaMemcpyHostToDevice, c->stream));
  INCA_CUDA(c, cudaStreamSynchronize(c->stream));
  c->nprim = nprim;
  c->batch_molecules = 0;
  c->prepared = false;
  c->evaluated = false;
  return INCA_OK;
}

// ijkl: n records of four 1-based int32 indices, the layout of the device's int4 array, so both
// arrays go to the device in one copy each straight from the caller's memory (a direct DMA when
// the caller's buffers are pinned).
static int upload_quartets(inca_ctx* c, int64_t n, const int32_t* ijkl, const double* v) {
  if (c->d_ijkl.reserve(std::max<int64_t>(n, 1)) || c->d_v.reserve(std::max<int64_t>(n, 1)))
    return set_error(c, INCA_E_NOMEM, "quartets");
  if (n > 0) {
    INCA_CUDA(c, cudaMemcpyAsync(c->d_ijkl.p, ijkl, sizeof(int4) * n, cudaMemcpyHostToDevice, c->stream));
    INCA_CUDA(c, cudaMemcpyAsync(c->d_v.p, v, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  c->nq = n;
  c->prepared = false;
  c->evaluated = false;
  return INCA_OK;
}

int inca_load_dm2p(inca_ctx* c, const char* path, int64_t* nread) {
  CTX_CHECK(c);
  if (!path) return set_error(c, INCA_E_ARG, "inca_load_dm2p: null path");
  if (c->nprim <= 0) return set_error(c, INCA_E_STATE, "inca_load_dm2p: set the primitives first");
  std::vector<int4> q;
  std::vector<double> v;
  std::string err;
  const int st = read_dm2p(path, c->nprim, q, v, err);
  if (st) return set_error(c, st, err);
  if (nread) *nread = static_cast<int64_t>(v.size());
  static_assert(sizeof(int4) == 4 * sizeof(int32_t), "int4 holds four int32 indices");
  return upload_quartets(c, static_cast<int64_t>(v.size()), reinterpret_cast<const int32_t*>(q.data()), v.data());
}

int inca_read_dm2p(const char* path, int32_t nprim, int64_t capacity, int32_t* ijkl, double* v, int64_t* nread,
                   char* errbuf, int32_t errlen) {
  if (errbuf && errlen > 0) errbuf[0] = '\0';
  if (!path || nprim <= 0 || capacity < 0 || !nread) return INCA_E_ARG;
  std::vector<int4> q;
  std::vector<double> vv;
  std::string err;
  const int st = read_dm2p(path, nprim, q, vv, err);
  if (st) {
    if (errbuf && errlen > 0) {
      std::strncpy(errbuf, err.c_str(), static_cast<size_t>(errlen) - 1);
      errbuf[errlen - 1] = '\0';
    }
    return st;
  }
  const int64_t n = static_cast<int64_t>(vv.size());
  *nread = n;
  if (!ijkl || !v) return INCA_OK;  // count only
  if (n > capacity) return INCA_E_LIMIT;
  std::memcpy(ijkl, q.data(), sizeof(int4) * static_cast<size_t>(n));
  std::memcpy(v, vv.data(), sizeof(double) * static_cast<size_t>(n));
  return INCA_OK;
}

int inca_set_quartets(inca_ctx* c, int64_t n, const int32_t* ijkl, const double* v) {
  CTX_CHECK(c);
  if (n < 0 || (n > 0 && (!ijkl || !v))) return set_error(c, INCA_E_ARG, "inca_set_quartets: bad arguments");
  return upload_quartets(c, n, ijkl, v);
}

int inca_gen_closed_shell_dm2(inca_ctx* c, const double* D, int unique, int64_t* nrecords) {
  CTX_CHECK(c);
  return gen_closed_shell_device(c, D, unique, nrecords);
}

int inca_prepare(inca_ctx* c, double thresh, int normalize, inca_counts* counts) {
  CTX_CHECK(c);
  const int st = prepare_device(c, thresh, normalize);
  if (st == INCA_OK && counts) *counts = c->counts;
  return st;
}

int inca_get_screening(inca_ctx* c, uint8_t* flags, double* s1, double* s2) {
  CTX_CHECK(c);
  if (!c->prepared) return set_error(c, INCA_E_STATE, "inca_get_screening: call inca_prepare first");
  if ((s1 || s2) && !c->have_screen_values)
    return set_error(c, INCA_E_LIMIT, "inca_get_screening: screening values kept only for <= 2^27 quartets");
  if (flags) INCA_CUDA(c, cudaMemcpy(flags, c->d_flags.p, c->nq, cudaMemcpyDeviceToHost));
  if (s1) INCA_CUDA(c, cudaMemcpy(s1, c->d_s1.p, sizeof(double) * c->nq, cudaMemcpyDeviceToHost));
  if (s2) INCA_CUDA(c, cudaMemcpy(s2, c->d_s2.p, sizeof(double) * c->nq, cudaMemcpyDeviceToHost));
  return INCA_OK;
}

int inca_get_records(inca_ctx* c, double* A, double* sqe, double* d, int32_t* L, double* C) {
  CTX_CHECK(c);
  if (!c->prepared) return set_error(c, INCA_E_STATE, "inca_get_records: call inca_prepare first");
  const int64_t ns = c->nsurv;
  if (ns == 0) return INCA_OK;
  int64_t total = 0;
  for (const ClassSeg& s : c->classes) total = std::max<int64_t>(total, s.off64 + s.count * s.stride);
  std::vector<double> rec(total);
  std::vector<int64_t> src(ns);
  INCA_CUDA(c, cudaMemcpy(rec.data(), c->d_rec64.p, sizeof(double) * total, cudaMemcpyDeviceToHost));
  INCA_CUDA(c, cudaMemcpy(src.data(), c->d_surv_src.p, sizeof(int64_t) * ns, cudaMemcpyDeviceToHost));
  // survivors in input order: rank of each sorted survivor by its source index
  std::vector<int64_t> order(ns);
  for (int64_t i = 0; i < ns; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return src[a] < src[b]; });
  std::vector<int64_t> rank(ns);
  for (int64_t r = 0; r < ns; ++r) rank[order[r]] = r;
  for (const ClassSeg& s : c->classes)
    for (int64_t k = 0; k < s.count; ++k) {
      const double* R = rec.data() + s.off64 + k * s.stride;
      const int64_t o = rank[s.first + k];
      if (A) A[o] = R[0];
      if (sqe) sqe[o] = R[1];
      if (d)
        for (int j = 0; j < 3; ++j) d[3 * o + j] = R[2 + j];
      if (L)
        for (int j = 0; j < 3; ++j) L[3 * o + j] = s.L[j];
      if (C) {
        int p = kRecHeader;
        for (int j = 0; j < 3; ++j) {
          for (int m = 0; m < kMaxCoef; ++m) C[(3 * o + j) * kMaxCoef + m] = m <= s.L[j] ? R[p + m] : 0.0;
          p += s.L[j] + 1;
        }
      }
    }
  return INCA_OK;
}

int inca_grid_radial(inca_ctx* c, int32_t nquad, const int32_t* nradc, const int32_t* nangc, const double* sfalpha,
                     const double* cent, const double* Ps, int nosym, int64_t* maxgrid, int64_t* rgrid,
                     int64_t* ngrid) {
  CTX_CHECK(c);
  if (nquad < 1 || !nradc || !nangc || !sfalpha || !cent || !Ps)
    return set_error(c, INCA_E_ARG, "inca_grid_radial: bad arguments");
  const int st = grid_radial_device(c, nquad, nradc, nangc, sfalpha, cent, Ps, nosym);
  if (st) return st;
  if (maxgrid) *maxgrid = c->maxgrid;
  if (rgrid) *rgrid = c->rgrid;
  if (ngrid) *ngrid = c->ngrid;
  return INCA_OK;
}

int inca_grid_scan(inca_ctx* c, int32_t nblock, const double* start, const double* end, const double* step,
                   const int32_t* nang, int nosym, int32_t* nradi, int64_t* ngrid) {
  CTX_CHECK(c);
  if (nblock < 1 || !start || !end || !step || !nang) return set_error(c, INCA_E_ARG, "inca_grid_scan: bad arguments");
  const int st = grid_scan_device(c, nblock, start, end, step, nang, nosym);
  if (st) return st;
  if (nradi) *nradi = c->nradi;
  if (ngrid) *ngrid = c->ngrid;
  return INCA_OK;
}

int inca_grid_cube(inca_ctx* c, const double* center, const double* step, const int32_t* np, int64_t* ngrid) {
  CTX_CHECK(c);
  if (!center || !step || !np) return set_error(c, INCA_E_ARG, "inca_grid_cube: bad arguments");
  const int st = grid_cube_device(c, center, step, np);
  if (st) return st;
  if (ngrid) *ngrid = c->ngrid;
  return INCA_OK;
}

int inca_grid_points(inca_ctx* c, int64_t n, const double* r) {
  CTX_CHECK(c);
  if (n < 1 || !r) return set_error(c, INCA_E_ARG, "inca_grid_points: bad arguments");
  std::vector<double> x(n), y(n), z(n);
  for (int64_t i = 0; i < n; ++i) {
    x[i] = r[3 * i];
    y[i] = r[3 * i + 1];
    z[i] = r[3 * i + 2];
  }
  if (c->d_px.reserve(n) || c->d_py.reserve(n) || c->d_pz.reserve(n)) return set_error(c, INCA_E_NOMEM, "points");
  INCA_CUDA(c, cudaMemcpyAsync(c->d_px.p, x.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  INCA_CUDA(c, cudaMemcpyAsync(c->d_py.p, y.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  INCA_CUDA(c, cudaMemcpyAsync(c->d_pz.p, z.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  INCA_CUDA(c, cudaStreamSynchronize(c->stream));
  c->grid_kind = GRID_POINTS;
  c->ngrid = c->rgrid = c->maxgrid = n;
  c->evaluated = false;
  ++c->grid_version;
  return INCA_OK;
}

int inca_grid_copy(inca_ctx* c, double* r, double* w, double* wvee, int32_t* cmap) {
  CTX_CHECK(c);
  if (c->grid_kind == GRID_NONE) return set_error(c, INCA_E_STATE, "inca_grid_copy: no grid");
  const int64_t n = c->ngrid;
  if (r) {
    std::vector<double> x(n), y(n), z(n);
    INCA_CUDA(c, cudaMemcpy(x.data(), c->d_px.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    INCA_CUDA(c, cudaMemcpy(y.data(), c->d_py.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    INCA_CUDA(c, cudaMemcpy(z.data(), c->d_pz.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < n; ++i) {
      r[3 * i] = x[i];
      r[3 * i + 1] = y[i];
      r[3 * i + 2] = z[i];
    }
  }
  const bool weighted = c->grid_kind == GRID_RADIAL || c->grid_kind == GRID_SCAN;
  if (w) {
    if (!weighted) return set_error(c, INCA_E_STATE, "inca_grid_copy: grid has no weights");
    INCA_CUDA(c, cudaMemcpy(w, c->d_w.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  }
  if (wvee) {
    if (c->grid_kind != GRID_RADIAL) return set_error(c, INCA_E_STATE, "inca_grid_copy: not a radial grid");
    INCA_CUDA(c, cudaMemcpy(wvee, c->d_wvee.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
  }
  if (cmap) {
    if (!weighted) return set_error(c, INCA_E_STATE, "inca_grid_copy: grid has no centre map");
    INCA_CUDA(c, cudaMemcpy(cmap, c->d_cmap.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < n; ++i) cmap[i] += 1;
  }
  return INCA_OK;
}

int inca_eval(inca_ctx* c, int mode, double tol, double* ivec) {
  CTX_CHECK(c);
  const int st = eval_device(c, mode, tol);
  if (st) return st;
  if (ivec) {
    INCA_CUDA(c, cudaMemcpyAsync(ivec, c->d_ivec.p, sizeof(double) * c->ngrid, cudaMemcpyDeviceToHost, c->stream));
    INCA_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return INCA_OK;
}

int inca_autotune(inca_ctx* c, double tol, int32_t reps, inca_tuning* chosen) {
  CTX_CHECK(c);
  if (!c->prepared) return set_error(c, INCA_E_STATE, "inca_autotune: call inca_prepare first");
  if (c->grid_kind == GRID_NONE || c->ngrid <= 0) return set_error(c, INCA_E_STATE, "inca_autotune: no grid");
  if (c->d_ivec.reserve(c->ngrid)) return set_error(c, INCA_E_NOMEM, "ivec");
  int ipc = 0, stride = 0, ctas = 0, slack = 0, ppt = 0;
  double safety = 0, drop = 0, best = 0, dflt = 0;
  const int st = autotune_mixed(c, tol > 0 ? tol : 1e-10, std::max(1, reps), &ipc, &stride, &safety, &drop, &ctas,
                                &slack, &ppt, &best, &dflt);
  if (st) return st;
  c->evaluated = true;
  if (chosen) {
    chosen->items_per_cta = ipc;
    chosen->sample_stride = stride;
    chosen->estimate_safety = safety;
    chosen->drop_fraction = drop;
    chosen->ctas_per_sm = ctas;
    chosen->cheap_slack = slack;
    chosen->points_per_lane = ppt;
    chosen->best_ms = best;
    chosen->default_ms = dflt;
  }
  return INCA_OK;
}

int inca_set_tuning(inca_ctx* c, const inca_tuning* t) {
  CTX_CHECK(c);
  if (t && (t->items_per_cta < 1 || t->items_per_cta > 1024 || t->sample_stride < 1 || t->sample_stride > 1024 ||
            !(t->estimate_safety >= 0.0) || !(t->drop_fraction < 0.5) ||
            !valid_pass_shape(t->points_per_lane ? t->points_per_lane : 4,
                              t->ctas_per_sm ? t->ctas_per_sm : 16) ||
            t->cheap_slack < 0 || t->cheap_slack > 30))
    return set_error(c, INCA_E_ARG, "inca_set_tuning: bad values");
  c->tune_items_per_cta = t ? t->items_per_cta : 0;
  c->tune_sample_stride = t ? t->sample_stride : 0;
  c->tune_safety = t ? t->estimate_safety : -1.0;
  c->tune_drop = t ? t->drop_fraction : -1.0;
  c->tune_ctas = t ? t->ctas_per_sm : 0;
  c->tune_cheap_slack = t ? t->cheap_slack : -1;
  c->tune_ppt = t ? t->points_per_lane : 0;
  return INCA_OK;
}

int inca_eval_graph(inca_ctx* c, int mode, double tol, double* ivec) {
  CTX_CHECK(c);
  const int st = eval_device(c, mode, tol, true);
  if (st) return st;
  if (ivec) INCA_CUDA(c, cudaMemcpy(ivec, c->d_ivec.p, sizeof(double) * c->ngrid, cudaMemcpyDeviceToHost));
  return INCA_OK;
}

int inca_radial_integral(inca_ctx* c, double* total, double* vee, double* per_centre, double* vee_per_centre) {
  CTX_CHECK(c);
  return radial_integral_device(c, total, vee, per_centre, vee_per_centre);
}

int inca_radial_plot(inca_ctx* c, double* radi, double* rintra) {
  CTX_CHECK(c);
  if (c->grid_kind != GRID_SCAN) return set_error(c, INCA_E_STATE, "inca_radial_plot: not a scan grid");
  if (radi) std::copy(c->h_radi.begin(), c->h_radi.end(), radi);
  if (!rintra) return INCA_OK;
  return radial_plot_device(c, rintra);
}

int inca_radial_smearing(inca_ctx* c, double u_max, int32_t n_bins, double sigma, double* u_axis, double* P_u,
                         double* I_avg) {
  CTX_CHECK(c);
  if (!P_u) return set_error(c, INCA_E_ARG, "inca_radial_smearing: P_u is null");
  return smearing_device(c, u_max, n_bins, sigma, u_axis, P_u, I_avg);
}

int inca_last_eval_timing(inca_ctx* c, double* total_ms, double* kernel_ms, int32_t* kernel_launches,
                          int32_t* launches) {
  if (!c) return INCA_E_ARG;
  if (total_ms) *total_ms = c->t_total_ms;
  if (kernel_ms) *kernel_ms = c->t_kernel_ms;
  if (kernel_launches) *kernel_launches = c->t_kernel_launches;
  if (launches) *launches = c->t_launches;
  return INCA_OK;
}

int inca_last_eval_stats(inca_ctx* c, int64_t* fp32_pairs, int64_t* precise_pairs, int64_t* skipped_pairs,
                         int64_t* corrected_terms) {
  if (!c) return INCA_E_ARG;
  if (fp32_pairs) *fp32_pairs = c->pairs_fp32;
  if (precise_pairs) *precise_pairs = c->pairs_fp64;
  if (skipped_pairs) *skipped_pairs = c->pairs_skip;
  if (corrected_terms) *corrected_terms = c->corrected_points;
  return INCA_OK;
}

int inca_last_eval_cheap_pairs(inca_ctx* c, int64_t* cheap_pairs) {
  if (!c) return INCA_E_ARG;
  if (cheap_pairs) *cheap_pairs = c->pairs_cheap;
  return INCA_OK;
}

int inca_last_eval_phases(inca_ctx* c, double* pass1_ms, double* pass2_ms) {
  if (!c) return INCA_E_ARG;
  if (pass1_ms) *pass1_ms = c->t_kernel_ms;
  if (pass2_ms) *pass2_ms = c->t_pass2_ms;
  return INCA_OK;
}

int inca_get_stream(inca_ctx* c, void** stream) {
  if (!c || !stream) return INCA_E_ARG;
  *stream = reinterpret_cast<void*>(c->stream);
  return INCA_OK;
}

int inca_kernel_launches(inca_ctx* c, int64_t* count) {
  if (!c || !count) return INCA_E_ARG;
  *count = c->launches;
  return INCA_OK;
}

}  // extern "C"
