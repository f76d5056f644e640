// Batches of molecules evaluated together: one screening pass over all their quartets and one
// launch of each evaluation kernel for all their grid points. No counterpart in the reference,
// which runs calculate_intracule (src/mod_intracule.f90:18-572) once per molecule and
// process; a batch runs its radial_plot job (lines 512-533) for every molecule at once.
//
// Layout: the molecules' primitives are concatenated (each primitive carries its molecule and
// that molecule's screening scale 1/(nprim(nprim+1)/2)); their DM2 records are generated into
// one quartet list with global primitive indices; the survivors are sorted by (molecule, angular
// class), so each molecule owns a contiguous range of work chunks; the scan grids are
// concatenated (shell tags offset per molecule), sorted by (molecule, Morton key), and cut into
// tiles that never straddle two molecules. Every evaluation kernel then pairs each tile with
// its own molecule's chunk range.
#include <algorithm>
#include <cmath>
#include <string>
#include <type_traits>
#include <vector>

#include "inca_internal.h"

namespace inca {

int prepare_device(inca_ctx* c, double thresh, int normalize);
int radial_plot_device(inca_ctx* c, double* rintra);

namespace {

__global__ void k_shift_fill(int64_t n, const int* __restrict__ src, int shift, int* dst, int mol, int* dmol) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  dst[i] = src[i] + shift;
  dmol[i] = mol;
}

}  // namespace

int batch_prepare(inca_ctx* c, double thresh, inca_counts* counts) {
  const int nmol = static_cast<int>(c->batch.size());
  if (nmol == 0) return set_error(c, INCA_E_STATE, "inca_batch_prepare: no molecules added");
  if (!(thresh > 0.0)) return set_error(c, INCA_E_ARG, "inca_batch_prepare: thresh must be > 0");
  // primitives
  int np = 0;
  for (const BatchMol& m : c->batch) np += m.nprim;
  std::vector<PrimD> h(np);
  c->h_alpha.clear(); c->h_x.clear(); c->h_y.clear(); c->h_z.clear();
  c->h_tmn.assign(3 * static_cast<size_t>(np), 0);
  std::vector<int> base(nmol);
  int o = 0;
  for (int mi = 0; mi < nmol; ++mi) {
    const BatchMol& m = c->batch[mi];
    base[mi] = o;
    for (int p = 0; p < m.nprim; ++p) {
      const int t[3] = {m.tmn[3 * p], m.tmn[3 * p + 1], m.tmn[3 * p + 2]};
      h[o + p] = make_prim(m.alpha[p], t, m.x[p], m.y[p], m.z[p], m.nprim, mi);
      for (int d = 0; d < 3; ++d) c->h_tmn[3 * (o + p) + d] = t[d];
      c->h_alpha.push_back(m.alpha[p]);
      c->h_x.push_back(m.x[p]);
      c->h_y.push_back(m.y[p]);
      c->h_z.push_back(m.z[p]);
    }
    o += m.nprim;
  }
  if (c->d_prims.reserve(np)) return set_error(c, INCA_E_NOMEM, "batch primitives");
  INCA_CUDA(c, cudaMemcpyAsync(c->d_prims.p, h.data(), sizeof(PrimD) * np, cudaMemcpyHostToDevice, c->stream));
  c->nprim = np;
  // DM2 records, one molecule after the other
  int64_t nrec = 0;
  for (const BatchMol& m : c->batch) nrec += closed_shell_records(m.nprim, m.unique);
  if (c->d_ijkl.reserve(nrec) || c->d_v.reserve(nrec)) return set_error(c, INCA_E_NOMEM, "batch quartet records");
  int64_t at = 0;
  for (int mi = 0; mi < nmol; ++mi) {
    const BatchMol& m = c->batch[mi];
    const int st = gen_closed_shell_into(c, m.nprim, m.D.data(), m.unique, base[mi], at);
    if (st) return st;
    at += closed_shell_records(m.nprim, m.unique);
  }
  c->nq = nrec;
  c->batch_molecules = nmol;
  int st = prepare_device(c, thresh, 1);
  if (st) return st;
  if (counts) *counts = c->counts;
  // grids: each molecule's scan grid, concatenated
  std::vector<int64_t> moff(nmol + 1, 0);
  std::vector<int> shoff(nmol + 1, 0);
  std::vector<int> smn;
  std::vector<double> radi;
  DevBuf<double> bx, by, bz, bw;
  DevBuf<int> bc, bm;
  auto rel = [&]() { bx.release(); by.release(); bz.release(); bw.release(); bc.release(); bm.release(); };
  for (int mi = 0; mi < nmol; ++mi) {
    const BatchMol& m = c->batch[mi];
    st = grid_scan_device(c, static_cast<int>(m.start.size()), m.start.data(), m.end.data(), m.step.data(),
                          m.nang.data(), m.nosym);
    if (st) {
      rel();
      return st;
    }
    const int64_t n = c->ngrid, o0 = moff[mi];
    moff[mi + 1] = o0 + n;
    shoff[mi + 1] = shoff[mi] + c->nradi;
    // grow the concatenation buffers (copying what they hold)
    auto grow = [&](auto& buf, int64_t want) -> cudaError_t {
      using T = std::remove_reference_t<decltype(*buf.p)>;
      if (static_cast<size_t>(want) <= buf.n) return cudaSuccess;
      DevBuf<T> nb;
      cudaError_t e = nb.reserve(std::max<int64_t>(want, 2 * static_cast<int64_t>(buf.n)));
      if (!e && o0 > 0) e = cudaMemcpyAsync(nb.p, buf.p, sizeof(T) * o0, cudaMemcpyDeviceToDevice, c->stream);
      if (!e) e = cudaStreamSynchronize(c->stream);
      buf.release();
      buf.p = nb.p;
      buf.n = nb.n;
      return e;
    };
    cudaError_t e = grow(bx, o0 + n);
    if (!e) e = grow(by, o0 + n);
    if (!e) e = grow(bz, o0 + n);
    if (!e) e = grow(bw, o0 + n);
    if (!e) e = grow(bc, o0 + n);
    if (!e) e = grow(bm, o0 + n);
    if (!e) e = cudaMemcpyAsync(bx.p + o0, c->d_px.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream);
    if (!e) e = cudaMemcpyAsync(by.p + o0, c->d_py.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream);
    if (!e) e = cudaMemcpyAsync(bz.p + o0, c->d_pz.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream);
    if (!e) e = cudaMemcpyAsync(bw.p + o0, c->d_w.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream);
    if (!e && n > 0) {
      INCA_LAUNCH(c, k_shift_fill, static_cast<unsigned>((n + 255) / 256), 256, 0, n, c->d_cmap.p, shoff[mi],
                  bc.p + o0, mi, bm.p + o0);
      e = cudaGetLastError();
    }
    if (!e) e = cudaStreamSynchronize(c->stream);
    if (e) {
      rel();
      return cuda_error(c, e, "batch grids");
    }
    smn.insert(smn.end(), c->h_smn.begin(), c->h_smn.end());
    radi.insert(radi.end(), c->h_radi.begin(), c->h_radi.end());
  }
  // the batch grid replaces the context's grid
  auto take = [](auto& dst, auto& src) {
    dst.release();
    dst.p = src.p;
    dst.n = src.n;
    src.p = nullptr;
    src.n = 0;
  };
  take(c->d_px, bx);
  take(c->d_py, by);
  take(c->d_pz, bz);
  take(c->d_w, bw);
  take(c->d_cmap, bc);
  take(c->d_pmol, bm);
  c->h_smn = smn;
  c->h_radi = radi;
  c->nradi = shoff[nmol];
  c->ngrid = moff[nmol];
  c->rgrid = c->ngrid;
  c->maxgrid = c->ngrid;
  c->grid_kind = GRID_SCAN;
  c->h_mol_off = moff;
  c->h_mol_shell_off = shoff;
  ++c->grid_version;
  c->batch_grid_version = c->grid_version;
  c->evaluated = false;
  return INCA_OK;
}

}  // namespace inca

using namespace inca;

#define CTX_CHECK(c)             \
  do {                           \
    if (!(c)) return INCA_E_ARG; \
    cudaSetDevice((c)->device);  \
  } while (0)

extern "C" {

int inca_batch_clear(inca_ctx* c) {
  CTX_CHECK(c);
  c->batch.clear();
  return INCA_OK;
}

int inca_batch_add_closed_shell(inca_ctx* c, int32_t nprim, const double* alpha, const int32_t* tmn,
                                const double* xn, const double* yn, const double* zn, const double* D, int unique,
                                int32_t nblock, const double* start, const double* end, const double* step,
                                const int32_t* nang, int nosym, int32_t* nradi) {
  CTX_CHECK(c);
  if (nprim <= 0 || !alpha || !tmn || !xn || !yn || !zn || !D || nblock < 1 || !start || !end || !step || !nang)
    return set_error(c, INCA_E_ARG, "inca_batch_add_closed_shell: bad arguments");
  if (static_cast<int>(c->batch.size()) >= INCA_MAX_BATCH)
    return set_error(c, INCA_E_LIMIT, "inca_batch_add_closed_shell: more than INCA_MAX_BATCH molecules");
  BatchMol m;
  m.nprim = nprim;
  m.alpha.assign(alpha, alpha + nprim);
  m.x.assign(xn, xn + nprim);
  m.y.assign(yn, yn + nprim);
  m.z.assign(zn, zn + nprim);
  m.tmn.assign(3 * static_cast<size_t>(nprim), 0);
  for (int p = 0; p < nprim; ++p) {
    if (!(alpha[p] > 0.0)) return set_error(c, INCA_E_ARG, "inca_batch_add_closed_shell: exponent <= 0");
    for (int d = 0; d < 3; ++d) {
      const int t = tmn[p + static_cast<size_t>(nprim) * d];  // TMN(nprim,3), column-major
      if (t < 0 || t > 4) return set_error(c, INCA_E_LIMIT, "inca_batch_add_closed_shell: Cartesian power outside 0..4");
      m.tmn[3 * p + d] = t;
    }
  }
  m.D.assign(D, D + static_cast<size_t>(nprim) * nprim);
  m.unique = unique ? 1 : 0;
  m.nradi = 0;
  for (int b = 0; b < nblock; ++b) {
    if (!(step[b] > 0.0) || !(end[b] >= start[b]))
      return set_error(c, INCA_E_ARG, "inca_batch_add_closed_shell: bad scan block");
    m.nradi += static_cast<int>((end[b] - start[b]) / step[b]) + 1;
  }
  m.start.assign(start, start + nblock);
  m.end.assign(end, end + nblock);
  m.step.assign(step, step + nblock);
  m.nang.assign(nang, nang + nblock);
  m.nosym = nosym ? 1 : 0;
  if (nradi) *nradi = m.nradi;
  c->batch.push_back(std::move(m));
  return INCA_OK;
}

int inca_batch_prepare(inca_ctx* c, double thresh, inca_counts* counts, int64_t* ngrid) {
  CTX_CHECK(c);
  const int st = batch_prepare(c, thresh, counts);
  if (st == INCA_OK && ngrid) *ngrid = c->ngrid;
  return st;
}

int inca_batch_eval(inca_ctx* c, int mode, double tol, double* rintra) {
  CTX_CHECK(c);
  if (c->batch_molecules == 0 || c->batch_grid_version != c->grid_version)
    return set_error(c, INCA_E_STATE, "inca_batch_eval: prepare the batch first");
  int st = eval_device(c, mode, tol);
  if (st) return st;
  return rintra ? radial_plot_device(c, rintra) : INCA_OK;
}

}  // extern "C"
