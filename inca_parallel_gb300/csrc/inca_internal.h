// Internal declarations of libinca_gpu.so (not part of the ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/inca_gpu.h"

namespace inca {

constexpr int kMaxDeg = INCA_MAX_DEGREE;  // per-dimension polynomial degree
constexpr int kMaxCoef = kMaxDeg + 1;
constexpr int kRecHeader = 6;             // A, sqe, d0, d1, d2, B (term bound factor)
constexpr int kMaxGH = 11;                // Gauss-Hermite nodes for L <= 21

// ---------------------------------------------------------------- status helpers
struct Error {
  int code;
  std::string msg;
};

// Device buffer owned by the context; grows, never shrinks until the context dies.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;  // capacity in elements
  cudaError_t reserve(size_t want) {
    if (want <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (want == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), want * sizeof(T));
    if (e == cudaSuccess) n = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// One primitive as the device kernels read it.
// lim_scale = 1 / (nprim (nprim + 1) / 2) of the primitive's molecule (the screening limit is
// thresh * lim_scale, src/mod_intracule.f90:163); mol: molecule index within a batch (else 0).
struct PrimD {
  double alpha, x, y, z, norm, lim_scale;
  int t[3];
  int mol;
};

// Angular class of survivors: all records of a class share (Lx, Ly, Lz) and a stride.
struct ClassSeg {
  int L[3];
  int stride;       // doubles per FP64 record (even)
  int64_t first;    // first survivor (class-sorted index)
  int64_t count;
  int64_t off64;    // offset of the segment in the FP64 record array (doubles)
  int64_t off32;    // offset of the segment in the FP32 record array (floats)
  int stride32;     // floats per FP32 record (multiple of 4)
  int mol;          // molecule of the segment (0 unless batched)
};

// A chunk of <= kChunk records of one class: the unit of work of the evaluation kernels.
struct WorkChunk {
  int cls;
  int count;
  int64_t rec;  // first class-sorted survivor index
};

// A tile of up to 128 points of the sorted grid (consecutive), and the molecule whose
// quartet chunks it is evaluated against (index into the per-molecule chunk ranges).
struct TileInfo {
  int64_t start;
  int count;
  int mol;
};

// The chunk range [begin, end) of one molecule.
struct ChunkRange {
  int begin, end;
};

// Work of one molecule in a persistent pass: its chunk range, its quartet splits, its tiles
// and sorted points, where its work items start, and where its partial sums and left-out
// bound masses start (partials: split-major over the molecule's points; masses: split-major
// over its tiles).
struct MolWork {
  int cb, ce;
  int nsplit;
  int pad;
  int64_t tile0, ntiles;
  int64_t p0, np;
  int64_t item0;
  int64_t poff, doff;
};

// Tiles and sorted points of one molecule in a sorted grid.
struct MolSpan {
  int64_t tile0, ntiles, p0, np;
};

// One molecule of a batch, as added (host copies until the batch is prepared).
struct BatchMol {
  int nprim = 0;
  std::vector<double> alpha, x, y, z, D;
  std::vector<int> tmn;  // row-major nprim x 3
  int unique = 0;
  std::vector<double> start, end, step;
  std::vector<int> nang;
  int nosym = 0;
  int nradi = 0;
};

enum GridKind { GRID_NONE = 0, GRID_RADIAL = 1, GRID_SCAN = 2, GRID_CUBE = 3, GRID_POINTS = 4 };

}  // namespace inca

struct inca_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string err;

  // primitives
  int nprim = 0;
  std::vector<double> h_alpha, h_x, h_y, h_z;
  std::vector<int> h_tmn;  // row-major nprim x 3
  inca::DevBuf<inca::PrimD> d_prims;

  // quartet input (device, 1-based indices)
  int64_t nq = 0;
  inca::DevBuf<int4> d_ijkl;
  inca::DevBuf<double> d_v;

  // screening results in input order
  bool prepared = false;
  inca_counts counts{0, 0, 0};
  double lim = 0.0;
  inca::DevBuf<uint8_t> d_flags;
  inca::DevBuf<double> d_ja8;  // JA8 of every primitive pair (screening)
  inca::DevBuf<double> d_s1, d_s2;
  bool have_screen_values = false;
  // scratch of inca_prepare (sort keys and indices, radix-sort temporary storage, run-length
  // encoding of the classes, counters); kept between calls for lists of moderate size
  inca::DevBuf<uint32_t> d_pkey, d_pkey2, d_pukeys;
  inca::DevBuf<int64_t> d_pidx, d_pidx2, d_pucounts;
  inca::DevBuf<unsigned char> d_ptmp;
  inca::DevBuf<int> d_pbad, d_pnruns;
  inca::DevBuf<unsigned long long> d_pn1;
  inca::DevBuf<unsigned char> d_pqrec;  // each survivor's screened quartet, read by the record build

  // survivors, grouped by class
  int64_t nsurv = 0;
  std::vector<inca::ClassSeg> classes;
  std::vector<inca::WorkChunk> chunks;
  inca::DevBuf<inca::ClassSeg> d_classes;
  inca::DevBuf<inca::WorkChunk> d_chunks;
  inca::DevBuf<double> d_rec64;     // FP64 records, class segments
  inca::DevBuf<float> d_rec32;      // FP32 records (mixed form), class segments
  inca::DevBuf<int64_t> d_surv_src; // input index of each class-sorted survivor
  int max_L = 0;
  int batch_molecules = 0;                   // molecules of the current batch (0: not batched)
  std::vector<inca::BatchMol> batch;         // molecules added since inca_batch_clear
  std::vector<int64_t> h_mol_off;            // first grid point of each molecule (+ total)
  std::vector<int> h_mol_shell_off;          // first shell of each molecule (+ total)
  inca::DevBuf<int> d_pmol;                  // molecule of each grid point (batch grids)
  int64_t batch_grid_version = -1;
  std::vector<inca::ChunkRange> mol_chunks;  // chunk range of each molecule (one entry unless batched)
  std::vector<int64_t> mol_surv;             // survivors of each molecule

  // grid
  int grid_kind = inca::GRID_NONE;
  int64_t ngrid = 0, maxgrid = 0, rgrid = 0;
  int nquad = 0;
  int nradi = 0;
  int cube_np[3] = {0, 0, 0};    // lattice points per axis (cube grids)
  std::vector<int> h_smn;        // points per shell (scan grids)
  std::vector<double> h_radi;    // shell radii (scan grids)
  std::vector<double> h_cent;    // centres (radial grids)
  inca::DevBuf<double> d_px, d_py, d_pz, d_w, d_wvee;
  inca::DevBuf<int> d_cmap;
  inca::DevBuf<double> d_ivec;
  // temporaries of the grid builders (candidates, tables, compaction), kept between calls
  inca::DevBuf<unsigned char> d_gscratch;
  // temporaries of the Morton sort of the mixed form (keys, indices, radix-sort storage, bounding
  // box), kept between calls
  inca::DevBuf<unsigned char> d_sscratch;
  inca::DevBuf<double> d_bbox;
  // scratch of the per-shell / per-centre reductions (segment offsets, sums), kept between calls
  inca::DevBuf<int64_t> d_roff;
  inca::DevBuf<double> d_rsum;
  bool evaluated = false;
  int64_t grid_version = 0;  // bumped by every grid builder

  // mixed evaluation: Morton-sorted copy of the grid (rebuilt when the grid changes)
  int64_t mix_version = -1;
  int mix_ppt = 4;                    // points per lane of its warp tiles (a tile: 32 x mix_ppt)
  inca::DevBuf<float4> d_phi, d_plo;  // FP32 hi / lo parts of the sorted points
  inca::DevBuf<int64_t> d_perm;       // sorted position -> grid index
  inca::DevBuf<float> d_wtbox;        // per warp tile: lo[3], hi[3], 2 pad
  inca::DevBuf<inca::TileInfo> d_tiles;  // tiles of the sorted grid
  int64_t ntiles = 0;
  std::vector<inca::MolSpan> mol_span;   // per molecule: its tiles and sorted points
  // the same for a strided sample of the grid (threshold estimates of the one-pass form)
  int64_t sample_version = -1;
  int64_t nsample = 0;
  inca::DevBuf<float4> d_phi_s, d_plo_s;
  inca::DevBuf<int64_t> d_perm_s;
  inca::DevBuf<float> d_wtbox_s;
  inca::DevBuf<inca::TileInfo> d_tiles_s;
  int64_t ntiles_s = 0;
  std::vector<inca::MolSpan> mol_span_s;
  inca::DevBuf<unsigned char> d_scratch_s;

  // separable cube evaluation: the lattice's axis coordinates (x, y, z runs; rebuilt when the
  // grid changes)
  inca::DevBuf<double> d_cube_axes;
  int64_t cube_axes_version = -1;
  float cube_floor_log2 = -120.0f;  // record floor of the last separable evaluation

  // scratch
  inca::DevBuf<double> d_partial;
  inca::DevBuf<unsigned char> d_scratch;

  // timing and tier statistics of the last evaluation
  double t_total_ms = 0, t_kernel_ms = 0, t_pass2_ms = 0;
  int t_kernel_launches = 0, t_launches = 0;
  int64_t pairs_fp32 = 0, pairs_fp64 = 0, pairs_skip = 0, corrected_points = 0, pairs_cheap = 0;
  int64_t launches = 0;  // own kernel launches since creation

  // schedule of the mixed evaluation (inca_autotune / inca_set_tuning; 0 or < 0: defaults)
  int tune_items_per_cta = 0;
  int tune_sample_stride = 0;
  double tune_safety = -1.0;
  double tune_drop = -1.0;
  int tune_ctas = 0;  // resident CTAs per SM of the one-pass kernel (0: the default)
  int tune_ppt = 0;   // points per lane of its warp tiles (0: the default, 4)
  int tune_cheap_slack = -1;  // cheap-tier slack in powers of two (-1: the default, 0)
  int sample_stride_built = 0;  // stride of the current sorted sample

  // graph replay of the mixed evaluation (captured for one grid, set of records and tolerance)
  inca::DevBuf<float2> d_exptab;  // 2^(j/256) table of the double-float exp2
  int64_t prepare_count = 0;      // bumped by every inca_prepare / batch preparation
  cudaGraphExec_t graph_exec = nullptr;
  int64_t graph_grid = -1, graph_launches = 0;
  std::vector<double> graph_sig;  // plan signature of the captured graph (mixed_eval.cu)
  bool graph_fused = false, graph_drop = false;
};

// ---- internal entry points between translation units
namespace inca {

int set_error(inca_ctx* c, int code, const std::string& msg);
PrimD make_prim(double alpha, const int t[3], double x, double y, double z, int nprim_mol, int mol);
int cuda_error(inca_ctx* c, cudaError_t e, const char* what);

// quartet_prep.cu
int prepare_device(inca_ctx* c, double thresh, int normalize);
int gen_closed_shell_device(inca_ctx* c, const double* D, int unique, int64_t* nrec);
int64_t closed_shell_records(int n, int unique);
int gen_closed_shell_into(inca_ctx* c, int n, const double* D, int unique, int base, int64_t at);

// intracule_eval.cu
int eval_device(inca_ctx* c, int mode, double tol, bool graph = false);
// mixed_eval.cu
int autotune_mixed(inca_ctx* c, double eps, int reps, int* ipc, int* stride, double* safety, double* drop,
                   int* ctas, int* slack, int* ppt, double* best_ms, double* default_ms);
bool valid_pass_shape(int ppt, int ctas);
int ensure_exp_table(inca_ctx* c);
// cube_eval.cu
bool cube_separable(const inca_ctx* c);
int eval_cube_separable(inca_ctx* c, double eps);
int eval_fp64_screened(inca_ctx* c, double eps, bool* plain);

// grid_build.cu
int grid_radial_device(inca_ctx* c, int nquad, const int* nradc, const int* nangc,
                       const double* sfalpha, const double* cent, const double* Ps, int nosym);
int grid_scan_device(inca_ctx* c, int nblock, const double* start, const double* end,
                     const double* step, const int* nang, int nosym);
int grid_cube_device(inca_ctx* c, const double* center, const double* step, const int* np);
int radial_integral_device(inca_ctx* c, double* total, double* vee, double* per_c, double* vee_c);
int radial_plot_device(inca_ctx* c, double* rintra);
int smearing_device(inca_ctx* c, double u_max, int n_bins, double sigma, double* u, double* P,
                    double* I);

// host_tables.cpp
int lebedev_rule(int nang, std::vector<double>& x, std::vector<double>& y,
                 std::vector<double>& z, std::vector<double>& w);
void gauss_legendre(int n, double* t, double* w);
int read_dm2p(const char* path, int nprim, std::vector<int4>& ijkl, std::vector<double>& v,
              std::string& err);

}  // namespace inca

// Launch one of this library's kernels on the context stream and count it.
#define INCA_LAUNCH(c, kernel, grid, block, smem, ...)                          \
  do {                                                                         \
    kernel<<<(grid), (block), (smem), (c)->stream>>>(__VA_ARGS__);             \
    ++(c)->launches;                                                           \
  } while (0)

#define INCA_CUDA(c, call)                                        \
  do {                                                            \
    cudaError_t e_ = (call);                                      \
    if (e_ != cudaSuccess) return inca::cuda_error((c), e_, #call); \
  } while (0)
