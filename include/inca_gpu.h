/*
 * inca_gpu.h -- C ABI of the GB300 intracule engine (libinca_gpu.so).
 *
 * Drop-in boundary for the intracule hot path of INCA (markelgtx/INCA_parallel). In the
 * reference that path is one Fortran subroutine, calculate_intracule(normalize_dm2p)
 * (src/mod_intracule.f90:18-572), fed through module globals and called once from the
 * main program (src/inca_main.f90:76). This header replaces it with plain C entry points
 * that a Fortran bind(C) interface, the C++ driver or ctypes can call. Conventions:
 *
 *  - The caller owns every host array; outputs go into caller-provided buffers.
 *  - Every call returns an int status (INCA_OK == 0). On failure inca_last_error(ctx)
 *    returns a message; the Fortran side prints it and stops, as the reference does.
 *  - Primitive and quartet indices are 1-based at the boundary, as in the .dm2p file.
 *  - Arrays shaped like Fortran arrays are column-major: TMN(nprim,3), r(3,ngrid),
 *    cartes(natoms,3).
 *  - One context per host thread; calls are synchronous (results are on the host when a
 *    call returns). A context owns one CUDA stream on one device.
 *  - No CPU fallback: a context cannot be created without a usable sm_103 device.
 */
#ifndef INCA_GPU_H
#define INCA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define INCA_ABI_VERSION 2

/* status codes */
#define INCA_OK 0
#define INCA_E_ARG 1     /* invalid argument: null pointer, bad size, unsupported rule   */
#define INCA_E_CUDA 2    /* CUDA runtime error (the message carries the CUDA string)      */
#define INCA_E_IO 3      /* file could not be opened or read                              */
#define INCA_E_FORMAT 4  /* unsupported or corrupt .dm2p content                          */
#define INCA_E_STATE 5   /* call order violated (e.g. evaluation before inca_prepare)     */
#define INCA_E_NOMEM 6   /* device memory exhausted                                       */
#define INCA_E_LIMIT 7   /* size beyond a documented maximum (e.g. per-dimension degree)  */
#define INCA_E_TIMEOUT 8 /* a bounded device wait gave up; the context stays usable       */

/* evaluation precision */
#define INCA_FP64 0  /* every quartet-point term in FP64 (the plain GPU form)              */
#define INCA_MIXED 1 /* FP32 terms with FP64 accumulation; terms whose FP32 error could
                        exceed the requested tolerance are evaluated in FP64             */
#define INCA_FP64_SCREENED 2 /* every term in FP64, leaving out the negligible (quartet,
                        tile) pairs that INCA_MIXED leaves out, within the same share of the
                        tolerance (grids of 2 048 points or more; cube lattices and smaller
                        grids run as INCA_FP64). No counterpart in the reference: it prices
                        the precision alone against INCA_MIXED                           */

/* maximum per-dimension polynomial degree t_i+t_j+t_k+t_l (g shells: 16) */
#define INCA_MAX_DEGREE 16

typedef struct inca_ctx inca_ctx;

/* Quartet counts as reported in the .out file (src/mod_intracule.f90:419-421). */
typedef struct inca_counts {
  int64_t read;          /* "Quartets in the dm2p file"   */
  int64_t after_screen1; /* "Quartets after 1st screening" */
  int64_t after_screen2; /* "Quartets actually computed"   */
} inca_counts;

int inca_abi_version(void);

/* Context on a CUDA device (the OpenMP team of mod_intracule.f90:203-388 becomes one GPU). */
int inca_ctx_create(inca_ctx** ctx, int device);
int inca_ctx_destroy(inca_ctx* ctx);
const char* inca_last_error(const inca_ctx* ctx);

/* Primitive basis in .dm2p order: Alpha, TMN, Xn/Yn/Zn of mod_geninfo
 * (src/mod_geninfo.f90:9-19, filled by filebas, src/mod_read_files.f90:695-726). */
int inca_set_primitives(inca_ctx* ctx, int32_t nprim, const double* alpha, const int32_t* tmn,
                        const double* xn, const double* yn, const double* zn);

/* DM2 quartets. Replaces the batched .dm2p read (src/mod_intracule.f90:164-262): the same
 * format sniffing (flat stream, or sequential records with 4-byte markers); reading stops
 * at end of file or at the first record whose index is out of range, as in the reference.
 * Formats with 8-byte or zero markers fail with INCA_E_FORMAT. nread may be NULL. */
int inca_load_dm2p(inca_ctx* ctx, const char* path, int64_t* nread);

/* The same .dm2p read on the host alone, without a context or a device: the records go into the
 * caller's arrays (ijkl[4*q+0..3], v[q]; at most `capacity` records, else INCA_E_LIMIT). With
 * ijkl or v NULL only *nread is set. Status as for inca_load_dm2p; the message goes to errbuf
 * (errlen bytes, NUL-terminated) when given. Replaces the same read as inca_load_dm2p
 * (src/mod_intracule.f90:164-262), for hosts that inspect or filter the records themselves. */
int inca_read_dm2p(const char* path, int32_t nprim, int64_t capacity, int32_t* ijkl, double* v, int64_t* nread,
                   char* errbuf, int32_t errlen);

/* Quartets from memory: ijkl[4*q+0..3] = i,j,k,l (1-based), v[q] = DM2 value. */
int inca_set_quartets(inca_ctx* ctx, int64_t n, const int32_t* ijkl, const double* v);

/* Closed-shell DM2 from a 1-RDM D(nprim,nprim) (column-major, primitive basis):
 * Gamma_{ik,jl} = D_ik D_jl - 1/2 D_il D_jk, folded into records with i<=k and j<=l.
 * unique != 0 additionally folds (ik)<->(jl), keeping pair(ik) <= pair(jl)
 * (a symmetry-unique list: evaluate it with nosym). The records are generated on the device. */
int inca_gen_closed_shell_dm2(inca_ctx* ctx, const double* D, int unique, int64_t* nrecords);

/* Screening and per-quartet set-up on the device (src/mod_intracule.f90:282-343 with
 * JA8/polycoef of src/mod_intrastuff.f90:32-194): normalisation (normalize != 0, as
 * calculate_intracule(.true.)), screen 1, Gaussian products, the three polynomial
 * coefficient vectors (LU with partial pivoting), screen 2. lim = thresh/(nprim(nprim+1)/2).
 * The survivors stay resident on the device, grouped by angular class. counts may be NULL.
 * Device memory: for lists of up to 2^26 quartets the context keeps the call's sort scratch
 * (about 24 B per quartet plus the radix sort's temporary storage) until inca_ctx_destroy, so
 * a repeated preparation allocates nothing; larger lists give it back before returning. */
int inca_prepare(inca_ctx* ctx, double thresh, int normalize, inca_counts* counts);

/* Per-quartet screening results of the last inca_prepare, in input order (for checks):
 * flags[q] = 0 (fails screen 1), 1 (passes 1, fails 2), 3 (passes both); s1/s2 values.
 * Any pointer may be NULL. */
int inca_get_screening(inca_ctx* ctx, uint8_t* flags, double* s1, double* s2);

/* Survivor records of the last inca_prepare in input order: A, sqe, d = P_ik - P_jl (3),
 * L (3) and coefficients C (3 x 17, highest degree first). Any pointer may be NULL. */
int inca_get_records(inca_ctx* ctx, double* A, double* sqe, double* d, int32_t* L, double* C);

/* ---- grids, built and kept on the device (src/mod_build_grid.f90) ---- */

/* Multicentre radial x Lebedev grid with TFVC weights (gridpoints + becke, lines 13-277 and
 * 474-575). cent is cent(3,nquad). Outputs: maxgrid (before halving), rgrid (after
 * symmetry halving), ngrid (after dropping weights <= 1e-106). */
int inca_grid_radial(inca_ctx* ctx, int32_t nquad, const int32_t* nradc, const int32_t* nangc,
                     const double* sfalpha, const double* cent, const double* Ps, int nosym,
                     int64_t* maxgrid, int64_t* rgrid, int64_t* ngrid);

/* Radial-scan shells for I(s) (gridpoints2, lines 281-408). */
int inca_grid_scan(inca_ctx* ctx, int32_t nblock, const double* start, const double* end,
                   const double* step, const int32_t* nang, int nosym, int32_t* nradi,
                   int64_t* ngrid);

/* Uniform lattice for the vector cube, x outer / z inner (gridpoints3, lines 412-440). */
int inca_grid_cube(inca_ctx* ctx, const double* center, const double* step, const int32_t* np,
                   int64_t* ngrid);

/* Explicit points r(3,n) (intracule_at_zero, intracule_two_points, mod_intracule.f90:114-129). */
int inca_grid_points(inca_ctx* ctx, int64_t n, const double* r);

/* Copy the resident grid to the host: r(3,ngrid), weights, Vee weights, centre index
 * (1-based) for radial grids; angular weights in w for scan grids. Pointers may be NULL. */
int inca_grid_copy(inca_ctx* ctx, double* r, double* w, double* wvee, int32_t* cmap);

/* ---- evaluation and reductions ---- */

/* Evaluate I at every point of the resident grid (mod_intracule.f90:345-358, all quartets).
 * mode: INCA_FP64, INCA_MIXED or INCA_FP64_SCREENED; tol: relative tolerance of the mixed form
 * on the grid's outputs (ignored for INCA_FP64; <= 0 selects 1e-10). ivec (ngrid) may be NULL (result
 * stays on the device for the reductions). On a cube lattice (inca_grid_cube, one molecule)
 * INCA_MIXED evaluates the lattice's separable factors in double-float (about 2^-44 relative
 * per term) and leaves out only quartets whose terms sum to at most 5% of tol times max|I|;
 * the environment variable INCA_CUBE_SEPARABLE=0 selects the general mixed form there instead. */
int inca_eval(inca_ctx* ctx, int mode, double tol, double* ivec);

/* Schedule of the mixed evaluation: work items per resident CTA of the persistent passes,
 * the stride of the grid sample that estimates the thresholds, the factor applied to the
 * estimates, the share of the tolerance given to left-out (quartet, tile) pairs
 * (drop_fraction, below 0.5; < 0: the default 0.1), and the register budget of the one-pass
 * kernel as resident one-warp CTAs per SM (ctas_per_sm: 12, 16 or 20; 0: the default 16) with
 * the points each lane of its warp tiles holds (points_per_lane: 3, 4 or 5; the pairs compiled
 * are (4, 12|16|20), (3, 16|20) and (5, 12|16), any other pair is INCA_E_ARG; 0: from the mean
 * surviving records per molecule, 3 up to 1e6, 5 from 1e7, else 4, and 4 where that value does
 * not pair with ctas_per_sm), and the slack of the cheap tier (cheap_slack, 0..30:
 * a (quartet, tile) pair is evaluated in plain FP32 when its rigorous error bound is at most
 * 2^cheap_slack times the tile's drop threshold; that bound joins the left-out mass, which is
 * checked after the pass as before, so a large slack can cost a repeat, never accuracy).
 * inca_autotune times complete INCA_MIXED evaluations of the current grid and records (median
 * of reps each) over candidate schedules by coordinate descent (two sweeps) and a joint sweep of
 * estimate_safety, drop_fraction and cheap_slack around the result, keeps the fastest in the
 * context and reports it with the time of the default schedule; the last evaluation's results
 * stay on the device. inca_set_tuning sets a schedule (NULL: the defaults). Every schedule meets
 * the tolerance. No counterpart in the reference. */
typedef struct inca_tuning {
  int32_t items_per_cta;
  int32_t sample_stride;
  double estimate_safety;
  double best_ms;     /* output of inca_autotune */
  double default_ms;  /* output of inca_autotune */
  double drop_fraction;
  int32_t ctas_per_sm;
  int32_t cheap_slack;
  int32_t points_per_lane;
} inca_tuning;
int inca_autotune(inca_ctx* ctx, double tol, int32_t reps, inca_tuning* chosen);
int inca_set_tuning(inca_ctx* ctx, const inca_tuning* tuning);

/* inca_eval replayed from a CUDA graph (INCA_MIXED; INCA_FP64 runs as inca_eval). The first
 * call after the grid, tol, the schedule (inca_set_tuning, inca_autotune) or the shape of the
 * record tables changes evaluates normally and captures the evaluation's launch sequence; later
 * calls launch the captured graph,
 * which runs every pass without returning to the host in between. Cube lattices evaluated by
 * the separable form (two launches, nothing to plan) run as inca_eval. No counterpart in the
 * reference. */
int inca_eval_graph(inca_ctx* ctx, int mode, double tol, double* ivec);

/* Radial integral, Vee and the per-centre TFVC decomposition (mod_intracule.f90:441-455)
 * of the last evaluation on a radial grid. per_centre/vee_per_centre (nquad) may be NULL. */
int inca_radial_integral(inca_ctx* ctx, double* total, double* vee, double* per_centre,
                         double* vee_per_centre);

/* I(s) per shell of the last evaluation on a scan grid (mod_intracule.f90:522-530). */
int inca_radial_plot(inca_ctx* ctx, double* radi, double* rintra);

/* Gaussian-smeared P(u) and I_avg(u) of the last radial-grid evaluation
 * (radial_smearing, mod_intracule.f90:576-649): n_bins values each. */
int inca_radial_smearing(inca_ctx* ctx, double u_max, int32_t n_bins, double sigma,
                         double* u_axis, double* P_u, double* I_avg);

/* Automatic integration centres (centercalc + get_bs_radius, src/mod_autogrid.f90:12-185).
 * an(natoms), cartes(natoms,3) in bohr. Output capacity: natoms*(natoms-1)+1 centres;
 * cent(3,nquad). Host-side (tiny). */
int inca_centercalc(int32_t natoms, const int32_t* an, const double* cartes, int nohydro,
                    int betaone, int32_t* nquad, double* cent, double* Ps, double* sfalpha);

/* Timing of the last inca_eval on the device (CUDA events): total milliseconds, the
 * milliseconds of its dominant kernel, the number of that kernel's launches and the
 * number of kernel launches of the call. Pointers may be NULL. */
int inca_last_eval_timing(inca_ctx* ctx, double* total_ms, double* kernel_ms,
                          int32_t* kernel_launches, int32_t* launches);

/* Work split of the last INCA_MIXED evaluation, in (quartet, 128-point tile) pairs: evaluated
 * in FP32, examined for corrections (the precise tier; in the one-pass form used on grids of
 * 2 048 points or more, the warp rounds of inline corrections plus the pairs examined by a
 * correction pass, if one ran), skipped (bound below 2^-120); and the number of (quartet,
 * point) terms re-evaluated in double-float arithmetic (a correction pass counts them in warps
 * of 32 points). The FP64 form reports zeros. Pointers may be NULL. */
int inca_last_eval_stats(inca_ctx* ctx, int64_t* fp32_pairs, int64_t* precise_pairs,
                         int64_t* skipped_pairs, int64_t* corrected_terms);

/* (Quartet, 128-point tile) pairs of the last INCA_MIXED evaluation that took the cheap tier of
 * the one-pass form: plain FP32 terms whose rigorous error bound is counted with the terms left
 * out, as a dropped term's bound is (0 for other forms; these pairs are not in fp32_pairs of
 * inca_last_eval_stats). No counterpart in the reference. */
int inca_last_eval_cheap_pairs(inca_ctx* ctx, int64_t* cheap_pairs);

/* Device milliseconds of the two passes of the last INCA_MIXED evaluation (estimate pass over
 * all terms; correction pass). The FP64 form reports its single kernel as pass 1. */
int inca_last_eval_phases(inca_ctx* ctx, double* pass1_ms, double* pass2_ms);

/* The context's CUDA stream (a cudaStream_t), for callers that order their own work or
 * record CUDA events around the library's calls. */
int inca_get_stream(inca_ctx* ctx, void** stream);

/* Number of this library's own kernels launched by the context since it was created
 * (library kernels such as CUB sorts are not counted). */
int inca_kernel_launches(inca_ctx* ctx, int64_t* count);

/* Measured FP32 FMA throughput of the context's GPU in TFLOP/s (2 flops per FMA; a short
 * microbenchmark on the context's stream). Diagnostic with no counterpart in the reference:
 * the roofline denominator of the evaluation kernels, which are bound by the FP32 pipe. */
int inca_fp32_fma_peak(inca_ctx* ctx, double* tflops);

/* ---------------------------------------------------------------------------------------
 * Batches of molecules. No counterpart in the reference, which runs calculate_intracule once per
 * molecule (one process each); a batch runs the radial_plot job (src/mod_intracule.f90:512-533)
 * for up to INCA_MAX_BATCH molecules with one screening pass and one launch of each evaluation
 * kernel. inca_batch_clear starts a batch; inca_batch_add_closed_shell appends a molecule (its
 * primitives as for inca_set_primitives, its closed-shell 1-RDM D(nprim,nprim) as for
 * inca_gen_closed_shell_dm2, and its radial-scan grid as for inca_grid_scan; nradi returns the
 * molecule's shell count); inca_batch_prepare generates and screens every molecule's DM2 and
 * builds the concatenated grid (it replaces the context's primitives, quartets and grid;
 * counts and ngrid, the total grid points, may be NULL); inca_batch_eval evaluates all molecules and writes their I(s)
 * molecule after molecule into rintra (sum of the nradi values; NULL keeps them on the device).
 * inca_eval and inca_radial_plot also work on a prepared batch. */
#define INCA_MAX_BATCH 128
int inca_batch_clear(inca_ctx* ctx);
int inca_batch_add_closed_shell(inca_ctx* ctx, int32_t nprim, const double* alpha, const int32_t* tmn,
                                const double* xn, const double* yn, const double* zn, const double* D,
                                int unique, int32_t nblock, const double* start, const double* end,
                                const double* step, const int32_t* nang, int nosym, int32_t* nradi);
int inca_batch_prepare(inca_ctx* ctx, double thresh, inca_counts* counts, int64_t* ngrid);
int inca_batch_eval(inca_ctx* ctx, int mode, double tol, double* rintra);

/* ---------------------------------------------------------------------------------------
 * A small multilayer perceptron trained and evaluated by this library's kernels, used to
 * predict per-centre radial-grid scales for the automatic multicentre grids
 * (inca_parallel_gb300/learned_grid.py). No counterpart in the reference (mod_autogrid,
 * src/mod_autogrid.f90:12-185, takes every centre's scale from Bragg-Slater radii; it stays the
 * fallback). Network: nin -> nhidden (tanh) -> nhidden (tanh) -> nout, FP32; parameters in one
 * array: W1[nhidden][nin], b1[nhidden], W2[nhidden][nhidden], b2[nhidden], W3[nout][nhidden],
 * b3[nout] (row-major). Loss: mean over rows of the squared error summed over outputs; Adam.
 * X is X[n][nin], T and Y are [n][nout] (host arrays). Deterministic for a given seed. */
typedef struct inca_mlp inca_mlp;
int inca_mlp_create(inca_mlp** mlp, int device, int32_t nin, int32_t nhidden, int32_t nout, uint64_t seed);
int inca_mlp_destroy(inca_mlp* mlp);
int inca_mlp_param_count(inca_mlp* mlp, int64_t* count);
int inca_mlp_get_params(inca_mlp* mlp, float* params);
int inca_mlp_set_params(inca_mlp* mlp, const float* params);
int inca_mlp_forward(inca_mlp* mlp, int64_t n, const float* X, float* Y);
/* loss and its gradient with respect to every parameter (grad: inca_mlp_param_count floats) */
int inca_mlp_gradient(inca_mlp* mlp, int64_t n, const float* X, const float* T, float* loss, float* grad);
/* epochs of minibatch Adam (rows shuffled by seed); final_loss: loss over all n rows */
int inca_mlp_train(inca_mlp* mlp, int64_t n, const float* X, const float* T, int32_t epochs, int32_t batch,
                   float lr, uint64_t seed, float* final_loss);

/* ---------------------------------------------------------------------------------------
 * Evaluation without allocation. No counterpart in the reference (the Fortran program
 * allocates its work arrays itself); this entry point exists for callers that must not
 * allocate device memory while they run: a solver that keeps all its device memory in its
 * own pool or arena, or a long-running service that allocates only at start-up so that it
 * can never fail for lack of memory later. The context API above cannot serve them, because
 * inca_eval grows its buffers with cudaMalloc.
 *
 * Computes ivec[g] = sum_q A[q] exp(-|r'|^2) Vx(r'_x) Vy(r'_y) Vz(r'_z),
 * r' = sqe[q] (r_g + d_q), in FP64, for nrec survivor records laid out as inca_get_records
 * returns them (A[nrec], sqe[nrec], d[nrec][3], L[nrec][3] with 0 <= L <= INCA_MAX_DEGREE,
 * C[nrec][3][INCA_MAX_DEGREE+1] highest degree first) and npts points r[npts][3].
 * Every pointer is DEVICE memory owned by the caller, on the current device; the work is
 * queued on `stream` (a cudaStream_t; NULL is the legacy default stream) and the call
 * returns without waiting for it. The result equals inca_eval(INCA_FP64) on the same
 * records and points up to summation order.
 *
 * Limits and behaviour:
 *  - npts <= INCA_NOALLOC_MAX_POINTS; a larger npts returns INCA_E_LIMIT and queues nothing.
 *    The intermediate sums live in a fixed 16 MiB device array inside the library.
 *  - The first call on a device sets that device up (it looks up the address of the fixed
 *    array in the current CUDA context). A call made under a different context than the last
 *    one on that device (for instance after cudaDeviceReset) sets the device up again.
 *  - Calls that overlap in time on one device (different streams or host threads) share the
 *    fixed array and race: order them, e.g. on one stream.
 *  - nrec == 0 writes zeros to ivec with one cudaMemsetAsync on `stream`.
 *  - Status codes only (there is no context for inca_last_error): INCA_E_ARG for negative
 *    sizes or null pointers, INCA_E_LIMIT as above, INCA_E_CUDA for a launch failure or for
 *    a CUDA error already pending on the calling thread (left pending; nothing is queued).
 */
#define INCA_NOALLOC_MAX_POINTS (1 << 21)
int inca_eval_records_noalloc(int64_t nrec, const double* A, const double* sqe,
                              const double* d, const int32_t* L, const double* C,
                              int64_t npts, const double* r, double* ivec, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* INCA_GPU_H */
