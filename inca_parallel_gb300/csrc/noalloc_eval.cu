// FP64 evaluation of the intracule (the point loop of src/mod_intracule.f90:345-358) from
// caller-owned device records into a caller-owned device output, allocating nothing.
//
// The context API (inca_eval) grows its own device buffers with cudaMalloc. Some callers
// cannot allow that: code running inside a caller-managed memory pool or arena, or a service
// that must not allocate after start-up so that it cannot run out of memory later. This entry
// point takes every input and output from the caller and keeps its only intermediate (the
// per-split partial sums) in a fixed file-scope device array.
//
// Work decomposition: a CTA owns 256 points (2 per thread) and one contiguous range of
// records (its split); it writes one partial per point into the fixed scratch array, and a
// second kernel adds the splits of each point in split order, so a call is deterministic.
// Every scratch element a call reads was written earlier in the same call: nothing has to
// be cleared beforehand. Calls that overlap in time on one device (two streams, two host
// threads) share the scratch array and race.
#include <algorithm>
#include <mutex>

#include <cuda.h>  // driver API types only: the two functions used are resolved at run time

#include "inca_internal.h"

// Scratch capacity: splits x points <= INCA_NOALLOC_MAX_POINTS doubles (16 MiB).
static __device__ __align__(256) double g_noalloc_scratch[INCA_NOALLOC_MAX_POINTS];

namespace {

constexpr int kThreads = 128;
constexpr int kPPT = 2;
constexpr int kTile = kThreads * kPPT;
constexpr int kMaxDevices = 256;
constexpr int kCoef = INCA_MAX_DEGREE + 1;

// Per-device set-up, done with that device current, once per CUDA context: the scratch
// array's address belongs to the context that loaded the module, so a context created anew
// on the device (after cudaDeviceReset, or a caller's own context) is set up again.
struct DeviceSlot {
  bool ready = false;
  unsigned long long ctx_id = 0;
  double* scratch = nullptr;
  int num_sms = 0;
};
std::mutex g_setup_mutex;
DeviceSlot g_slots[kMaxDevices];

using PfnCtxGetCurrent = CUresult (*)(CUcontext*);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);
PfnCtxGetCurrent g_ctx_get_current = nullptr;
PfnCtxGetId g_ctx_get_id = nullptr;

__global__ void __launch_bounds__(kThreads)
k_eval_records(int64_t nrec, int64_t per_split, const double* __restrict__ A,
               const double* __restrict__ sqe, const double* __restrict__ d,
               const int32_t* __restrict__ L, const double* __restrict__ C, int64_t npts,
               const double* __restrict__ r, double* __restrict__ partial) {
  const int tid = threadIdx.x;
  const int64_t base = static_cast<int64_t>(blockIdx.x) * kTile;
  double x[kPPT], y[kPPT], z[kPPT], acc[kPPT];
#pragma unroll
  for (int p = 0; p < kPPT; ++p) {
    const int64_t g = base + tid + p * kThreads;
    const bool ok = g < npts;
    x[p] = ok ? r[3 * g + 0] : 0.0;
    y[p] = ok ? r[3 * g + 1] : 0.0;
    z[p] = ok ? r[3 * g + 2] : 0.0;
    acc[p] = 0.0;
  }
  const int64_t q0 = static_cast<int64_t>(blockIdx.y) * per_split;
  const int64_t q1 = min(nrec, q0 + per_split);
  for (int64_t q = q0; q < q1; ++q) {
    const double a = A[q], s = sqe[q];
    const double d0 = d[3 * q + 0], d1 = d[3 * q + 1], d2 = d[3 * q + 2];
    // degrees outside 0..INCA_MAX_DEGREE are clamped so that reads stay inside the record
    const int Lx = min(max(L[3 * q + 0], 0), INCA_MAX_DEGREE);
    const int Ly = min(max(L[3 * q + 1], 0), INCA_MAX_DEGREE);
    const int Lz = min(max(L[3 * q + 2], 0), INCA_MAX_DEGREE);
    const double* Cx = C + 3 * q * kCoef;  // highest degree first
    const double* Cy = Cx + kCoef;
    const double* Cz = Cy + kCoef;
#pragma unroll
    for (int p = 0; p < kPPT; ++p) {
      const double rx = s * (x[p] + d0), ry = s * (y[p] + d1), rz = s * (z[p] + d2);
      double vx = Cx[0], vy = Cy[0], vz = Cz[0];
      for (int m = 1; m <= Lx; ++m) vx = fma(vx, rx, Cx[m]);
      for (int m = 1; m <= Ly; ++m) vy = fma(vy, ry, Cy[m]);
      for (int m = 1; m <= Lz; ++m) vz = fma(vz, rz, Cz[m]);
      const double e = exp(-(rx * rx + ry * ry + rz * rz));
      acc[p] += a * e * vx * vy * vz;
    }
  }
#pragma unroll
  for (int p = 0; p < kPPT; ++p) {
    const int64_t g = base + tid + p * kThreads;
    if (g < npts) partial[static_cast<int64_t>(blockIdx.y) * npts + g] = acc[p];
  }
}

__global__ void k_sum_record_splits(const double* __restrict__ partial, int nsplit, int64_t npts,
                                    double* __restrict__ out) {
  const int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (g >= npts) return;
  double s = 0.0;
  for (int k = 0; k < nsplit; ++k) s += partial[static_cast<int64_t>(k) * npts + g];
  out[g] = s;
}

// Id of the calling thread's current CUDA context (0: none is current yet). Ids are unique
// for the life of the process, so a context created after a reset has a new one.
int current_ctx_id(unsigned long long* id) {
  if (!g_ctx_get_current || !g_ctx_get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return INCA_E_CUDA;
    g_ctx_get_current = reinterpret_cast<PfnCtxGetCurrent>(f1);
    g_ctx_get_id = reinterpret_cast<PfnCtxGetId>(f2);
  }
  CUcontext c = nullptr;
  if (g_ctx_get_current(&c) != CUDA_SUCCESS) return INCA_E_CUDA;
  *id = 0;
  if (c && g_ctx_get_id(c, id) != CUDA_SUCCESS) return INCA_E_CUDA;
  return INCA_OK;
}

// Set-up of a device for the current context: resolve the scratch array's address and the
// SM count (first call on the device, and again whenever the current context has changed).
int device_setup(int dev, DeviceSlot* out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  unsigned long long id = 0;
  int st = current_ctx_id(&id);
  if (st != INCA_OK) return st;
  DeviceSlot& s = g_slots[dev];
  if (!s.ready || id == 0 || s.ctx_id != id) {
    void* p = nullptr;
    // with no context current yet, this call also initialises the device's primary context
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return INCA_E_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return INCA_E_CUDA;
    if (id == 0 && ((st = current_ctx_id(&id)) != INCA_OK || id == 0)) return st != INCA_OK ? st : INCA_E_CUDA;
    s.scratch = static_cast<double*>(p);
    s.num_sms = sms;
    s.ctx_id = id;
    s.ready = true;
  }
  *out = s;
  return INCA_OK;
}

}  // namespace

extern "C" int inca_eval_records_noalloc(int64_t nrec, const double* A, const double* sqe,
                                         const double* d, const int32_t* L, const double* C,
                                         int64_t npts, const double* r, double* ivec,
                                         void* stream) {
  if (nrec < 0 || npts < 0) return INCA_E_ARG;
  if (npts > INCA_NOALLOC_MAX_POINTS) return INCA_E_LIMIT;
  if (npts == 0) return INCA_OK;
  if (!r || !ivec || (nrec > 0 && (!A || !sqe || !d || !L || !C))) return INCA_E_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return INCA_E_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return INCA_E_LIMIT;
  // an error left pending by the caller's own work is reported, not cleared, and nothing is
  // queued (otherwise the launch checks below would take it for a failure of this call)
  if (cudaPeekAtLastError() != cudaSuccess) return INCA_E_CUDA;
  DeviceSlot slot;
  const int st = device_setup(dev, &slot);
  if (st != INCA_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (nrec == 0) {
    return cudaMemsetAsync(ivec, 0, sizeof(double) * npts, s) == cudaSuccess ? INCA_OK : INCA_E_CUDA;
  }
  // Splits: enough (tiles x splits) CTAs to fill the GPU a few times over, bounded by the
  // number of record groups of 32 and by the scratch capacity.
  const int64_t tiles = (npts + kTile - 1) / kTile;
  const int64_t target = static_cast<int64_t>(slot.num_sms) * 16;
  int64_t nsplit = (target + tiles - 1) / tiles;
  nsplit = std::min<int64_t>(nsplit, (nrec + 31) / 32);
  nsplit = std::min<int64_t>(nsplit, INCA_NOALLOC_MAX_POINTS / npts);
  nsplit = std::max<int64_t>(std::min<int64_t>(nsplit, 4096), 1);
  const int64_t per_split = (nrec + nsplit - 1) / nsplit;
  dim3 grid(static_cast<unsigned>(tiles), static_cast<unsigned>(nsplit));
  k_eval_records<<<grid, kThreads, 0, s>>>(nrec, per_split, A, sqe, d, L, C, npts, r, slot.scratch);
  if (cudaGetLastError() != cudaSuccess) return INCA_E_CUDA;
  k_sum_record_splits<<<static_cast<unsigned>((npts + 255) / 256), 256, 0, s>>>(
      slot.scratch, static_cast<int>(nsplit), npts, ivec);
  if (cudaGetLastError() != cudaSuccess) return INCA_E_CUDA;
  return INCA_OK;
}
