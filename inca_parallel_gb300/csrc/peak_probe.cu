// FP32 FMA throughput of the context's GPU, measured with a dependent-free FMA loop: the
// denominator of the evaluation kernels' roofline (they are bound by the FP32 pipe, not by
// HBM or the tensor cores).
#include "inca_internal.h"

namespace {

constexpr int kChains = 8;       // independent FMA chains per thread
constexpr int kIters = 4096;     // loop trips (each: kChains FMAs)
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fma_peak(float seed, float* out) {
  float a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) a[c] = seed + static_cast<float>(threadIdx.x + c);
  const float m = 0.999999f, b = 1.0e-7f;
#pragma unroll 16
  for (int i = 0; i < kIters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = __fmaf_rn(a[c], m, b);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c];
  if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the loop live; practically never taken
}

}  // namespace

extern "C" int inca_fp32_fma_peak(inca_ctx* c, double* tflops) {
  if (!c || !tflops) return INCA_E_ARG;
  const int blocks = c->num_sms * 8;
  float* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(float) * blocks);
  if (!e) e = cudaEventCreate(&e0);
  if (!e) e = cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5 && !e; ++rep) {
    cudaEventRecord(e0, c->stream);
    INCA_LAUNCH(c, k_fma_peak, blocks, kThreads, 0, 1.0f, out);
    cudaEventRecord(e1, c->stream);
    e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (!e) e = cudaEventElapsedTime(&ms, e0, e1);
    if (!e && rep > 0) best = ms < best ? ms : best;  // first launch is the warm-up
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  if (e) return inca::cuda_error(c, e, "inca_fp32_fma_peak");
  const double flops = 2.0 * kChains * static_cast<double>(kIters) * kThreads * blocks;
  *tflops = flops / (best * 1e-3) / 1e12;
  return INCA_OK;
}
