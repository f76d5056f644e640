// Device helpers shared by the FP32-pipe evaluation kernels (mixed_eval.cu, cube_eval.cu):
// double-buffered staging of quartet-record chunks into shared memory by 1-D TMA bulk copies
// (cp.async.bulk + mbarrier, every wait bounded), the persistent work counter, and
// double-float (hi + lo FP32 pair, ~2^-44 relative) arithmetic with its exp2.
// Explicit round-to-nearest intrinsics only: results do not depend on FMA contraction.
#pragma once
#include <cstdint>

#include "inca_internal.h"

namespace inca {
namespace {

constexpr int kChunkMax = 32;        // records per work chunk
constexpr int kExpTab = 256;         // 2^(j/256), j = -128..128 (double-float exp2 table)
constexpr int kWaitLimit = 1 << 22;  // bounded mbarrier waits
// |u_d| limit for the polynomial factors: 2^(-u^2 + ks) is zero beyond sqrt(126 + ks) < 64
// for every representable A' scale ks used here, and 64^16 stays finite in FP32
constexpr float kUClamp = 64.0f;

// ---------------------------------------------------------------- TMA bulk staging
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// One thread: expect `bytes` on the barrier and start the bulk copy global -> shared.
// Requires 16-byte aligned addresses and a size that is a multiple of 16.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Bounded wait for the barrier phase with the given parity; false if the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = kWaitLimit) {
  for (int it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

struct ChunkRef {
  const float* src;
  uint32_t bytes;
};
__device__ __forceinline__ ChunkRef chunk_ref(const WorkChunk* chunks, const ClassSeg* segs, const float* rec32,
                                              int ch) {
  const WorkChunk w = chunks[ch];
  const ClassSeg sg = segs[w.cls];
  return {rec32 + sg.off32 + (w.rec - sg.first) * sg.stride32,
          static_cast<uint32_t>(w.count * sg.stride32 * sizeof(float))};
}

// Shared-memory stage of a warp-CTA (dynamic shared memory): two barriers, then two chunk
// buffers of `floats` floats each (32 records of the largest stride present).
// Buffer k & 1 is addressed by arithmetic on the shared-memory base (not by indexing an array of
// pointers, which the compiler keeps in local memory): the record reads stay shared-memory loads.
struct Stage {
  uint64_t* bar;
  float* buf0;
  int floats;
  __device__ __forceinline__ float* buf(int k) const { return buf0 + (k & 1) * floats; }
};
__device__ __forceinline__ Stage stage_view(unsigned char* dsm, int floats) {
  Stage S;
  S.bar = reinterpret_cast<uint64_t*>(dsm);
  S.buf0 = reinterpret_cast<float*>(dsm + 128);
  S.floats = floats;
  return S;
}

// Set up the two barriers (once per CTA; they then serve every work item of the CTA).
__device__ __forceinline__ void stage_init(const Stage& S) {
  if (threadIdx.x == 0) {
    mbar_init(&S.bar[0]);
    mbar_init(&S.bar[1]);
    fence_mbar_init();
  }
  __syncwarp();
}

// Start the copy of an item's first chunk (global chunk counter k) into buffer k & 1.
// issue = false (test of the bounded waits only): no copy is started, so the wait on that
// buffer runs out.
__device__ __forceinline__ void stage_first(const Stage& S, const WorkChunk* chunks, const ClassSeg* segs,
                                            const float* rec32, int k, int ch, bool issue = true) {
  if (threadIdx.x == 0 && issue) {
    fence_proxy_async();  // earlier generic-proxy reads of that buffer are done (warp-synchronous)
    const ChunkRef r = chunk_ref(chunks, segs, rec32, ch);
    bulk_load(S.buf(k), r.src, r.bytes, &S.bar[k & 1]);
  }
}

// The molecule owning a work item / sorted point / tile: the last entry whose start is <= x
// (molecules without work share their start with the next one and are never returned).
__device__ __forceinline__ int mol_of_item(const MolWork* __restrict__ mw, int nmol, int64_t x) {
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mw[mid].item0 <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}
__device__ __forceinline__ int mol_of_point(const MolWork* __restrict__ mw, int nmol, int64_t x) {
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mw[mid].p0 <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}
__device__ __forceinline__ int mol_of_tile(const MolWork* __restrict__ mw, int nmol, int64_t x) {
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mw[mid].tile0 <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Next work item of a persistent CTA: (tile, split) pairs, taken from a device counter.
__device__ __forceinline__ int64_t next_item(unsigned long long* work) {
  unsigned long long it = 0;
  if (threadIdx.x == 0) it = atomicAdd(work, 1ull);
  return static_cast<int64_t>(__shfl_sync(0xffffffffu, it, 0));
}

// Before working on chunk k: start the copy of the next chunk into the other buffer, then wait
// for this one. Returns false if the wait gave up; the other buffer's copy (if started) is then
// drained, again with a bounded wait, so no copy is left in flight when the CTA exits.
// limit / issue: the wait limit, and whether copies are started (see stage_first).
__device__ __forceinline__ bool stage_next(const Stage& S, const WorkChunk* chunks, const ClassSeg* segs,
                                           const float* rec32, int k, int next, int nchunks,
                                           int limit = kWaitLimit, bool issue = true) {
  if (threadIdx.x == 0 && next < nchunks && issue) {
    fence_proxy_async();  // the generic-proxy reads of that buffer (chunk k-1) are done
    const ChunkRef r = chunk_ref(chunks, segs, rec32, next);
    bulk_load(S.buf(k + 1), r.src, r.bytes, &S.bar[(k + 1) & 1]);
  }
  if (mbar_wait(&S.bar[k & 1], static_cast<uint32_t>((k >> 1) & 1), limit)) return true;
  if (next < nchunks) mbar_wait(&S.bar[(k + 1) & 1], static_cast<uint32_t>(((k + 1) >> 1) & 1), limit);
  return false;
}

// ---------------------------------------------------------------- double-float arithmetic
struct f2 {
  float hi, lo;
};
__device__ __forceinline__ f2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ f2 fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ f2 df_add(f2 x, f2 y) {
  const f2 s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ f2 df_mul(f2 x, f2 y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ f2 df_sqr(f2 x) {
  const float p = __fmul_rn(x.hi, x.hi);
  float e = __fmaf_rn(x.hi, x.hi, -p);
  e = __fmaf_rn(__fadd_rn(x.hi, x.hi), x.lo, e);
  return {p, e};
}

// 2^y in double-float for y <= 0: y = n + j/256 + g, |g| <= 1/512;
// 2^g = e^x, x = g ln2 (double-float), e^x = 1 + x + x^2/2 + x^3/6 + x^4/24 (tail in FP32).
__device__ __forceinline__ f2 df_exp2(f2 y, int ks, const float2* __restrict__ tab) {
  const float n = rintf(y.hi);
  if (n + static_cast<float>(ks) < -125.0f) return {0.0f, 0.0f};  // compared in FP32: n may be huge
  const float f = __fsub_rn(y.hi, n);  // exact
  const float j = rintf(__fmul_rn(f, 256.0f));
  const float g = __fsub_rn(f, __fmul_rn(j, 0.00390625f));  // exact
  const float kLn2Hi = 0.693147182464599609375f, kLn2Lo = -1.904654323148236e-09f;
  const float xh = __fmul_rn(g, kLn2Hi);
  float xl = __fmaf_rn(g, kLn2Hi, -xh);
  xl = __fmaf_rn(g, kLn2Lo, xl);
  xl = __fmaf_rn(y.lo, kLn2Hi, xl);
  const f2 x = fast_two_sum(xh, xl);
  float q = __fmaf_rn(x.hi, 0.041666666666666664f, 0.16666666666666666f);
  q = __fmaf_rn(x.hi, q, 0.5f);
  q = __fmul_rn(__fmul_rn(x.hi, x.hi), q);
  q = __fmaf_rn(x.hi, x.lo, q);
  const f2 s = two_sum(1.0f, x.hi);
  const f2 ex = fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, q)));
  const float2 T = tab[static_cast<int>(j) + kExpTab / 2];
  const f2 r = df_mul({T.x, T.y}, ex);
  const float sc = __int_as_float(min(static_cast<int>(n) + ks + 127, 254) << 23);  // 2^(n + ks)
  return {__fmul_rn(r.hi, sc), __fmul_rn(r.lo, sc)};
}

// log2 upper bound of |A'| E prod_d P_d over a box lo[3], hi[3] of points, from an FP32 record
// (mixed_eval.cu: u = s (r + d), E = 2^(-|u|^2), P_d = sum_k |Cn_dk| |u_d|^k): la + sum_d
// [L_d log2 max(1, M_d) - m_d^2] with m_d / M_d the smallest / largest |u_d| over the box, widened
// by a relative and absolute 1e-5; *lerr gets the log2 bound of the FP32 error bound e over the box
// and *umax the largest M_d.
__device__ __forceinline__ float log2_bound(const float* __restrict__ R, const int L[3], const float* box,
                                           float* lerr = nullptr, float* umax = nullptr) {
  float lb = R[10] + 0.02f;
  float y2 = 0.0f, mm = 0.0f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float s = R[0], b = R[2 + d];
    const float a0 = fmaf(s, box[d], b), a1 = fmaf(s, box[3 + d], b);
    float m = (a0 <= 0.0f && a1 >= 0.0f) ? 0.0f : fminf(fabsf(a0), fabsf(a1));
    float M = fmaxf(fabsf(a0), fabsf(a1));
    m = fmaxf(0.0f, m * (1.0f - 1e-5f) - 1e-5f);
    M = M * (1.0f + 1e-5f) + 1e-5f;
    lb += static_cast<float>(L[d]) * __log2f(fmaxf(M, 1.0f)) - m * m;
    y2 = fmaf(M, M, y2);
    mm = fmaxf(mm, M);
  }
  if (umax) *umax = mm;
  if (lerr) *lerr = lb - 24.0f + __log2f(static_cast<float>(10 + 2 * (L[0] + L[1] + L[2])) + 3.0f * y2) + 0.02f;
  return lb;
}

}  // namespace
}  // namespace inca
