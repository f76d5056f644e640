// A small multilayer perceptron trained and evaluated on the GPU by this library's own kernels:
// nin -> nhidden (tanh) -> nhidden (tanh) -> nout (linear), FP32, mean-squared-error loss, Adam.
// It predicts per-centre radial-grid parameters for the automatic multicentre grids (see
// inca_parallel_gb300/learned_grid.py); no counterpart in the reference, whose mod_autogrid
// (src/mod_autogrid.f90:12-185) sets every centre's radial scale from Bragg-Slater radii.
//
// Every reduction runs in a fixed order (one thread per output element looping over the
// batch), so training is deterministic: the same data, seed and settings give the same
// weights bit for bit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "inca_internal.h"

struct inca_mlp {
  int device = 0;
  int nin = 0, nh = 0, nout = 0;
  cudaStream_t stream = nullptr;
  // parameters (contiguous): W1 [nh x nin], b1 [nh], W2 [nh x nh], b2 [nh], W3 [nout x nh], b3 [nout]
  inca::DevBuf<float> params, grad, m1, m2;
  int64_t nparam = 0;
  int64_t adam_t = 0;
  // activations and deltas for a batch
  inca::DevBuf<float> x, t, a1, a2, y, d1, d2, dy;
  inca::DevBuf<float> data_x, data_t;
  inca::DevBuf<int64_t> idx;
  inca::DevBuf<float> loss;
  int64_t cap = 0;
};

namespace inca {
namespace {

enum Act { kLinear = 0, kTanh = 1 };

// out[n][m] = act(sum_k W[m][k] in[n][k] + b[m]); one thread per (n, m)
__global__ void k_dense(int64_t n, int K, int M, const float* __restrict__ in, const float* __restrict__ W,
                        const float* __restrict__ b, int act, float* out) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n * M) return;
  const int64_t s = i / M;
  const int m = static_cast<int>(i - s * M);
  float z = b[m];
  for (int k = 0; k < K; ++k) z = fmaf(W[m * K + k], in[s * K + k], z);
  out[i] = act == kTanh ? tanhf(z) : z;
}

// dy = 2 (y - t) / n (gradient of the mean squared error); loss summed in a fixed order
__global__ void k_mse(int64_t n, int M, const float* __restrict__ y, const float* __restrict__ t, float* dy,
                      float* loss) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < n * M) dy[i] = 2.0f * (y[i] - t[i]) / static_cast<float>(n);
  if (i == 0 && loss) {
    double s = 0.0;
    for (int64_t j = 0; j < n * M; ++j) {
      const double d = static_cast<double>(y[j]) - static_cast<double>(t[j]);
      s += d * d;
    }
    *loss = static_cast<float>(s / static_cast<double>(n));
  }
}

// dW[m][k] = sum_s delta[s][m] in[s][k], db[m] = sum_s delta[s][m]; one thread per (m, k) or m
__global__ void k_grad_w(int64_t n, int K, int M, const float* __restrict__ delta, const float* __restrict__ in,
                         float* dW, float* db) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < M * K) {
    const int m = i / K, k = i - m * K;
    float s = 0.0f;
    for (int64_t r = 0; r < n; ++r) s = fmaf(delta[r * M + m], in[r * K + k], s);
    dW[i] = s;
  } else if (i < M * K + M) {
    const int m = i - M * K;
    float s = 0.0f;
    for (int64_t r = 0; r < n; ++r) s += delta[r * M + m];
    db[m] = s;
  }
}

// d_in[s][k] = (sum_m W[m][k] delta[s][m]) * (1 - a_in[s][k]^2)  (through the tanh of the layer below)
__global__ void k_backprop_tanh(int64_t n, int K, int M, const float* __restrict__ delta, const float* __restrict__ W,
                                const float* __restrict__ a_in, float* d_in) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n * K) return;
  const int64_t s = i / K;
  const int k = static_cast<int>(i - s * K);
  float g = 0.0f;
  for (int m = 0; m < M; ++m) g = fmaf(W[m * K + k], delta[s * M + m], g);
  const float a = a_in[i];
  d_in[i] = g * (1.0f - a * a);
}

__global__ void k_adam(int64_t np, float* p, const float* __restrict__ g, float* m1, float* m2, float lr, float b1,
                       float b2, float c1, float c2, float eps) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= np) return;
  const float gi = g[i];
  m1[i] = b1 * m1[i] + (1.0f - b1) * gi;
  m2[i] = b2 * m2[i] + (1.0f - b2) * gi * gi;
  const float mh = m1[i] / c1, vh = m2[i] / c2;
  p[i] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void k_gather_rows(int64_t n, int D, const int64_t* __restrict__ idx, const float* __restrict__ src,
                              float* dst) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n * D) return;
  const int64_t r = i / D;
  dst[i] = src[idx[r] * D + (i - r * D)];
}

inline unsigned nb(int64_t n) { return static_cast<unsigned>((n + 255) / 256); }

struct Layout {
  int64_t W1, b1, W2, b2, W3, b3, total;
};
Layout layout(int nin, int nh, int nout) {
  Layout L;
  L.W1 = 0;
  L.b1 = L.W1 + static_cast<int64_t>(nh) * nin;
  L.W2 = L.b1 + nh;
  L.b2 = L.W2 + static_cast<int64_t>(nh) * nh;
  L.W3 = L.b2 + nh;
  L.b3 = L.W3 + static_cast<int64_t>(nout) * nh;
  L.total = L.b3 + nout;
  return L;
}

cudaError_t reserve_batch(inca_mlp* m, int64_t n) {
  if (n <= m->cap) return cudaSuccess;
  cudaError_t e = m->x.reserve(n * m->nin);
  if (!e) e = m->t.reserve(n * m->nout);
  if (!e) e = m->a1.reserve(n * m->nh);
  if (!e) e = m->a2.reserve(n * m->nh);
  if (!e) e = m->y.reserve(n * m->nout);
  if (!e) e = m->d1.reserve(n * m->nh);
  if (!e) e = m->d2.reserve(n * m->nh);
  if (!e) e = m->dy.reserve(n * m->nout);
  if (!e) m->cap = n;
  return e;
}

// forward of n rows already in m->x
void forward(inca_mlp* m, int64_t n) {
  const Layout L = layout(m->nin, m->nh, m->nout);
  float* P = m->params.p;
  k_dense<<<nb(n * m->nh), 256, 0, m->stream>>>(n, m->nin, m->nh, m->x.p, P + L.W1, P + L.b1, kTanh, m->a1.p);
  k_dense<<<nb(n * m->nh), 256, 0, m->stream>>>(n, m->nh, m->nh, m->a1.p, P + L.W2, P + L.b2, kTanh, m->a2.p);
  k_dense<<<nb(n * m->nout), 256, 0, m->stream>>>(n, m->nh, m->nout, m->a2.p, P + L.W3, P + L.b3, kLinear, m->y.p);
}

// gradient of the mean squared error over n rows in m->x, m->t into m->grad (and loss)
void backward(inca_mlp* m, int64_t n, float* loss) {
  const Layout L = layout(m->nin, m->nh, m->nout);
  float* P = m->params.p;
  float* G = m->grad.p;
  k_mse<<<nb(n * m->nout), 256, 0, m->stream>>>(n, m->nout, m->y.p, m->t.p, m->dy.p, loss);
  k_grad_w<<<nb(m->nout * m->nh + m->nout), 256, 0, m->stream>>>(n, m->nh, m->nout, m->dy.p, m->a2.p, G + L.W3,
                                                                  G + L.b3);
  k_backprop_tanh<<<nb(n * m->nh), 256, 0, m->stream>>>(n, m->nh, m->nout, m->dy.p, P + L.W3, m->a2.p, m->d2.p);
  k_grad_w<<<nb(m->nh * m->nh + m->nh), 256, 0, m->stream>>>(n, m->nh, m->nh, m->d2.p, m->a1.p, G + L.W2, G + L.b2);
  k_backprop_tanh<<<nb(n * m->nh), 256, 0, m->stream>>>(n, m->nh, m->nh, m->d2.p, P + L.W2, m->a1.p, m->d1.p);
  k_grad_w<<<nb(m->nh * m->nin + m->nh), 256, 0, m->stream>>>(n, m->nin, m->nh, m->d1.p, m->x.p, G + L.W1, G + L.b1);
}

// splitmix64 (seeded parameter initialisation and shuffles on the host)
uint64_t mix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform(uint64_t& s) { return static_cast<double>(mix(s) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace
}  // namespace inca

using namespace inca;

extern "C" {

int inca_mlp_create(inca_mlp** out, int device, int32_t nin, int32_t nhidden, int32_t nout, uint64_t seed) {
  if (!out || nin < 1 || nhidden < 1 || nout < 1 || nin > 1024 || nhidden > 1024 || nout > 64) return INCA_E_ARG;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return INCA_E_CUDA;
  inca_mlp* m = new inca_mlp;
  m->device = device;
  m->nin = nin;
  m->nh = nhidden;
  m->nout = nout;
  const Layout L = layout(nin, nhidden, nout);
  m->nparam = L.total;
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess || m->params.reserve(L.total) ||
      m->grad.reserve(L.total) || m->m1.reserve(L.total) || m->m2.reserve(L.total) || m->loss.reserve(1)) {
    delete m;
    return INCA_E_NOMEM;
  }
  // Glorot-uniform weights, zero biases
  std::vector<float> h(L.total, 0.0f);
  uint64_t s = seed;
  auto fill = [&](int64_t off, int rows, int cols) {
    const double a = std::sqrt(6.0 / double(rows + cols));
    for (int64_t i = 0; i < static_cast<int64_t>(rows) * cols; ++i)
      h[off + i] = static_cast<float>((2.0 * uniform(s) - 1.0) * a);
  };
  fill(L.W1, nhidden, nin);
  fill(L.W2, nhidden, nhidden);
  fill(L.W3, nout, nhidden);
  cudaMemcpy(m->params.p, h.data(), sizeof(float) * L.total, cudaMemcpyHostToDevice);
  cudaMemset(m->m1.p, 0, sizeof(float) * L.total);
  cudaMemset(m->m2.p, 0, sizeof(float) * L.total);
  *out = m;
  return INCA_OK;
}

int inca_mlp_destroy(inca_mlp* m) {
  if (!m) return INCA_E_ARG;
  cudaSetDevice(m->device);
  for (auto* b : {&m->params, &m->grad, &m->m1, &m->m2, &m->x, &m->t, &m->a1, &m->a2, &m->y, &m->d1, &m->d2, &m->dy,
                  &m->data_x, &m->data_t, &m->loss})
    b->release();
  m->idx.release();
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return INCA_OK;
}

int inca_mlp_param_count(inca_mlp* m, int64_t* count) {
  if (!m || !count) return INCA_E_ARG;
  *count = m->nparam;
  return INCA_OK;
}

int inca_mlp_get_params(inca_mlp* m, float* params) {
  if (!m || !params) return INCA_E_ARG;
  cudaSetDevice(m->device);
  return cudaMemcpy(params, m->params.p, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost) ? INCA_E_CUDA : INCA_OK;
}

int inca_mlp_set_params(inca_mlp* m, const float* params) {
  if (!m || !params) return INCA_E_ARG;
  cudaSetDevice(m->device);
  return cudaMemcpy(m->params.p, params, sizeof(float) * m->nparam, cudaMemcpyHostToDevice) ? INCA_E_CUDA : INCA_OK;
}

int inca_mlp_forward(inca_mlp* m, int64_t n, const float* X, float* Y) {
  if (!m || n < 0 || (n > 0 && (!X || !Y))) return INCA_E_ARG;
  if (n == 0) return INCA_OK;
  cudaSetDevice(m->device);
  if (reserve_batch(m, n)) return INCA_E_NOMEM;
  cudaError_t e = cudaMemcpyAsync(m->x.p, X, sizeof(float) * n * m->nin, cudaMemcpyHostToDevice, m->stream);
  if (!e) {
    forward(m, n);
    e = cudaGetLastError();
  }
  if (!e) e = cudaMemcpyAsync(Y, m->y.p, sizeof(float) * n * m->nout, cudaMemcpyDeviceToHost, m->stream);
  if (!e) e = cudaStreamSynchronize(m->stream);
  return e ? INCA_E_CUDA : INCA_OK;
}

int inca_mlp_gradient(inca_mlp* m, int64_t n, const float* X, const float* T, float* loss, float* grad) {
  if (!m || n < 1 || !X || !T) return INCA_E_ARG;
  cudaSetDevice(m->device);
  if (reserve_batch(m, n)) return INCA_E_NOMEM;
  cudaError_t e = cudaMemcpyAsync(m->x.p, X, sizeof(float) * n * m->nin, cudaMemcpyHostToDevice, m->stream);
  if (!e) e = cudaMemcpyAsync(m->t.p, T, sizeof(float) * n * m->nout, cudaMemcpyHostToDevice, m->stream);
  if (!e) {
    forward(m, n);
    backward(m, n, m->loss.p);
    e = cudaGetLastError();
  }
  if (!e && loss) e = cudaMemcpyAsync(loss, m->loss.p, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (!e && grad) e = cudaMemcpyAsync(grad, m->grad.p, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost, m->stream);
  if (!e) e = cudaStreamSynchronize(m->stream);
  return e ? INCA_E_CUDA : INCA_OK;
}

int inca_mlp_train(inca_mlp* m, int64_t n, const float* X, const float* T, int32_t epochs, int32_t batch, float lr,
                   uint64_t seed, float* final_loss) {
  if (!m || n < 1 || !X || !T || epochs < 1 || batch < 1 || !(lr > 0.0f)) return INCA_E_ARG;
  cudaSetDevice(m->device);
  const int64_t bs = std::min<int64_t>(batch, n);
  if (reserve_batch(m, std::max(bs, n)) || m->data_x.reserve(n * m->nin) || m->data_t.reserve(n * m->nout) ||
      m->idx.reserve(n))
    return INCA_E_NOMEM;
  cudaError_t e = cudaMemcpyAsync(m->data_x.p, X, sizeof(float) * n * m->nin, cudaMemcpyHostToDevice, m->stream);
  if (!e) e = cudaMemcpyAsync(m->data_t.p, T, sizeof(float) * n * m->nout, cudaMemcpyHostToDevice, m->stream);
  std::vector<int64_t> perm(n);
  for (int64_t i = 0; i < n; ++i) perm[i] = i;
  uint64_t s = seed;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs && !e; ++ep) {
    for (int64_t i = n - 1; i > 0; --i) std::swap(perm[i], perm[static_cast<int64_t>(uniform(s) * double(i + 1))]);
    e = cudaMemcpyAsync(m->idx.p, perm.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, m->stream);
    for (int64_t o = 0; o < n && !e; o += bs) {
      const int64_t nn = std::min(bs, n - o);
      k_gather_rows<<<nb(nn * m->nin), 256, 0, m->stream>>>(nn, m->nin, m->idx.p + o, m->data_x.p, m->x.p);
      k_gather_rows<<<nb(nn * m->nout), 256, 0, m->stream>>>(nn, m->nout, m->idx.p + o, m->data_t.p, m->t.p);
      forward(m, nn);
      backward(m, nn, nullptr);
      ++m->adam_t;
      const float c1 = 1.0f - std::pow(b1, static_cast<float>(m->adam_t));
      const float c2 = 1.0f - std::pow(b2, static_cast<float>(m->adam_t));
      k_adam<<<nb(m->nparam), 256, 0, m->stream>>>(m->nparam, m->params.p, m->grad.p, m->m1.p, m->m2.p, lr, b1, b2, c1,
                                                   c2, eps);
      e = cudaGetLastError();
    }
    if (!e) e = cudaStreamSynchronize(m->stream);  // the permutation buffer is reused next epoch
  }
  if (!e && final_loss) {  // loss over the whole training set
    e = cudaMemcpyAsync(m->x.p, m->data_x.p, sizeof(float) * n * m->nin, cudaMemcpyDeviceToDevice, m->stream);
    if (!e) e = cudaMemcpyAsync(m->t.p, m->data_t.p, sizeof(float) * n * m->nout, cudaMemcpyDeviceToDevice, m->stream);
    if (!e) {
      forward(m, n);
      k_mse<<<nb(n * m->nout), 256, 0, m->stream>>>(n, m->nout, m->y.p, m->t.p, m->dy.p, m->loss.p);
      e = cudaMemcpyAsync(final_loss, m->loss.p, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
    }
    if (!e) e = cudaStreamSynchronize(m->stream);
  }
  return e ? INCA_E_CUDA : INCA_OK;
}

}  // extern "C"
