// Training kernels of the alpha-guess MLP: forward + backward per sample,
// gradient reduction in a fixed order (so a gradient is reproducible bit for
// bit), Adam (Kingma & Ba, 2015). FP32 master weights; inference quantises
// them to BF16 (mlp_device.cuh).

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "mlp_train.h"

namespace mlbm {

constexpr int PMAX = 32 * MLBM_MLP_MAX_IN + 32 + 32 * 32 + 32 + 32 + 1;

struct Offsets {
  int w1, b1, w2, b2, w3, b3;
  __host__ __device__ explicit Offsets(int n_in) {
    w1 = 0; b1 = 32 * n_in; w2 = b1 + 32; b2 = w2 + 32 * 32; w3 = b2 + 32; b3 = w3 + 32;
  }
};

__global__ void __launch_bounds__(128) fwd_bwd_kernel(const float* __restrict__ theta, int n_in,
                                                      const float* __restrict__ X,
                                                      const float* __restrict__ y,
                                                      const float* __restrict__ scale,
                                                      float out_scale, long long nb, float inv_n,
                                                      float* H1, float* H2, float* dH1, float* dH2,
                                                      float* dY, float* L) {
  __shared__ float th[PMAX];
  const Offsets o(n_in);
  const int P = o.b3 + 1;
  for (int i = threadIdx.x; i < P; i += blockDim.x) th[i] = theta[i];
  __syncthreads();
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  float x[MLBM_MLP_MAX_IN];
  for (int i = 0; i < n_in; ++i) x[i] = X[b * n_in + i] * scale[i];
  float h1[32], h2[32];
  for (int j = 0; j < 32; ++j) {
    float a = th[o.b1 + j];
    for (int i = 0; i < n_in; ++i) a = fmaf(th[o.w1 + j * n_in + i], x[i], a);
    h1[j] = tanhf(a);
  }
  float yv = th[o.b3];
  for (int k = 0; k < 32; ++k) {
    float a = th[o.b2 + k];
    for (int j = 0; j < 32; ++j) a = fmaf(th[o.w2 + k * 32 + j], h1[j], a);
    h2[k] = tanhf(a);
    yv = fmaf(th[o.w3 + k], h2[k], yv);
  }
  const float e = 2.0f + out_scale * yv - y[b];
  L[b] = e * e;
  const float dy = 2.0f * e * out_scale * inv_n;
  dY[b] = dy;
  float dh2[32];
  for (int k = 0; k < 32; ++k) {
    dh2[k] = dy * th[o.w3 + k] * (1.0f - h2[k] * h2[k]);
    H2[b * 32 + k] = h2[k];
    dH2[b * 32 + k] = dh2[k];
  }
  for (int j = 0; j < 32; ++j) {
    float a = 0.0f;
    for (int k = 0; k < 32; ++k) a = fmaf(th[o.w2 + k * 32 + j], dh2[k], a);
    H1[b * 32 + j] = h1[j];
    dH1[b * 32 + j] = a * (1.0f - h1[j] * h1[j]);
  }
}

// One block per parameter row; each thread sums its column over the batch in
// order b = 0..nb-1 (deterministic).
__global__ void grad_kernel(int n_in, const float* __restrict__ X, const float* __restrict__ scale,
                            long long nb, const float* __restrict__ H1, const float* __restrict__ H2,
                            const float* __restrict__ dH1, const float* __restrict__ dH2,
                            const float* __restrict__ dY, float* __restrict__ grad) {
  const Offsets o(n_in);
  const int r = blockIdx.x, t = threadIdx.x;
  if (r < 32) {  // W1 row r (t < n_in) and b1[r] (t == n_in)
    if (t > n_in) return;
    float s = 0.0f;
    if (t < n_in) {
      for (long long b = 0; b < nb; ++b) s = fmaf(dH1[b * 32 + r], X[b * n_in + t] * scale[t], s);
      grad[o.w1 + r * n_in + t] = s;
    } else {
      for (long long b = 0; b < nb; ++b) s += dH1[b * 32 + r];
      grad[o.b1 + r] = s;
    }
  } else if (r < 64) {  // W2 row k (t < 32) and b2[k] (t == 32)
    const int k = r - 32;
    if (t > 32) return;
    float s = 0.0f;
    if (t < 32) {
      for (long long b = 0; b < nb; ++b) s = fmaf(dH2[b * 32 + k], H1[b * 32 + t], s);
      grad[o.w2 + k * 32 + t] = s;
    } else {
      for (long long b = 0; b < nb; ++b) s += dH2[b * 32 + k];
      grad[o.b2 + k] = s;
    }
  } else {  // w3 (t < 32) and b3 (t == 32)
    if (t > 32) return;
    float s = 0.0f;
    if (t < 32) {
      for (long long b = 0; b < nb; ++b) s = fmaf(dY[b], H2[b * 32 + t], s);
      grad[o.w3 + t] = s;
    } else {
      for (long long b = 0; b < nb; ++b) s += dY[b];
      grad[o.b3] = s;
    }
  }
}

__global__ void sum_kernel(const float* __restrict__ v, long long n, float scale_out,
                           float* __restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s += v[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = (float)(sh[0] * scale_out);
}

__global__ void adam_kernel(float* __restrict__ theta, const float* __restrict__ g,
                            float* __restrict__ m1, float* __restrict__ m2, int P, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.0f - b1) * gi;
  const float v = b2 * m2[i] + (1.0f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = v;
  theta[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

__global__ void gather_kernel(const float* __restrict__ X, const float* __restrict__ y,
                              const long long* __restrict__ perm, long long off, long long nb,
                              int n_in, float* __restrict__ Xb, float* __restrict__ yb) {
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const long long s = perm[off + b];
  for (int i = 0; i < n_in; ++i) Xb[b * n_in + i] = X[s * n_in + i];
  yb[b] = y[s];
}

template <int Q>
__global__ void __launch_bounds__(128) predict_kernel(const MlpDev* __restrict__ m,
                                                      const float* __restrict__ X, long long n,
                                                      float* __restrict__ out) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float x[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) x[i] = s < n ? X[s * Q + i] : 0.0f;
  const float g = mlp_guess_block<Q>(m, x);
  if (s < n) out[s] = 2.0f + g;
}

cudaError_t mlp_predict(const MlpDev* m, int n_in, const float* X, long long n, float* out,
                        cudaStream_t s) {
  const unsigned grid = (unsigned)((n + 127) / 128);
  switch (n_in) {
    case 9: predict_kernel<9><<<grid, 128, 0, s>>>(m, X, n, out); break;
    case 19: predict_kernel<19><<<grid, 128, 0, s>>>(m, X, n, out); break;
    case 27: predict_kernel<27><<<grid, 128, 0, s>>>(m, X, n, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---- trainer ------------------------------------------------------------------
static cudaError_t dalloc(void** p, size_t bytes) { return cudaMalloc(p, bytes); }

cudaError_t MlpTrainer::init(int nin, long long batch, cudaStream_t stream) {
  n_in = nin;
  cap = batch;
  s = stream;
  const int P = mlp_param_count(n_in);
  cudaError_t e;
  if ((e = dalloc((void**)&theta, sizeof(float) * P)) || (e = dalloc((void**)&grad, sizeof(float) * P)) ||
      (e = dalloc((void**)&m1, sizeof(float) * P)) || (e = dalloc((void**)&m2, sizeof(float) * P)) ||
      (e = dalloc((void**)&scale, sizeof(float) * n_in)) ||
      (e = dalloc((void**)&Xb, sizeof(float) * cap * n_in)) || (e = dalloc((void**)&yb, sizeof(float) * cap)) ||
      (e = dalloc((void**)&H1, sizeof(float) * cap * 32)) || (e = dalloc((void**)&H2, sizeof(float) * cap * 32)) ||
      (e = dalloc((void**)&dH1, sizeof(float) * cap * 32)) || (e = dalloc((void**)&dH2, sizeof(float) * cap * 32)) ||
      (e = dalloc((void**)&dY, sizeof(float) * cap)) || (e = dalloc((void**)&L, sizeof(float) * cap)) ||
      (e = dalloc((void**)&loss, sizeof(float))))
    return e;
  cudaMemsetAsync(m1, 0, sizeof(float) * P, s);
  cudaMemsetAsync(m2, 0, sizeof(float) * P, s);
  return cudaGetLastError();
}

cudaError_t MlpTrainer::set_data(const float* hX, const float* hy, long long nn) {
  n = nn;
  cudaError_t e;
  if ((e = dalloc((void**)&X, sizeof(float) * n * n_in)) || (e = dalloc((void**)&y, sizeof(float) * n)) ||
      (e = dalloc((void**)&perm, sizeof(long long) * n)))
    return e;
  if ((e = cudaStreamSynchronize(s))) return e;
  if ((e = cudaMemcpy(X, hX, sizeof(float) * n * n_in, cudaMemcpyHostToDevice))) return e;
  return cudaMemcpy(y, hy, sizeof(float) * n, cudaMemcpyHostToDevice);
}

static void pack(const mlbm_mlp& m, int n_in, std::vector<float>& th) {
  const Offsets o(n_in);
  th.assign(mlp_param_count(n_in), 0.0f);
  for (int j = 0; j < 32; ++j) {
    for (int i = 0; i < n_in; ++i) th[o.w1 + j * n_in + i] = m.w1[j * n_in + i];
    th[o.b1 + j] = m.b1[j];
    for (int i = 0; i < 32; ++i) th[o.w2 + j * 32 + i] = m.w2[j * 32 + i];
    th[o.b2 + j] = m.b2[j];
    th[o.w3 + j] = m.w3[j];
  }
  th[o.b3] = m.b3;
}

static void unpack(const std::vector<float>& th, int n_in, mlbm_mlp* m) {
  const Offsets o(n_in);
  for (int j = 0; j < 32; ++j) {
    for (int i = 0; i < n_in; ++i) m->w1[j * n_in + i] = th[o.w1 + j * n_in + i];
    m->b1[j] = th[o.b1 + j];
    for (int i = 0; i < 32; ++i) m->w2[j * 32 + i] = th[o.w2 + j * 32 + i];
    m->b2[j] = th[o.b2 + j];
    m->w3[j] = th[o.w3 + j];
  }
  m->b3 = th[o.b3];
}

cudaError_t MlpTrainer::set_model(const mlbm_mlp& m) {
  model = m;
  out_scale = m.output_scale;
  std::vector<float> th;
  pack(m, n_in, th);
  cudaError_t e = cudaMemcpy(theta, th.data(), sizeof(float) * th.size(), cudaMemcpyHostToDevice);
  if (e) return e;
  return cudaMemcpy(scale, m.input_scale, sizeof(float) * n_in, cudaMemcpyHostToDevice);
}

cudaError_t MlpTrainer::gradient(long long nb, float* loss_out) {
  if (nb > cap) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)((nb + 127) / 128);
  fwd_bwd_kernel<<<grid, 128, 0, s>>>(theta, n_in, X, y, scale, out_scale, nb, 1.0f / (float)nb,
                                      H1, H2, dH1, dH2, dY, L);
  grad_kernel<<<65, 64, 0, s>>>(n_in, X, scale, nb, H1, H2, dH1, dH2, dY, grad);
  sum_kernel<<<1, 256, 0, s>>>(L, nb, 1.0f / (float)nb, loss);
  launches += 3;
  cudaError_t e = cudaGetLastError();
  if (e) return e;
  // the kernels run on the handle's (non-blocking) stream
  if ((e = cudaMemcpyAsync(loss_out, loss, sizeof(float), cudaMemcpyDeviceToHost, s))) return e;
  return cudaStreamSynchronize(s);
}

cudaError_t MlpTrainer::train(const mlbm_train_cfg& cfg, float* last_loss) {
  const int P = mlp_param_count(n_in);
  std::mt19937_64 rng(cfg.seed);
  std::vector<long long> idx(n);
  const long long B = cap;
  double epoch_loss = 0.0;
  long long t = 0;
  for (int ep = 0; ep < cfg.epochs; ++ep) {
    for (long long i = 0; i < n; ++i) idx[i] = i;
    std::shuffle(idx.begin(), idx.end(), rng);
    cudaError_t e = cudaMemcpyAsync(perm, idx.data(), sizeof(long long) * n, cudaMemcpyHostToDevice, s);
    if (e) return e;
    epoch_loss = 0.0;
    long long batches = 0;
    std::vector<float> losses;
    for (long long off = 0; off + B <= n || (off < n && off == 0); off += B) {
      const long long nb = std::min(B, n - off);
      const unsigned g = (unsigned)((nb + 127) / 128);
      gather_kernel<<<g, 128, 0, s>>>(X, y, perm, off, nb, n_in, Xb, yb);
      fwd_bwd_kernel<<<g, 128, 0, s>>>(theta, n_in, Xb, yb, scale, out_scale, nb, 1.0f / (float)nb,
                                       H1, H2, dH1, dH2, dY, L);
      grad_kernel<<<65, 64, 0, s>>>(n_in, Xb, scale, nb, H1, H2, dH1, dH2, dY, grad);
      ++t;
      const float c1 = 1.0f - std::pow(cfg.beta1, (float)t), c2 = 1.0f - std::pow(cfg.beta2, (float)t);
      adam_kernel<<<(P + 255) / 256, 256, 0, s>>>(theta, grad, m1, m2, P, cfg.learning_rate, cfg.beta1,
                                                  cfg.beta2, cfg.eps, c1, c2);
      sum_kernel<<<1, 256, 0, s>>>(L, nb, 1.0f / (float)nb, loss);
      launches += 5;
      float l = 0.0f;
      if ((e = cudaMemcpyAsync(&l, loss, sizeof(float), cudaMemcpyDeviceToHost, s))) return e;
      if ((e = cudaStreamSynchronize(s))) return e;
      epoch_loss += l;
      ++batches;
    }
    epoch_loss /= (double)(batches ? batches : 1);
  }
  *last_loss = (float)epoch_loss;
  return cudaGetLastError();
}

cudaError_t MlpTrainer::get_model(mlbm_mlp* out) {
  std::vector<float> th(mlp_param_count(n_in));
  cudaError_t e = cudaStreamSynchronize(s);
  if (e) return e;
  e = cudaMemcpy(th.data(), theta, sizeof(float) * th.size(), cudaMemcpyDeviceToHost);
  if (e) return e;
  *out = model;
  unpack(th, n_in, out);
  return cudaSuccess;
}

cudaError_t MlpTrainer::get_gradient(mlbm_mlp* out) {
  std::vector<float> th(mlp_param_count(n_in));
  cudaError_t e = cudaStreamSynchronize(s);
  if (e) return e;
  e = cudaMemcpy(th.data(), grad, sizeof(float) * th.size(), cudaMemcpyDeviceToHost);
  if (e) return e;
  std::memset(out, 0, sizeof *out);
  out->n_in = n_in;
  out->n_hidden = 32;
  unpack(th, n_in, out);
  return cudaSuccess;
}

void MlpTrainer::release() {
  void* ps[] = {X, y, theta, grad, m1, m2, scale, Xb, yb, H1, H2, dH1, dH2, dY, L, loss, perm};
  for (void* p : ps)
    if (p) cudaFree(p);
}

}  // namespace mlbm
