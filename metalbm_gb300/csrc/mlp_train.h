// GPU training of the alpha-guess MLP with the library's own kernels
// (forward, backward, deterministic gradient reduction, Adam).
#pragma once

#include <cuda_runtime.h>

#include "../../include/mlbm/mlbm.h"
#include "mlp_device.cuh"

namespace mlbm {

// Parameter vector: W1 [32][n_in], b1 [32], W2 [32][32], b2 [32], w3 [32], b3.
inline int mlp_param_count(int n_in) { return 32 * n_in + 32 + 32 * 32 + 32 + 32 + 1; }

struct MlpTrainer {
  int n_in = 0;
  long long cap = 0;     // batch capacity
  long long n = 0;       // samples
  cudaStream_t s = nullptr;
  unsigned launches = 0;
  float* X = nullptr;    // [n][n_in]
  float* y = nullptr;    // [n]
  float* theta = nullptr;
  float* grad = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  float* scale = nullptr;  // input scale [n_in]
  float out_scale = 1.0f;
  float* Xb = nullptr;
  float* yb = nullptr;
  float* H1 = nullptr;
  float* H2 = nullptr;
  float* dH1 = nullptr;
  float* dH2 = nullptr;
  float* dY = nullptr;
  float* L = nullptr;
  float* loss = nullptr;
  long long* perm = nullptr;
  mlbm_mlp model{};

  cudaError_t init(int n_in, long long batch, cudaStream_t stream);
  cudaError_t set_data(const float* X, const float* y, long long n);
  cudaError_t set_model(const mlbm_mlp& m);
  cudaError_t gradient(long long nb, float* loss_out);  // on the first nb samples
  cudaError_t train(const mlbm_train_cfg& cfg, float* last_loss);
  cudaError_t get_model(mlbm_mlp* out);
  cudaError_t get_gradient(mlbm_mlp* out);
  void release();
};

// Inference with the fused kernel's BF16 tensor-core path.
cudaError_t mlp_predict(const MlpDev* m, int n_in, const float* X, long long n, float* out,
                        cudaStream_t s);

void count_launches(unsigned n);

}  // namespace mlbm
