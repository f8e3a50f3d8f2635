// Learned coarse correction for the V-cycle (no counterpart in the
// reference, whose coarse correction is min(50, n) Jacobi sweeps on the
// coarsest level, cons/mgpcg_gpu.py:216-224).  A 3-layer message-passing
// network over the graph of the level-1 (aggregate) matrix A_c computes, once
// per matrix, one weight per aggregate; each V-cycle then applies the linear
// correction e = w * r / diag(A_c), with w_i = c_i sigmoid(y_i) in (0, c_i),
// c_i = 1.9 / sum_j |Ah_ij| (below 2 / sum_j |Ah_ij| the correction cannot
// over-correct a mode, so the V-cycle stays positive definite).  Forward, backward and Adam run
// on the GPU (mpnn.cu); the dense layers run on the tensor cores (bf16
// operands, float32 accumulation).
//
// Network on a scalar node field r (n aggregates, F = 64), with
// s_i = sqrt(1/A_ii) and Ah = S A S:
//   sigma = rms(S r),  u = S r / sigma,  a1 = Ah u
//   H1 = relu(u w1s + a1 w1n + b1)
//   H2 = relu([H1, Ah H1] W2 + b2),  H3 = relu([H2, Ah H2] W3 + b3)
//   y  = H3 wo + bo,  e = sigma S y
// The network's y is taken on the field r = sqrt(diag A) (u = 1, a1 = row
// sums of Ah).  Training loss over a batch of restricted residuals r_s, with
// u_s = S r_s / sigma_s and v_s = w * u_s:
//   L = mean_s (1/2 v_s^T Ah v_s - v_s^T u_s) / n
// (the coarse energy of the correction, scaled; minimised by A_c^-1 r).
// The "field" mode trains the network as a map r -> e instead, with
// L = mean_s (1/2 y^T Ah y - y^T u_s) / n.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "common.h"

namespace mgpbd {

constexpr int kNetF = 64;
// parameter vector layout (float32), also the gradient layout
constexpr int kNetOffW1s = 0, kNetOffW1n = 64, kNetOffB1 = 128;
constexpr int kNetOffW2 = 192;
constexpr int kNetOffB2 = kNetOffW2 + 2 * kNetF * kNetF;
constexpr int kNetOffW3 = kNetOffB2 + kNetF;
constexpr int kNetOffB3 = kNetOffW3 + 2 * kNetF * kNetF;
constexpr int kNetOffWo = kNetOffB3 + kNetF;
constexpr int kNetOffBo = kNetOffWo + kNetF;
constexpr int kNetParams = kNetOffBo + 1;  // 16,769
constexpr int kNetModeWeights = 0;  // loss of the per-aggregate weights
constexpr int kNetModeField = 1;    // loss of the map r -> e

// The aggregate graph: a CSR matrix with its 1/diag (device arrays).
struct NetGraph {
  int32_t n = 0;
  int64_t nnz = 0;
  const int32_t* indptr = nullptr;
  const int32_t* indices = nullptr;
  const float* data = nullptr;
  const float* diag_inv = nullptr;
};

class CoarseNet {
 public:
  // Glorot-uniform weights from `seed`, zero biases.
  explicit CoarseNet(uint64_t seed);
  CoarseNet(const CoarseNet&) = delete;
  CoarseNet& operator=(const CoarseNet&) = delete;

  float* params() const { return p_.p; }
  float* grad() const { return g_.p; }
  // refresh the bf16 tensor-core copies of W2, W3 after params changed
  void sync_params(cudaStream_t s);
  // w = per-aggregate weights of the graph (device vector of g.n)
  void weights(const NetGraph& g, float* w, cudaStream_t s);
  // e = the network applied to the field r (device vectors of g.n)
  void forward(const NetGraph& g, const float* r, float* e, cudaStream_t s);
  // loss (device double, at loss_dev) and gradient (grad()) of the batch of
  // residuals first, first + 1, ... first + batch - 1 (indices mod
  // n_samples) of the n_samples stored back to back; grad is overwritten
  void loss_grad(const NetGraph& g, const float* samples, int32_t n_samples, int32_t first,
                 int32_t batch, double* loss_dev, int32_t mode, cudaStream_t s);
  // `steps` Adam steps, step k on the batch starting at sample k * batch;
  // losses_dev[k] gets step k's loss
  void train(const NetGraph& g, const float* samples, int32_t n_samples, int32_t batch,
             int32_t steps, float lr, double* losses_dev, cudaStream_t s);
  // one bias-corrected Adam step on params() from grad(); refreshes bf16 copies
  void adam(float lr, float beta1, float beta2, float eps, cudaStream_t s);
  int64_t adam_steps() const { return t_; }
  void reset_adam(cudaStream_t s);

 private:
  void ensure(const NetGraph& g);
  void run_forward(const NetGraph& g, const float* r, float* e, float* y_out, bool train,
                   float* cap_out, cudaStream_t s);
  void backward_layers(const NetGraph& g, cudaStream_t s);

  DevBuf<float> p_, g_, m_, v_;
  DevBuf<__nv_bfloat16> wt_;  // W2^T then W3^T, each [64 out][128 in]
  int32_t cap_ = -1;
  // workspace (cap_ rows)
  DevBuf<double> part_, sumsq_;
  DevBuf<float> u_, a1_, y_, e_, h3_, gy_, gz_, gself_, q_, wpart_;
  DevBuf<float> ah_;    // Ah = S A S per nonzero, written by layer 1
  DevBuf<float> feat_;  // the feature field sqrt(diag A)
  DevBuf<float> wcap_, wv_, dw_;  // weight bound, squashed weights, dw/dy
  DevBuf<__nv_bfloat16> h1_, g1_, h2_, g2_;
  int64_t t_ = 0;
};

// e = max(w, 0) * diag_inv * r: the coarse correction of the weights
void apply_coarse_weights(int32_t n, const float* w, const float* diag_inv, const float* r,
                          float* e, cudaStream_t s);

}  // namespace mgpbd
