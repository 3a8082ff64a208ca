// Host side of the learned per-ommatidium denoiser (kernels in mlp.cu).
//
// Network: kFeatureWidth -> 128 -> 128 -> 128 -> 3 (output padded to 8),
// ReLU hidden layers, predicting a correction added to the 8-sample mean.
// fp32 master weights with Adam moments, bf16 working copies; every GEMM is
// bf16 x bf16 with fp32 accumulation.  Parameter vector layout (floats):
//   W1 [112 x 128] row-major (in x out), b1 [128], W2 [128 x 128], b2,
//   W3 [128 x 128], b3, W4 [128 x 8], b4 [8].
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "device_api.hpp"

namespace cr {

class Denoiser {
 public:
  static constexpr int kHidden = kMlpHidden;
  static constexpr int kOut = kMlpOut;  // 3 used
  static constexpr size_t offW1 = 0;
  static constexpr size_t offB1 = offW1 + size_t(kFeatureWidth) * kHidden;
  static constexpr size_t offW2 = offB1 + kHidden;
  static constexpr size_t offB2 = offW2 + size_t(kHidden) * kHidden;
  static constexpr size_t offW3 = offB2 + kHidden;
  static constexpr size_t offB3 = offW3 + size_t(kHidden) * kHidden;
  static constexpr size_t offW4 = offB3 + kHidden;
  static constexpr size_t offB4 = offW4 + size_t(kHidden) * kOut;
  static constexpr size_t kParams = offB4 + kOut;

  ~Denoiser() { release(); }
  void release();

  // He-normal initialisation from `seed` (output layer scaled by 0.1).
  void init(uint32_t seed, cudaStream_t s);
  bool ready() const { return params_ != nullptr; }

  // Appends rows to the training set (device arrays: X bf16 rows x 112,
  // base and target fp32 rows x 3; copied).
  void addRows(const void* X, const float* base, const float* target, size_t rows, cudaStream_t s);
  size_t rows() const { return rows_; }
  void clearRows() { rows_ = 0; }

  // `steps` Adam steps on minibatches of `batch` rows drawn by a seeded
  // shuffle of the training set; returns the mean squared error of each step
  // in `loss` (host, `steps` floats) if given.
  // tc: the GEMMs run on the tcgen05 tensor cores (gemmBf16Tc), else on
  // mma.sync (gemmBf16, the path the layer-by-layer prediction repeats).
  void train(int steps, int batch, float lr, uint32_t seed, float* loss, cudaStream_t s, bool tc = true);

  // Prediction for `rows` feature rows (device): out = base + net(X)[:, :3],
  // layer by layer.
  void infer(const void* X, const float* base, size_t rows, float* out, cudaStream_t s);

  // Current bf16 weights and fp32 biases (device pointers) for the fused
  // inference kernel.
  MlpWeights weights() const;

  // One forward/backward on the given rows with the current weights:
  // returns the loss and copies gradients and parameters to the host.
  float gradient(const void* X, const float* base, const float* target, int rows, float* gradsHost, float* paramsHost,
                 cudaStream_t s, bool tc = false);

  // Scales the output layer (W4, b4) by alpha: the network's correction
  // becomes alpha times what it was (the layer is linear); alpha 0 leaves the
  // 8-sample mean.  Refreshes the bf16 copies.
  void scaleOutput(float alpha, cudaStream_t s);

  void save(const std::string& path, cudaStream_t s);
  void load(const std::string& path, cudaStream_t s);

 private:
  void ensureBatch(int rows);
  float forwardBackward(const void* X, const float* base, const float* target, int rows, bool wantLoss,
                        cudaStream_t s);
  void step(const void* X, const float* base, const float* target, int rows, float* lossAcc, cudaStream_t s,
            const int* lossIndex = nullptr);
  void forward(const void* X, int rows, cudaStream_t s);

  float* params_ = nullptr;
  float* grads_ = nullptr;
  float* m_ = nullptr;
  float* v_ = nullptr;
  void* wbf_ = nullptr;  // bf16 copy of params_
  void* wbfT_ = nullptr;  // bf16 transposes of the weight matrices, at the same offsets
  static WeightBlocks weightBlocks() {
    return WeightBlocks{4,
                        {int(offW1), int(offW2), int(offW3), int(offW4)},
                        {kFeatureWidth, kHidden, kHidden, kHidden},
                        {kHidden, kHidden, kHidden, kOut}};
  }
  int adamT_ = 0;
  bool tc_ = false;  // GEMMs of the running train() on tcgen05
  cudaError_t gemm(int mode, int M, int N, int K, const void* A, int lda, bool aTrans, const void* B, int ldb,
                   bool bTrans, float* Cf, void* Hb, int ldc, const float* bias, const void* mask, cudaStream_t s) {
    return tc_ ? gemmBf16Tc(mode, M, N, K, A, lda, aTrans, B, ldb, bTrans, Cf, Hb, ldc, bias, mask, s)
               : gemmBf16(mode, M, N, K, A, lda, aTrans, B, ldb, bTrans, Cf, Hb, ldc, bias, mask, s);
  }
  // batch work buffers
  int cap_ = 0;
  void* Xb_ = nullptr;
  float* baseb_ = nullptr;
  float* targetb_ = nullptr;
  float* zs_ = nullptr;
  void* h_[3] = {nullptr, nullptr, nullptr};
  void* dz_[3] = {nullptr, nullptr, nullptr};
  float* y_ = nullptr;
  float* dyf_ = nullptr;
  void* dyb_ = nullptr;
  float* lossSum_ = nullptr;
  uint32_t* idx_ = nullptr;
  // training set
  void* X_ = nullptr;
  float* base_ = nullptr;
  float* target_ = nullptr;
  size_t rows_ = 0, rowCap_ = 0;
};

}  // namespace cr
