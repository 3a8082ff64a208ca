// Host side of the learned per-ommatidium denoiser; see denoiser.hpp.
#include "denoiser.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <numeric>
#include <random>
#include <stdexcept>

namespace cr {
namespace {

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string("denoiser ") + what + ": " + cudaGetErrorString(e));
}

template <typename T>
T* dalloc(size_t n) {
  void* p = nullptr;
  ck(cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)), "cudaMalloc");
  return static_cast<T*>(p);
}

void dfree(void* p) {
  if (p) cudaFree(p);
}

constexpr uint32_t kMagic = 0x4e445243;  // checkpoint tag
constexpr uint32_t kVersion = 1;

}  // namespace

void Denoiser::release() {
  for (void* p : {static_cast<void*>(params_), static_cast<void*>(grads_), static_cast<void*>(m_), static_cast<void*>(v_),
                  wbf_, wbfT_, Xb_, static_cast<void*>(baseb_), static_cast<void*>(targetb_), static_cast<void*>(zs_), h_[0],
                  h_[1], h_[2], dz_[0], dz_[1], dz_[2], static_cast<void*>(y_), static_cast<void*>(dyf_), dyb_,
                  static_cast<void*>(lossSum_), static_cast<void*>(idx_), X_, static_cast<void*>(base_),
                  static_cast<void*>(target_)})
    dfree(p);
  params_ = grads_ = m_ = v_ = nullptr;
  wbf_ = wbfT_ = Xb_ = nullptr;
  baseb_ = targetb_ = zs_ = y_ = dyf_ = lossSum_ = nullptr;
  for (int i = 0; i < 3; ++i) h_[i] = dz_[i] = nullptr;
  dyb_ = nullptr;
  idx_ = nullptr;
  X_ = nullptr;
  base_ = target_ = nullptr;
  cap_ = 0;
  rows_ = rowCap_ = 0;
  adamT_ = 0;
}

void Denoiser::init(uint32_t seed, cudaStream_t s) {
  release();
  params_ = dalloc<float>(kParams);
  grads_ = dalloc<float>(kParams);
  m_ = dalloc<float>(kParams);
  v_ = dalloc<float>(kParams);
  wbf_ = dalloc<uint16_t>(kParams);
  wbfT_ = dalloc<uint16_t>(kParams);
  ck(cudaMemsetAsync(wbfT_, 0, kParams * 2, s), "memset");
  std::vector<float> h(kParams, 0.f);
  std::mt19937 rng(seed);
  auto fill = [&](size_t off, int fanIn, int fanOut, float scale) {
    std::normal_distribution<float> nd(0.f, std::sqrt(2.0f / static_cast<float>(fanIn)) * scale);
    for (size_t i = 0; i < size_t(fanIn) * fanOut; ++i) h[off + i] = nd(rng);
  };
  fill(offW1, kFeatureWidth, kHidden, 1.f);
  fill(offW2, kHidden, kHidden, 1.f);
  fill(offW3, kHidden, kHidden, 1.f);
  fill(offW4, kHidden, kOut, 0.01f);  // start close to the 8-sample mean
  ck(cudaMemcpyAsync(params_, h.data(), kParams * 4, cudaMemcpyHostToDevice, s), "upload");
  ck(cudaMemsetAsync(m_, 0, kParams * 4, s), "memset");
  ck(cudaMemsetAsync(v_, 0, kParams * 4, s), "memset");
  ck(toBf16(params_, wbf_, kParams, s), "bf16 copy");
  ck(transposeWeightsBf16(params_, kParams, wbfT_, weightBlocks(), s), "bf16 transposes");
  ck(cudaStreamSynchronize(s), "init");
  adamT_ = 0;
}

void Denoiser::ensureBatch(int rows) {
  if (rows <= cap_) return;
  for (void* p : {Xb_, static_cast<void*>(baseb_), static_cast<void*>(targetb_), static_cast<void*>(zs_), h_[0], h_[1],
                  h_[2], dz_[0], dz_[1], dz_[2], static_cast<void*>(y_), static_cast<void*>(dyf_), dyb_,
                  static_cast<void*>(lossSum_), static_cast<void*>(idx_)})
    dfree(p);
  cap_ = rows;
  const size_t r = static_cast<size_t>(rows);
  Xb_ = dalloc<uint16_t>(r * kFeatureWidth);
  baseb_ = dalloc<float>(r * 3);
  targetb_ = dalloc<float>(r * 3);
  zs_ = dalloc<float>(r * kHidden);
  for (int i = 0; i < 3; ++i) {
    h_[i] = dalloc<uint16_t>(r * kHidden);
    dz_[i] = dalloc<uint16_t>(r * kHidden);
  }
  y_ = dalloc<float>(r * kOut);
  dyf_ = dalloc<float>(r * kOut);
  dyb_ = dalloc<uint16_t>(r * kOut);
  lossSum_ = dalloc<float>(1);
  idx_ = dalloc<uint32_t>(r);
}

void Denoiser::forward(const void* X, int rows, cudaStream_t s) {
  // B operand of each layer: the tcgen05 GEMMs read the transposed weights
  // (K contiguous), the mma.sync GEMMs the row-major ones.
  const uint16_t* w = static_cast<const uint16_t*>(tc_ ? wbfT_ : wbf_);
  auto ldw = [&](int kin, int nout) { return tc_ ? kin : nout; };
  ck(gemm(1, rows, kHidden, kFeatureWidth, X, kFeatureWidth, false, w + offW1, ldw(kFeatureWidth, kHidden), tc_,
          zs_, h_[0], kHidden, params_ + offB1, nullptr, s),
     "layer 1");
  ck(gemm(1, rows, kHidden, kHidden, h_[0], kHidden, false, w + offW2, ldw(kHidden, kHidden), tc_, zs_, h_[1],
          kHidden, params_ + offB2, nullptr, s),
     "layer 2");
  ck(gemm(1, rows, kHidden, kHidden, h_[1], kHidden, false, w + offW3, ldw(kHidden, kHidden), tc_, zs_, h_[2],
          kHidden, params_ + offB3, nullptr, s),
     "layer 3");
  ck(gemm(3, rows, kOut, kHidden, h_[2], kHidden, false, w + offW4, ldw(kHidden, kOut), tc_, y_, nullptr, kOut,
          params_ + offB4, nullptr, s),
     "layer 4");
}

float Denoiser::forwardBackward(const void* X, const float* base, const float* target, int rows, bool wantLoss,
                                cudaStream_t s) {
  if (wantLoss) ck(cudaMemsetAsync(lossSum_, 0, 4, s), "memset");
  step(X, base, target, rows, wantLoss ? lossSum_ : nullptr, s);
  if (!wantLoss) return 0.f;
  float e2 = 0.f;
  ck(cudaMemcpyAsync(&e2, lossSum_, 4, cudaMemcpyDeviceToHost, s), "loss readback");
  ck(cudaStreamSynchronize(s), "step");
  return e2 / (3.0f * static_cast<float>(rows));
}

// Forward, loss gradient and backward of one minibatch into grads_, with the
// summed squared error added to lossAcc[*lossIndex] (device; index 0 when
// lossIndex is null) when lossAcc is given.  No host sync.
void Denoiser::step(const void* X, const float* base, const float* target, int rows, float* lossAcc, cudaStream_t s,
                    const int* lossIndex) {
  const uint16_t* w = static_cast<const uint16_t*>(wbf_);
  forward(X, rows, s);
  ck(mlpLoss(y_, kOut, base, target, rows, nullptr, dyf_, dyb_, lossAcc, s, lossIndex), "loss");
  // Output layer.
  ck(gemm(0, kHidden, kOut, rows, h_[2], kHidden, true, dyb_, kOut, false, grads_ + offW4, nullptr, kOut, nullptr,
              nullptr, s),
     "dW4");
  ck(colSumF32(dyf_, rows, kOut, kOut, grads_ + offB4, s), "db4");
  ck(gemm(2, rows, kHidden, kOut, dyb_, kOut, false, w + offW4, kOut, true, nullptr, dz_[2], kHidden, nullptr, h_[2],
              s),
     "dZ3");
  // Hidden layers 3, 2, 1.
  const size_t offW[3] = {offW1, offW2, offW3};
  const size_t offB[3] = {offB1, offB2, offB3};
  for (int l = 2; l >= 0; --l) {
    const void* in = l == 0 ? X : h_[l - 1];
    const int kin = l == 0 ? kFeatureWidth : kHidden;
    ck(gemm(0, kin, kHidden, rows, in, kin, true, dz_[l], kHidden, false, grads_ + offW[l], nullptr, kHidden,
                nullptr, nullptr, s),
       "dW");
    ck(colSumBf16(dz_[l], rows, kHidden, kHidden, grads_ + offB[l], s), "db");
    if (l > 0)
      ck(gemm(2, rows, kHidden, kHidden, dz_[l], kHidden, false, w + offW[l], kHidden, true, nullptr, dz_[l - 1],
                  kHidden, nullptr, h_[l - 1], s),
         "dZ");
  }
}

void Denoiser::addRows(const void* X, const float* base, const float* target, size_t rows, cudaStream_t s) {
  if (rows_ + rows > rowCap_) {
    const size_t cap = std::max(rows_ + rows, rowCap_ * 2);
    void* nX = dalloc<uint16_t>(cap * kFeatureWidth);
    float* nb = dalloc<float>(cap * 3);
    float* nt = dalloc<float>(cap * 3);
    if (rows_) {
      ck(cudaMemcpyAsync(nX, X_, rows_ * kFeatureWidth * 2, cudaMemcpyDeviceToDevice, s), "copy");
      ck(cudaMemcpyAsync(nb, base_, rows_ * 12, cudaMemcpyDeviceToDevice, s), "copy");
      ck(cudaMemcpyAsync(nt, target_, rows_ * 12, cudaMemcpyDeviceToDevice, s), "copy");
    }
    ck(cudaStreamSynchronize(s), "grow");
    dfree(X_);
    dfree(base_);
    dfree(target_);
    X_ = nX;
    base_ = nb;
    target_ = nt;
    rowCap_ = cap;
  }
  ck(cudaMemcpyAsync(static_cast<uint16_t*>(X_) + rows_ * kFeatureWidth, X, rows * kFeatureWidth * 2,
                     cudaMemcpyDeviceToDevice, s),
     "append");
  ck(cudaMemcpyAsync(base_ + rows_ * 3, base, rows * 12, cudaMemcpyDeviceToDevice, s), "append");
  ck(cudaMemcpyAsync(target_ + rows_ * 3, target, rows * 12, cudaMemcpyDeviceToDevice, s), "append");
  rows_ += rows;
}

void Denoiser::train(int steps, int batch, float lr, uint32_t seed, float* loss, cudaStream_t s, bool tc) {
  if (!ready()) throw std::runtime_error("denoiser not initialised");
  if (rows_ == 0) throw std::runtime_error("no training rows");
  if (steps <= 0) return;
  batch = static_cast<int>(std::min<size_t>(static_cast<size_t>(batch), rows_));
  ensureBatch(batch);
  // The shuffled order of an epoch, the step sizes and Adam's bias
  // corrections of every step, the per-step losses and the loop's position
  // (TrainState) live on the device.  The first step runs as plain launches
  // (it sets up what the kernels need), the next is captured as a CUDA graph
  // and replayed for the rest; the host only reshuffles between epochs.
  std::mt19937 rng(seed);
  std::vector<uint32_t> perm(rows_);
  std::iota(perm.begin(), perm.end(), 0u);
  std::shuffle(perm.begin(), perm.end(), rng);
  std::vector<float> sched(3 * static_cast<size_t>(steps));
  const float b1 = 0.9f, b2 = 0.999f;
  for (int st = 0; st < steps; ++st) {
    // half-cosine decay of the step size over this call, down to 5%
    const float decay = 0.05f + 0.95f * 0.5f * (1.0f + std::cos(3.14159265f * static_cast<float>(st) / steps));
    const float t = static_cast<float>(adamT_ + st + 1);
    sched[3 * st] = lr * decay;
    sched[3 * st + 1] = 1.f / (1.f - powf(b1, t));
    sched[3 * st + 2] = 1.f / (1.f - powf(b2, t));
  }
  uint32_t* permDev = dalloc<uint32_t>(rows_);
  float* lossDev = dalloc<float>(static_cast<size_t>(steps));
  float* schedDev = dalloc<float>(sched.size());
  TrainState* state = dalloc<TrainState>(1);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  auto cleanup = [&]() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    dfree(permDev);
    dfree(lossDev);
    dfree(schedDev);
    dfree(state);
  };
  tc_ = tc;
  try {
    ck(cudaMemcpyAsync(permDev, perm.data(), rows_ * 4, cudaMemcpyHostToDevice, s), "perm");
    ck(cudaMemcpyAsync(schedDev, sched.data(), sched.size() * 4, cudaMemcpyHostToDevice, s), "schedule");
    ck(cudaMemsetAsync(lossDev, 0, static_cast<size_t>(steps) * 4, s), "memset");
    ck(cudaMemsetAsync(state, 0, sizeof(TrainState), s), "memset");
    const WeightBlocks blocks = weightBlocks();
    auto oneStep = [&]() {
      ck(gatherRows(X_, base_, target_, permDev, batch, Xb_, baseb_, targetb_, s, &state->offset), "gather");
      step(Xb_, baseb_, targetb_, batch, loss ? lossDev : nullptr, s, &state->step);
      ck(adamStep(params_, grads_, m_, v_, static_cast<int>(kParams), 0.f, b1, b2, 1e-8f, 1, wbf_, s, wbfT_, &blocks,
                  schedDev, &state->step),
         "adam");
      ck(advanceTrainState(state, static_cast<uint32_t>(batch), s), "advance");
    };
    size_t cursor = 0;
    for (int st = 0; st < steps;) {
      if (cursor + static_cast<size_t>(batch) > rows_) {
        ck(cudaStreamSynchronize(s), "epoch");  // the previous order is no longer read
        std::shuffle(perm.begin(), perm.end(), rng);
        ck(cudaMemcpyAsync(permDev, perm.data(), rows_ * 4, cudaMemcpyHostToDevice, s), "perm");
        const TrainState at{st, 0u};
        ck(cudaMemcpyAsync(state, &at, sizeof(at), cudaMemcpyHostToDevice, s), "state");
        ck(cudaStreamSynchronize(s), "epoch");
        cursor = 0;
      }
      const int run = static_cast<int>(std::min<size_t>(static_cast<size_t>(steps - st),
                                                        (rows_ - cursor) / static_cast<size_t>(batch)));
      int done = 0;
      if (!exec) {
        oneStep();
        done = 1;
        if (run > 1) {
          ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture");
          try {
            oneStep();
          } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
            throw;
          }
          ck(cudaStreamEndCapture(s, &graph), "capture");
          ck(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
        }
      }
      for (; done < run; ++done) ck(cudaGraphLaunch(exec, s), "graph launch");
      st += run;
      cursor += static_cast<size_t>(run) * static_cast<size_t>(batch);
    }
    adamT_ += steps;
    if (loss) {
      ck(cudaMemcpyAsync(loss, lossDev, static_cast<size_t>(steps) * 4, cudaMemcpyDeviceToHost, s), "loss readback");
    }
    ck(cudaStreamSynchronize(s), "train");
    tc_ = false;
    if (tc) {
      uint32_t flags = 0;
      ck(takeTcGemmError(&flags), "tcgen05 GEMM status");
      if (flags) throw std::runtime_error("a tcgen05 GEMM wait timed out during training");
    }
  } catch (...) {
    tc_ = false;
    cleanup();
    throw;
  }
  cleanup();
  if (loss)
    for (int st = 0; st < steps; ++st) loss[st] /= 3.0f * static_cast<float>(batch);
}

void Denoiser::infer(const void* X, const float* base, size_t rows, float* out, cudaStream_t s) {
  if (!ready()) throw std::runtime_error("denoiser not initialised");
  const size_t chunk = 1 << 16;
  ensureBatch(static_cast<int>(std::min(rows, chunk)));
  for (size_t r0 = 0; r0 < rows; r0 += chunk) {
    const int r = static_cast<int>(std::min(chunk, rows - r0));
    forward(static_cast<const uint16_t*>(X) + r0 * kFeatureWidth, r, s);
    ck(mlpLoss(y_, kOut, base + 3 * r0, nullptr, r, out + 3 * r0, nullptr, nullptr, nullptr, s), "prediction");
  }
}

MlpWeights Denoiser::weights() const {
  if (!ready()) throw std::runtime_error("denoiser not initialised");
  const __nv_bfloat16* w = static_cast<const __nv_bfloat16*>(wbf_);
  return MlpWeights{w + offW1, w + offW2, w + offW3, w + offW4,
                    params_ + offB1, params_ + offB2, params_ + offB3, params_ + offB4};
}

float Denoiser::gradient(const void* X, const float* base, const float* target, int rows, float* gradsHost,
                         float* paramsHost, cudaStream_t s, bool tc) {
  if (!ready()) throw std::runtime_error("denoiser not initialised");
  ensureBatch(rows);
  tc_ = tc;
  float l;
  try {
    l = forwardBackward(X, base, target, rows, true, s);
  } catch (...) {
    tc_ = false;
    throw;
  }
  tc_ = false;
  if (tc) {
    uint32_t flags = 0;
    ck(takeTcGemmError(&flags), "tcgen05 GEMM status");
    if (flags) throw std::runtime_error("a tcgen05 GEMM wait timed out");
  }
  if (gradsHost) ck(cudaMemcpyAsync(gradsHost, grads_, kParams * 4, cudaMemcpyDeviceToHost, s), "grads");
  if (paramsHost) ck(cudaMemcpyAsync(paramsHost, params_, kParams * 4, cudaMemcpyDeviceToHost, s), "params");
  ck(cudaStreamSynchronize(s), "gradient");
  return l;
}

void Denoiser::scaleOutput(float alpha, cudaStream_t s) {
  if (!ready()) throw std::runtime_error("denoiser not initialised");
  const size_t n = kParams - offW4;  // W4 and b4
  std::vector<float> h(n);
  ck(cudaMemcpyAsync(h.data(), params_ + offW4, n * 4, cudaMemcpyDeviceToHost, s), "scale");
  ck(cudaStreamSynchronize(s), "scale");
  for (float& v : h) v *= alpha;
  ck(cudaMemcpyAsync(params_ + offW4, h.data(), n * 4, cudaMemcpyHostToDevice, s), "scale");
  ck(toBf16(params_, wbf_, kParams, s), "bf16 copy");
  ck(transposeWeightsBf16(params_, kParams, wbfT_, weightBlocks(), s), "bf16 transposes");
  ck(cudaStreamSynchronize(s), "scale");
}

// Checkpoint: magic, version, parameter count, Adam step, then the fp32
// parameters and the two Adam moment vectors.
void Denoiser::save(const std::string& path, cudaStream_t s) {
  if (!ready()) throw std::runtime_error("denoiser not initialised");
  std::vector<float> p(kParams), m(kParams), v(kParams);
  ck(cudaMemcpyAsync(p.data(), params_, kParams * 4, cudaMemcpyDeviceToHost, s), "save");
  ck(cudaMemcpyAsync(m.data(), m_, kParams * 4, cudaMemcpyDeviceToHost, s), "save");
  ck(cudaMemcpyAsync(v.data(), v_, kParams * 4, cudaMemcpyDeviceToHost, s), "save");
  ck(cudaStreamSynchronize(s), "save");
  std::ofstream f(path, std::ios::binary);
  if (!f.is_open()) throw std::runtime_error("cannot write '" + path + "'");
  const uint32_t hdr[4] = {kMagic, kVersion, static_cast<uint32_t>(kParams), static_cast<uint32_t>(adamT_)};
  f.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
  f.write(reinterpret_cast<const char*>(p.data()), kParams * 4);
  f.write(reinterpret_cast<const char*>(m.data()), kParams * 4);
  f.write(reinterpret_cast<const char*>(v.data()), kParams * 4);
  if (!f.good()) throw std::runtime_error("short write to '" + path + "'");
}

void Denoiser::load(const std::string& path, cudaStream_t s) {
  std::ifstream f(path, std::ios::binary);
  if (!f.is_open()) throw std::runtime_error("cannot read '" + path + "'");
  uint32_t hdr[4] = {0, 0, 0, 0};
  f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
  if (hdr[0] != kMagic || hdr[1] != kVersion || hdr[2] != kParams)
    throw std::runtime_error("'" + path + "' is not a denoiser checkpoint of this layout");
  std::vector<float> p(kParams), m(kParams), v(kParams);
  f.read(reinterpret_cast<char*>(p.data()), kParams * 4);
  f.read(reinterpret_cast<char*>(m.data()), kParams * 4);
  f.read(reinterpret_cast<char*>(v.data()), kParams * 4);
  if (!f.good()) throw std::runtime_error("truncated checkpoint '" + path + "'");
  if (!ready()) init(0, s);
  ck(cudaMemcpyAsync(params_, p.data(), kParams * 4, cudaMemcpyHostToDevice, s), "load");
  ck(cudaMemcpyAsync(m_, m.data(), kParams * 4, cudaMemcpyHostToDevice, s), "load");
  ck(cudaMemcpyAsync(v_, v.data(), kParams * 4, cudaMemcpyHostToDevice, s), "load");
  ck(toBf16(params_, wbf_, kParams, s), "bf16 copy");
  ck(transposeWeightsBf16(params_, kParams, wbfT_, weightBlocks(), s), "bf16 transposes");
  ck(cudaStreamSynchronize(s), "load");
  adamT_ = static_cast<int>(hdr[3]);
}

}  // namespace cr
