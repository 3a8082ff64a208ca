// Learned per-ommatidium denoiser: a 4-layer MLP (width 128, ReLU) trained
// and run on the GPU with BF16 tensor-core GEMMs accumulating in FP32.
//
// The denoiser maps an 8-sample estimate of an ommatidium and of its six
// nearest neighbours (sample statistics from the feature render, the
// ommatidial axis and acceptance angle) to a correction of the 8-sample mean
// colour; the target is a high-sample render of the same pose.  Everything
// here is device code driven by the host class in denoiser.cpp:
//   gemmKernel       C = A * B with bf16 operands (mma.sync m16n8k16, fp32
//                    accumulators) and fused epilogues (bias, ReLU, ReLU
//                    derivative mask, plain fp32 store);
//   colSumKernel     bias gradients;
//   lossKernel       residual prediction, squared error and its gradient;
//   adamKernel       Adam on fp32 master weights, refreshing the bf16 copy
//                    and the transposed bf16 weight matrices;
//   knnKernel        six nearest ommatidia by axis direction;
//   featureKernel    assembles the 112-wide bf16 feature rows.
// These mma.sync GEMMs are the path the layer-by-layer prediction uses and
// the training path of crSetDenoiserKernel(0); training runs on the tcgen05
// GEMMs of mlp_tc.cu by default.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "device_api.hpp"
#include "features.cuh"

namespace cr {
namespace {

constexpr int BM = 64, BN = 64, BK = 32;
constexpr int kPad = 8;  // bf16 elements of padding per smem row

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return static_cast<uint32_t>(__bfloat16_as_ushort(lo)) | (static_cast<uint32_t>(__bfloat16_as_ushort(hi)) << 16);
}

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[M x N] = A[M x K] * B[K x N].
//  A: aTrans ? stored K x M row-major (A[m][k] = A[k*lda + m]) : M x K (A[m*lda + k]).
//  B: bTrans ? stored N x K row-major (B[k][n] = B[n*ldb + k]) : K x N (B[k*ldb + n]).
// Epilogue (mode):
//  0: Cf[m*ldc+n] = acc
//  1: Cf = acc + bias[n]; Hb[m*ldc+n] = bf16(max(Cf, 0))        (hidden layer forward)
//  2: Hb[m*ldc+n] = bf16(acc * (mask[m*ldc+n] > 0))             (back through ReLU)
//  3: Cf = acc + bias[n]                                       (output layer)
template <int kMode>
__global__ void __launch_bounds__(128) gemmKernel(int M, int N, int K, const __nv_bfloat16* __restrict__ A, int lda,
                                                  bool aTrans, const __nv_bfloat16* __restrict__ B, int ldb,
                                                  bool bTrans, float* __restrict__ Cf, __nv_bfloat16* __restrict__ Hb,
                                                  int ldc, const float* __restrict__ bias,
                                                  const __nv_bfloat16* __restrict__ mask, int kSlice = 0) {
  __shared__ __nv_bfloat16 As[BM][BK + kPad];
  __shared__ __nv_bfloat16 Bs[BN][BK + kPad];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;  // 2 x 2 warps of 32 x 32
  const int g = lane >> 2, q = lane & 3;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  // Split K: block z covers [z * kSlice, (z + 1) * kSlice) and writes its
  // partial tile to slice z of Cf (M x N each, ldc = N).
  const int kBeg = kSlice ? static_cast<int>(blockIdx.z) * kSlice : 0;
  const int kEnd = kSlice ? min(K, kBeg + kSlice) : K;
  if (kSlice) Cf += static_cast<size_t>(blockIdx.z) * M * N;
  for (int k0 = kBeg; k0 < kEnd; k0 += BK) {
    // Tile loads walk the operand's contiguous dimension with consecutive
    // threads (k for a row-major A / transposed B, m or n otherwise).
    for (int e = tid; e < BM * BK; e += 128) {
      const int r = aTrans ? e % BM : e / BK, c = aTrans ? e / BM : e % BK;
      const int m = m0 + r, k = k0 + c;
      __nv_bfloat16 v = zero;
      if (m < M && k < kEnd) v = aTrans ? A[static_cast<size_t>(k) * lda + m] : A[static_cast<size_t>(m) * lda + k];
      As[r][c] = v;
    }
    for (int e = tid; e < BN * BK; e += 128) {
      const int r = bTrans ? e / BK : e % BN, c = bTrans ? e % BK : e / BN;
      const int n = n0 + r, k = k0 + c;
      __nv_bfloat16 v = zero;
      if (n < N && k < kEnd) v = bTrans ? B[static_cast<size_t>(n) * ldb + k] : B[static_cast<size_t>(k) * ldb + n];
      Bs[r][c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r0 = wm * 32 + i * 16 + g;
        const int c0 = kk + q * 2;
        af[i][0] = pack2(As[r0][c0], As[r0][c0 + 1]);
        af[i][1] = pack2(As[r0 + 8][c0], As[r0 + 8][c0 + 1]);
        af[i][2] = pack2(As[r0][c0 + 8], As[r0][c0 + 9]);
        af[i][3] = pack2(As[r0 + 8][c0 + 8], As[r0 + 8][c0 + 9]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int nr = wn * 32 + j * 8 + g;
        const int c0 = kk + q * 2;
        bf[j][0] = pack2(Bs[nr][c0], Bs[nr][c0 + 1]);
        bf[j][1] = pack2(Bs[nr][c0 + 8], Bs[nr][c0 + 9]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma16816(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int m = m0 + wm * 32 + i * 16 + g + (r >= 2 ? 8 : 0);
        const int n = n0 + wn * 32 + j * 8 + q * 2 + (r & 1);
        if (m >= M || n >= N) continue;
        const size_t o = static_cast<size_t>(m) * ldc + n;
        float v = acc[i][j][r];
        if (kMode == 0) {
          Cf[o] = v;
        } else if (kMode == 1) {
          v += bias[n];
          Cf[o] = v;
          Hb[o] = __float2bfloat16(fmaxf(v, 0.f));
        } else if (kMode == 2) {
          Hb[o] = __float2bfloat16(__bfloat162float(mask[o]) > 0.f ? v : 0.f);
        } else {
          Cf[o] = v + bias[n];
        }
      }
}

// out[n] = sum over m of in[m*ld + n], for bf16 or fp32 input.  Block
// (g, slab) sums columns 32g .. 32g + 31 (one per lane, so a warp reads 32
// consecutive columns of a row) over one slab of rows, its 8 warps taking
// every 8th row; the slab's sum goes to a scratch row, and the block that
// finishes a column group last adds the slabs' sums in slab order.  The
// result does not depend on which block finishes when.  Launches share the
// scratch and the counters, so they must not run concurrently (the denoiser
// issues them on one stream).
constexpr int kColSumMaxSlabs = 64;
constexpr int kColSumMaxGroups = 128;  // N <= 4096
__device__ float g_colSumPart[kColSumMaxSlabs * kColSumMaxGroups * 32];
__device__ unsigned int g_colSumDone[kColSumMaxGroups];

template <typename T>
__global__ void __launch_bounds__(256) colSumKernel(const T* __restrict__ in, int M, int N, int ld, int rowsPerSlab,
                                                    float* __restrict__ out) {
  __shared__ float part[8][32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = blockIdx.x, slab = blockIdx.y;
  const int n = g * 32 + lane;
  const int m0 = slab * rowsPerSlab, m1 = min(M, m0 + rowsPerSlab);
  auto val = [&](int m) {
    if constexpr (sizeof(T) == 2) return __bfloat162float(in[static_cast<size_t>(m) * ld + n]);
    else return static_cast<float>(in[static_cast<size_t>(m) * ld + n]);
  };
  float s0 = 0.f, s1 = 0.f;
  if (n < N) {
    int m = m0 + w;
    for (; m + 8 < m1; m += 16) {
      s0 += val(m);
      s1 += val(m + 8);
    }
    for (; m < m1; m += 8) s0 += val(m);
  }
  part[w][lane] = s0 + s1;
  __syncthreads();
  if (w == 0) {
    float t = 0.f;
    for (int k = 0; k < 8; ++k) t += part[k][lane];
    g_colSumPart[(slab * kColSumMaxGroups + g) * 32 + lane] = t;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&g_colSumDone[g], 1u) == gridDim.y - 1;
  __syncthreads();
  if (last && w == 0) {
    __threadfence();
    float t = 0.f;
    for (int sl = 0; sl < static_cast<int>(gridDim.y); ++sl)
      t += __ldcg(&g_colSumPart[(sl * kColSumMaxGroups + g) * 32 + lane]);
    if (n < N) out[n] = t;
    if (lane == 0) g_colSumDone[g] = 0u;
  }
}

template <typename T>
cudaError_t colSum(const T* in, int M, int N, int ld, float* out, cudaStream_t stream) {
  if (N <= 0) return cudaSuccess;
  const int groups = (N + 31) / 32;
  if (groups > kColSumMaxGroups) return cudaErrorInvalidValue;
  if (M <= 0) return cudaMemsetAsync(out, 0, static_cast<size_t>(N) * sizeof(float), stream);
  const int rowsPerSlab = std::max(64, (M + kColSumMaxSlabs - 1) / kColSumMaxSlabs);
  const int slabs = (M + rowsPerSlab - 1) / rowsPerSlab;  // <= kColSumMaxSlabs
  colSumKernel<T><<<dim3(groups, slabs), 256, 0, stream>>>(in, M, N, ld, rowsPerSlab, out);
  return cudaGetLastError();
}

// Prediction = base + y[:, :3]; squared error against target; gradient of
// the mean squared error w.r.t. y (fp32 and bf16 copies, padded columns 0).
__global__ void lossKernel(const float* __restrict__ y, int ldy, const float* __restrict__ base,
                           const float* __restrict__ target, int rows, float* __restrict__ pred,
                           float* __restrict__ dyf, __nv_bfloat16* __restrict__ dyb, float* __restrict__ lossSum,
                           const int* __restrict__ lossIndex) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (lossSum && lossIndex) lossSum += *lossIndex;
  float e2 = 0.f;
  if (r < rows) {
    const float scale = 2.0f / (3.0f * static_cast<float>(rows));
    for (int c = 0; c < ldy; ++c) {
      float g = 0.f;
      if (c < 3) {
        const float p = base[3 * r + c] + y[static_cast<size_t>(r) * ldy + c];
        if (pred) pred[3 * r + c] = p;
        if (target) {
          const float d = p - target[3 * r + c];
          e2 += d * d;
          g = scale * d;
        }
      }
      if (dyf) dyf[static_cast<size_t>(r) * ldy + c] = g;
      if (dyb) dyb[static_cast<size_t>(r) * ldy + c] = __float2bfloat16(g);
    }
  }
  if (lossSum) {
    for (int m = 16; m >= 1; m >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, m);
    if ((threadIdx.x & 31) == 0) atomicAdd(lossSum, e2);
  }
}

// The transposed bf16 copy of parameter i, if it lies in one of `blocks`.
__device__ __forceinline__ void putTransposed(int i, float wi, __nv_bfloat16* __restrict__ wbT, const WeightBlocks& b) {
  for (int k = 0; k < b.count; ++k) {
    const int j = i - b.off[k];
    if (j >= 0 && j < b.rows[k] * b.cols[k]) {
      const int r = j / b.cols[k], c = j - r * b.cols[k];
      wbT[b.off[k] + c * b.rows[k] + r] = __float2bfloat16(wi);
      return;
    }
  }
}

// Explicitly rounded single-precision operations (no FTZ, no contraction),
// so the --use_fast_math build of this file leaves Adam's arithmetic exact
// IEEE and a CPU restatement can repeat it bit for bit.
__device__ __forceinline__ float radd(float a, float b) {
  float r;
  asm("add.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float rsub(float a, float b) {
  float r;
  asm("sub.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float rmul(float a, float b) {
  float r;
  asm("mul.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float rdiv(float a, float b) {
  float r;
  asm("div.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float rsqrt_rn(float a) {
  float r;
  asm("sqrt.rn.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}

// Adam (Kingma & Ba 2015) with the bias corrections folded in as
// c1 = 1 / (1 - b1^t), c2 = 1 / (1 - b2^t):
//   m = b1 m + (1 - b1) g;  v = b2 v + (1 - b2) g g;
//   w = w - lr (m c1) / (sqrt(v c2) + eps)
// one correctly rounded float operation at a time, in this order.
__global__ void adamKernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                           float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2,
                           __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wbT, WeightBlocks blocks,
                           const float* __restrict__ sched, const int* __restrict__ stepIdx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (sched) {
    const float* e = sched + 3 * static_cast<size_t>(*stepIdx);
    lr = e[0];
    c1 = e[1];
    c2 = e[2];
  }
  const float gi = g[i];
  const float mi = radd(rmul(b1, m[i]), rmul(rsub(1.f, b1), gi));
  const float vi = radd(rmul(b2, v[i]), rmul(rmul(rsub(1.f, b2), gi), gi));
  m[i] = mi;
  v[i] = vi;
  const float wi = rsub(w[i], rdiv(rmul(lr, rmul(mi, c1)), radd(rsqrt_rn(rmul(vi, c2)), eps)));
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16(wi);
  if (wbT) putTransposed(i, wi, wbT, blocks);
}

__global__ void transposeWeightsKernel(const float* __restrict__ w, int n, __nv_bfloat16* __restrict__ wbT,
                                       WeightBlocks blocks) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) putTransposed(i, w[i], wbT, blocks);
}

__global__ void toBf16Kernel(const float* __restrict__ in, __nv_bfloat16* __restrict__ out, size_t n) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2bfloat16(in[i]);
}

// Six nearest ommatidia of each ommatidium by the angle between axes.
__global__ void knnKernel(const float4* __restrict__ omm, uint32_t N, int* __restrict__ nb) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= N) return;
  const float4 a = omm[2 * o], b = omm[2 * o + 1];
  float ax = a.w, ay = b.x, az = b.y;
  const float il = rsqrtf(fmaxf(ax * ax + ay * ay + az * az, 1e-30f));
  ax *= il;
  ay *= il;
  az *= il;
  float best[kNeighbours];
  int idx[kNeighbours];
  for (int k = 0; k < kNeighbours; ++k) {
    best[k] = -2.f;
    idx[k] = static_cast<int>(o);
  }
  for (uint32_t j = 0; j < N; ++j) {
    if (j == o) continue;
    const float4 c = omm[2 * j], d = omm[2 * j + 1];
    const float l = rsqrtf(fmaxf(c.w * c.w + d.x * d.x + d.y * d.y, 1e-30f));
    const float s = (ax * c.w + ay * d.x + az * d.y) * l;
    if (s <= best[kNeighbours - 1]) continue;
    int k = kNeighbours - 1;
    while (k > 0 && best[k - 1] < s) {
      best[k] = best[k - 1];
      idx[k] = idx[k - 1];
      --k;
    }
    best[k] = s;
    idx[k] = static_cast<int>(j);
  }
  for (int k = 0; k < kNeighbours; ++k) nb[kNeighbours * o + k] = idx[k];
}

__global__ void featureKernel(const float* __restrict__ stats, const float4* __restrict__ omm,
                              const int* __restrict__ nb, uint32_t N, uint32_t P, __nv_bfloat16* __restrict__ X,
                              float* __restrict__ base) {
  const size_t row = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (row >= static_cast<size_t>(P) * N) return;
  feat::featureRow(stats, omm, nb, N, row, true, 0, kNeighbours, X + row * kFeatureWidth, base);
}

// ---------------------------------------------------------------------------
// Fused inference: feature rows, the four layers and the residual sum for
// tiles of 128 rows, with all weights resident in shared memory.  A
// persistent grid (one block per SM) stages the weights once, transposed to
// [out][in] so every B fragment is one 32-bit shared load; each of the 8
// warps owns 16 rows and keeps all 128 hidden outputs of a layer in
// registers (16 m16n8 tiles), so activations never leave the SM.  The
// k-steps run in the same order as gemmKernel's, so a row's prediction is
// bit-identical to the layer-by-layer path.
// ---------------------------------------------------------------------------
constexpr int kInferRows = 128;
constexpr int kInferThreads = 256;
constexpr int kS1 = kFeatureWidth + 8;  // padded row strides (bf16 elements)
constexpr int kSH = kMlpHidden + 8;
constexpr size_t kInferSmem = (size_t(kMlpHidden) * kS1 + 2 * size_t(kMlpHidden) * kSH + size_t(kMlpOut) * kSH +
                               size_t(kInferRows) * kSH) * 2 +
                              (3 * kMlpHidden + kMlpOut) * 4;

// One hidden layer for the warp's 16 rows, in place: h[16 x K] -> h[16 x 128].
template <int K, int kStrideW>
__device__ __forceinline__ void hiddenLayer(__nv_bfloat16* h, const __nv_bfloat16* wt, const float* bias, int lane) {
  const int g = lane >> 2, q = lane & 3;
  float acc[kMlpHidden / 8][4];
#pragma unroll
  for (int j = 0; j < kMlpHidden / 8; ++j)
#pragma unroll
    for (int r = 0; r < 4; ++r) acc[j][r] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < K; k0 += 16) {
    uint32_t a[4];
    const __nv_bfloat16* hr = h + g * kSH + k0 + 2 * q;
    a[0] = *reinterpret_cast<const uint32_t*>(hr);
    a[1] = *reinterpret_cast<const uint32_t*>(hr + 8 * kSH);
    a[2] = *reinterpret_cast<const uint32_t*>(hr + 8);
    a[3] = *reinterpret_cast<const uint32_t*>(hr + 8 * kSH + 8);
#pragma unroll
    for (int j = 0; j < kMlpHidden / 8; ++j) {
      const __nv_bfloat16* wr = wt + (j * 8 + g) * kStrideW + k0 + 2 * q;
      uint32_t b[2] = {*reinterpret_cast<const uint32_t*>(wr), *reinterpret_cast<const uint32_t*>(wr + 8)};
      mma16816(acc[j], a, b);
    }
  }
  __syncwarp();
#pragma unroll
  for (int j = 0; j < kMlpHidden / 8; ++j) {
    const int c = j * 8 + 2 * q;
    const float v0 = acc[j][0] + bias[c], v1 = acc[j][1] + bias[c + 1];
    const float v2 = acc[j][2] + bias[c], v3 = acc[j][3] + bias[c + 1];
    *reinterpret_cast<uint32_t*>(h + g * kSH + c) =
        pack2(__float2bfloat16(fmaxf(v0, 0.f)), __float2bfloat16(fmaxf(v1, 0.f)));
    *reinterpret_cast<uint32_t*>(h + (g + 8) * kSH + c) =
        pack2(__float2bfloat16(fmaxf(v2, 0.f)), __float2bfloat16(fmaxf(v3, 0.f)));
  }
  __syncwarp();
}

__global__ void __launch_bounds__(kInferThreads, 1)
    inferKernel(const float* __restrict__ stats, const float4* __restrict__ omm, const int* __restrict__ nb,
                uint32_t N, uint64_t rows, MlpWeights w, bool residual, float* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16* w1t = reinterpret_cast<__nv_bfloat16*>(smem);
  __nv_bfloat16* w2t = w1t + kMlpHidden * kS1;
  __nv_bfloat16* w3t = w2t + kMlpHidden * kSH;
  __nv_bfloat16* w4t = w3t + kMlpHidden * kSH;
  __nv_bfloat16* h = w4t + kMlpOut * kSH;
  float* b1 = reinterpret_cast<float*>(h + kInferRows * kSH);
  float* b2 = b1 + kMlpHidden;
  float* b3 = b2 + kMlpHidden;
  float* b4 = b3 + kMlpHidden;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // Stage the weights transposed: wt[n][k] = W[k][n].
  for (int e = tid; e < kFeatureWidth * kMlpHidden; e += kInferThreads)
    w1t[(e % kMlpHidden) * kS1 + e / kMlpHidden] = w.w1[e];
  for (int e = tid; e < kMlpHidden * kMlpHidden; e += kInferThreads) {
    w2t[(e % kMlpHidden) * kSH + e / kMlpHidden] = w.w2[e];
    w3t[(e % kMlpHidden) * kSH + e / kMlpHidden] = w.w3[e];
  }
  for (int e = tid; e < kMlpHidden * kMlpOut; e += kInferThreads) w4t[(e % kMlpOut) * kSH + e / kMlpOut] = w.w4[e];
  for (int e = tid; e < kMlpHidden; e += kInferThreads) {
    b1[e] = w.b1[e];
    b2[e] = w.b2[e];
    b3[e] = w.b3[e];
  }
  if (tid < kMlpOut) b4[tid] = w.b4[tid];
  const uint64_t tiles = (rows + kInferRows - 1) / kInferRows;
  const int g = lane >> 2, q = lane & 3;
  __nv_bfloat16* hw = h + warp * 16 * kSH;
  for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    __syncthreads();  // weights staged / previous tile's rows consumed
    {
      const int r = tid >> 1, half = tid & 1;
      const uint64_t row = tile * kInferRows + r;
      __nv_bfloat16* x = h + r * kSH;
      if (row < rows) {
        feat::featureRow(stats, omm, nb, N, row, half == 0, half == 0 ? 0 : 3, half == 0 ? 3 : kNeighbours, x, nullptr);
      } else {
        for (int k = half; k < kFeatureWidth; k += 2) x[k] = __float2bfloat16(0.f);
      }
    }
    __syncthreads();
    hiddenLayer<kFeatureWidth, kS1>(hw, w1t, b1, lane);
    hiddenLayer<kMlpHidden, kSH>(hw, w2t, b2, lane);
    hiddenLayer<kMlpHidden, kSH>(hw, w3t, b3, lane);
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k0 = 0; k0 < kMlpHidden; k0 += 16) {
      uint32_t a[4];
      const __nv_bfloat16* hr = hw + g * kSH + k0 + 2 * q;
      a[0] = *reinterpret_cast<const uint32_t*>(hr);
      a[1] = *reinterpret_cast<const uint32_t*>(hr + 8 * kSH);
      a[2] = *reinterpret_cast<const uint32_t*>(hr + 8);
      a[3] = *reinterpret_cast<const uint32_t*>(hr + 8 * kSH + 8);
      const __nv_bfloat16* wr = w4t + g * kSH + k0 + 2 * q;
      uint32_t b[2] = {*reinterpret_cast<const uint32_t*>(wr), *reinterpret_cast<const uint32_t*>(wr + 8)};
      mma16816(acc, a, b);
    }
    // acc: rows g / g+8, output columns 2q, 2q+1; columns 0..2 are colours.
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int c = 2 * q + (r & 1);
      const uint64_t row = tile * kInferRows + warp * 16 + g + (r >= 2 ? 8 : 0);
      if (c < 3 && row < rows) {
        const float y = acc[r] + b4[c];
        out[3 * row + c] = residual ? stats[row * kFeatureStats + c] + y : y;
      }
    }
  }
}

__global__ void gatherRowsKernel(const __nv_bfloat16* __restrict__ X, const float* __restrict__ base,
                                 const float* __restrict__ target, const uint32_t* __restrict__ idx, int rows,
                                 __nv_bfloat16* __restrict__ Xo, float* __restrict__ baseo, float* __restrict__ targeto,
                                 const uint32_t* __restrict__ offset) {
  const int r = blockIdx.x;
  if (r >= rows) return;
  const size_t src = idx[(offset ? *offset : 0u) + r];
  for (int k = threadIdx.x; k < kFeatureWidth; k += blockDim.x)
    Xo[static_cast<size_t>(r) * kFeatureWidth + k] = X[src * kFeatureWidth + k];
  if (threadIdx.x < 3) {
    baseo[3 * r + threadIdx.x] = base[3 * src + threadIdx.x];
    targeto[3 * r + threadIdx.x] = target[3 * src + threadIdx.x];
  }
}

}  // namespace

namespace {
// Split-K partial sums: slices[s][m][n] summed in slice order into C.
__global__ void splitKReduceKernel(const float* __restrict__ part, int slices, int M, int N, float* __restrict__ C,
                                   int ldc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * N) return;
  const int m = i / N, n = i % N;
  float s = 0.f;
  for (int k = 0; k < slices; ++k) s += part[static_cast<size_t>(k) * M * N + i];
  C[static_cast<size_t>(m) * ldc + n] = s;
}
float* g_splitK = nullptr;
size_t g_splitKFloats = 0;
}  // namespace

cudaError_t gemmBf16(int mode, int M, int N, int K, const void* A, int lda, bool aTrans, const void* B, int ldb,
                     bool bTrans, float* Cf, void* Hb, int ldc, const float* bias, const void* mask,
                     cudaStream_t stream) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  // Weight gradients (a long K over the minibatch, a small M x N) split K
  // into slices of 256 so that enough blocks run; the partial tiles are then
  // summed in slice order (deterministic).
  const int tiles = ((N + BN - 1) / BN) * ((M + BM - 1) / BM);
  if (mode == 0 && K >= 1024 && tiles < 64 && !bTrans) {
    const int slice = 256, slices = (K + slice - 1) / slice;
    const size_t need = static_cast<size_t>(slices) * M * N;
    if (need > g_splitKFloats) {
      if (g_splitK) cudaFree(g_splitK);
      g_splitK = nullptr;
      g_splitKFloats = 0;
      cudaError_t e = cudaMalloc(&g_splitK, need * sizeof(float));
      if (e != cudaSuccess) return e;
      g_splitKFloats = need;
    }
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, slices);
    gemmKernel<0><<<grid, 128, 0, stream>>>(M, N, K, static_cast<const __nv_bfloat16*>(A), lda, aTrans,
                                            static_cast<const __nv_bfloat16*>(B), ldb, bTrans, g_splitK, nullptr, N,
                                            nullptr, nullptr, slice);
    splitKReduceKernel<<<(M * N + 255) / 256, 256, 0, stream>>>(g_splitK, slices, M, N, Cf, ldc);
    return cudaGetLastError();
  }
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  auto a = static_cast<const __nv_bfloat16*>(A);
  auto b = static_cast<const __nv_bfloat16*>(B);
  auto h = static_cast<__nv_bfloat16*>(Hb);
  auto mk = static_cast<const __nv_bfloat16*>(mask);
  switch (mode) {
    case 0: gemmKernel<0><<<grid, 128, 0, stream>>>(M, N, K, a, lda, aTrans, b, ldb, bTrans, Cf, h, ldc, bias, mk); break;
    case 1: gemmKernel<1><<<grid, 128, 0, stream>>>(M, N, K, a, lda, aTrans, b, ldb, bTrans, Cf, h, ldc, bias, mk); break;
    case 2: gemmKernel<2><<<grid, 128, 0, stream>>>(M, N, K, a, lda, aTrans, b, ldb, bTrans, Cf, h, ldc, bias, mk); break;
    default: gemmKernel<3><<<grid, 128, 0, stream>>>(M, N, K, a, lda, aTrans, b, ldb, bTrans, Cf, h, ldc, bias, mk); break;
  }
  return cudaGetLastError();
}

cudaError_t colSumBf16(const void* in, int M, int N, int ld, float* out, cudaStream_t stream) {
  return colSum(static_cast<const __nv_bfloat16*>(in), M, N, ld, out, stream);
}

cudaError_t colSumF32(const float* in, int M, int N, int ld, float* out, cudaStream_t stream) {
  return colSum(in, M, N, ld, out, stream);
}

cudaError_t mlpLoss(const float* y, int ldy, const float* base, const float* target, int rows, float* pred, float* dyf,
                    void* dyb, float* lossSum, cudaStream_t stream, const int* lossIndex) {
  if (rows <= 0) return cudaSuccess;
  lossKernel<<<(rows + 255) / 256, 256, 0, stream>>>(y, ldy, base, target, rows, pred, dyf,
                                                      static_cast<__nv_bfloat16*>(dyb), lossSum, lossIndex);
  return cudaGetLastError();
}

cudaError_t adamStep(float* w, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                     int t, void* wb, cudaStream_t stream, void* wbT, const WeightBlocks* blocks, const float* sched,
                     const int* stepIdx) {
  const float c1 = 1.f / (1.f - powf(b1, static_cast<float>(t)));
  const float c2 = 1.f / (1.f - powf(b2, static_cast<float>(t)));
  WeightBlocks none{};
  adamKernel<<<(n + 255) / 256, 256, 0, stream>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2,
                                                   static_cast<__nv_bfloat16*>(wb), static_cast<__nv_bfloat16*>(wbT),
                                                   wbT && blocks ? *blocks : none, sched && stepIdx ? sched : nullptr,
                                                   stepIdx);
  return cudaGetLastError();
}

cudaError_t transposeWeightsBf16(const float* w, size_t n, void* wbT, const WeightBlocks& blocks, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  transposeWeightsKernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(
      w, static_cast<int>(n), static_cast<__nv_bfloat16*>(wbT), blocks);
  return cudaGetLastError();
}

cudaError_t toBf16(const float* in, void* out, size_t n, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  toBf16Kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(in, static_cast<__nv_bfloat16*>(out), n);
  return cudaGetLastError();
}

cudaError_t nearestOmmatidia(const float4* omm, uint32_t N, int* nb, cudaStream_t stream) {
  if (N == 0) return cudaSuccess;
  knnKernel<<<(N + 127) / 128, 128, 0, stream>>>(omm, N, nb);
  return cudaGetLastError();
}

cudaError_t assembleFeatures(const float* stats, const float4* omm, const int* nb, uint32_t N, uint32_t P, void* X,
                             float* base, cudaStream_t stream) {
  const size_t rows = static_cast<size_t>(P) * N;
  if (rows == 0) return cudaSuccess;
  featureKernel<<<static_cast<unsigned>((rows + 127) / 128), 128, 0, stream>>>(
      stats, omm, nb, N, P, static_cast<__nv_bfloat16*>(X), base);
  return cudaGetLastError();
}

cudaError_t inferDenoiser(const float* stats, const float4* omm, const int* nb, uint32_t N, uint32_t P,
                          const MlpWeights& w, float* out, cudaStream_t stream, bool residual) {
  const uint64_t rows = static_cast<uint64_t>(N) * P;
  if (rows == 0) return cudaSuccess;
  static int smCount = 0;
  static bool attrSet = false;
  if (!attrSet) {
    cudaError_t e = cudaFuncSetAttribute(inferKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(kInferSmem));
    if (e != cudaSuccess) return e;
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smCount, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    attrSet = true;
  }
  const uint64_t tiles = (rows + kInferRows - 1) / kInferRows;
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(tiles, static_cast<uint64_t>(smCount)));
  inferKernel<<<grid, kInferThreads, kInferSmem, stream>>>(stats, omm, nb, N, rows, w, residual, out);
  return cudaGetLastError();
}

cudaError_t gatherRows(const void* X, const float* base, const float* target, const uint32_t* idx, int rows, void* Xo,
                       float* baseo, float* targeto, cudaStream_t stream, const uint32_t* offset) {
  if (rows <= 0) return cudaSuccess;
  gatherRowsKernel<<<rows, 128, 0, stream>>>(static_cast<const __nv_bfloat16*>(X), base, target, idx, rows,
                                             static_cast<__nv_bfloat16*>(Xo), baseo, targeto, offset);
  return cudaGetLastError();
}

__global__ void advanceTrainKernel(TrainState* state, uint32_t rows) {
  state->step += 1;
  state->offset += rows;
}

cudaError_t advanceTrainState(TrainState* state, uint32_t rows, cudaStream_t stream) {
  advanceTrainKernel<<<1, 1, 0, stream>>>(state, rows);
  return cudaGetLastError();
}

}  // namespace cr
