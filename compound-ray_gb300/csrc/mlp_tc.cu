// Fused denoiser inference on the 5th-generation tensor cores (tcgen05).
//
// Same function as inferKernel in mlp.cu (feature rows from the feature-render
// statistics, 112 -> 128 -> 128 -> 128 -> 8 network with bf16 operands and
// fp32 accumulation, bias + ReLU between layers, residual add), laid out for
// sm_103a's MMA unit:
//   * one persistent block of 512 threads per SM; all weights staged once in
//     shared memory as K-major UMMA operands (transposed to [out][in]) in the
//     canonical no-swizzle layout: 8-row x 16-byte core matrices, core
//     matrices along K 128 bytes apart (leading byte offset) and 8-row groups
//     K*16 bytes apart (stride byte offset);
//   * per tile of 128 rows, four threads assemble each row's 112 features
//     (own block + neighbour 0 / neighbours 1-2 / 3-4 / 5 + padding) into the
//     activation buffer in the same layout; one elected thread issues the
//     layer's tcgen05.mma instructions (M = 128, N = 128, K = 16 each) into a
//     128-column TMEM accumulator and commits them to an mbarrier;
//   * warp w reads accumulator lanes 32 (w % 4) .. +31, columns 32 (w / 4)
//     .. +31 back with tcgen05.ld, adds the bias, applies ReLU, rounds to
//     bf16 and writes the next layer's operand; the last layer (N padded to
//     16) adds the residual base.
// The accumulators live in TMEM, so the epilogue needs 32 registers per
// chunk instead of 64 per thread for a whole layer.  Every wait on the
// mbarrier is bounded: on timeout the block records an error bit, waits
// (bounded) for its last commit, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "device_api.hpp"
#include "features.cuh"

namespace cr {
namespace {

constexpr int kTcRows = 128;
constexpr int kTcThreads = 512;  // 4 threads per row for the features; 16 warps share the epilogue
constexpr int kTmemCols = 128;
constexpr uint32_t kSpinLimit = 1u << 26;  // bounded waits (far longer than one layer's MMAs)

// Byte offset of element (r, k) in a K-major no-swizzle operand with K
// elements per row: 8x8 core matrices of bf16.
__host__ __device__ constexpr uint32_t coreOffset(uint32_t r, uint32_t k, uint32_t K) {
  return (r >> 3) * (K * 16u) + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor: start address, leading byte offset
// (between core matrices along K), stride byte offset (between 8-row
// groups), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smemDesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;  // version
  return d;
}

// Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N and M.
__host__ __device__ constexpr uint32_t instrDesc(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mmaBf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void commitTo(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ bool tryWait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool waitParity(uint32_t mbar, uint32_t parity) {
  for (uint32_t i = 0; i < kSpinLimit; ++i)
    if (tryWait(mbar, parity)) return true;
  return false;
}

__device__ __forceinline__ void fenceAsyncShared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tcFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tcFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive fp32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmemLoad32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmemLoad4(uint32_t taddr, float* v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t packBf16(float lo, float hi) {
  return static_cast<uint32_t>(__bfloat16_as_ushort(__float2bfloat16(lo))) |
         (static_cast<uint32_t>(__bfloat16_as_ushort(__float2bfloat16(hi))) << 16);
}

// Shared memory plan (bytes).
constexpr uint32_t kW1Bytes = kMlpHidden * kFeatureWidth * 2;  // 128 x 112
constexpr uint32_t kWBytes = kMlpHidden * kMlpHidden * 2;      // 128 x 128
constexpr uint32_t kW4Rows = 16;                               // N of the last layer, padded
constexpr uint32_t kW4Bytes = kW4Rows * kMlpHidden * 2;
constexpr uint32_t kActBytes = kTcRows * kMlpHidden * 2;
constexpr uint32_t kOffW1 = 0;
constexpr uint32_t kOffW2 = kOffW1 + kW1Bytes;
constexpr uint32_t kOffW3 = kOffW2 + kWBytes;
constexpr uint32_t kOffW4 = kOffW3 + kWBytes;
constexpr uint32_t kOffA0 = kOffW4 + kW4Bytes;
constexpr uint32_t kOffA1 = kOffA0 + kActBytes;
constexpr uint32_t kOffBias = kOffA1 + kActBytes;                    // 3 x 128 + 16 floats
constexpr uint32_t kOffBar = kOffBias + (3 * kMlpHidden + 16) * 4;  // mbarrier (8 B) + TMEM address (4 B)
constexpr uint32_t kTcSmem = kOffBar + 16 + 128;                    // + alignment slack

// Row (pose * N + ommatidium) processed at position x: poses in order, the
// ommatidia of a pose in the eye's direction order, so that a tile's rows
// are neighbouring ommatidia whose neighbour statistics overlap in L1.
__device__ __forceinline__ uint64_t rowAt(uint64_t x, uint32_t N, const uint32_t* __restrict__ order) {
  const uint64_t p = x / N;
  const uint32_t j = static_cast<uint32_t>(x - p * N);
  return p * N + (order ? __ldg(order + j) : j);
}

// Stages W[in x out] (global, bf16, row-major) as a K-major operand of
// `rows` output rows (zero beyond `out`) and `in` columns.
__device__ void stageWeights(unsigned char* dst, const __nv_bfloat16* __restrict__ w, int in, int out, int rows) {
  for (int e = threadIdx.x; e < rows * in; e += blockDim.x) {
    const int n = e / in, k = e % in;
    const __nv_bfloat16 v = n < out ? w[static_cast<size_t>(k) * out + n] : __float2bfloat16(0.f);
    *reinterpret_cast<__nv_bfloat16*>(dst + coreOffset(n, k, in)) = v;
  }
}

__global__ void __launch_bounds__(kTcThreads, 1)
    inferTcKernel(const float* __restrict__ stats, const float4* __restrict__ omm, const int* __restrict__ nb,
                  uint32_t N, uint64_t rows, MlpWeights w, bool residual, float* __restrict__ out,
                  uint32_t* errFlag, const uint32_t* __restrict__ order) {
  extern __shared__ __align__(128) unsigned char smemRaw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smemRaw) + 127) & ~uintptr_t(127));
  float* bias = reinterpret_cast<float*>(sm + kOffBias);  // b1 | b2 | b3 | b4 (16)
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kOffBar);
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(sm + kOffBar + 8);
  const int tid = threadIdx.x, warp = tid >> 5;

  stageWeights(sm + kOffW1, w.w1, kFeatureWidth, kMlpHidden, kMlpHidden);
  stageWeights(sm + kOffW2, w.w2, kMlpHidden, kMlpHidden, kMlpHidden);
  stageWeights(sm + kOffW3, w.w3, kMlpHidden, kMlpHidden, kMlpHidden);
  stageWeights(sm + kOffW4, w.w4, kMlpHidden, kMlpOut, kW4Rows);
  for (int e = tid; e < kMlpHidden; e += kTcThreads) {
    bias[e] = w.b1[e];
    bias[kMlpHidden + e] = w.b2[e];
    bias[2 * kMlpHidden + e] = w.b3[e];
  }
  if (tid < 16) bias[3 * kMlpHidden + tid] = tid < kMlpOut ? w.b4[tid] : 0.f;
  const uint32_t mbar = smemAddr(bar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(tmemSlot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fenceAsyncShared();
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = *tmemSlot;
  const int lq = warp & 3, cb = warp >> 2;  // TMEM lane quarter and 32-column block of this warp
  const uint32_t laneBase = tmem + (static_cast<uint32_t>(lq * 32) << 16);
  const int myRow = lq * 32 + (tid & 31);   // tile row whose accumulators this thread reads

  uint32_t phase = 0;
  bool ok = true;
  const uint64_t tiles = (rows + kTcRows - 1) / kTcRows;
  const uint32_t sW[4] = {smemAddr(sm + kOffW1), smemAddr(sm + kOffW2), smemAddr(sm + kOffW3), smemAddr(sm + kOffW4)};
  const uint32_t sA[2] = {smemAddr(sm + kOffA0), smemAddr(sm + kOffA1)};

  for (uint64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    // Features of row tid / 4 into A0 (K = 112 layout), a quarter per thread.
    {
      const uint32_t r = static_cast<uint32_t>(tid >> 2), q = static_cast<uint32_t>(tid & 3);
      const uint64_t fpos = tile * kTcRows + r;
      const uint64_t frow = fpos < rows ? rowAt(fpos, N, order) : fpos;
      unsigned char* a0 = sm + kOffA0;
      auto put = [a0, r](int k, __nv_bfloat16 v) {
        *reinterpret_cast<__nv_bfloat16*>(a0 + coreOffset(r, static_cast<uint32_t>(k), kFeatureWidth)) = v;
      };
      static constexpr int kBegin[4] = {0, 1, 3, 5}, kEnd[4] = {1, 3, 5, kNeighbours};
      if (fpos < rows) {
        feat::featureRowTo(stats, omm, nb, N, frow, q == 0, kBegin[q], kEnd[q], put, nullptr);
      } else {
        for (int k = static_cast<int>(q); k < kFeatureWidth; k += 4) put(k, __float2bfloat16(0.f));
      }
    }
    // Four layers: A (buffer cur) x W -> TMEM -> bias/ReLU -> A (buffer 1-cur).
    int cur = 0;
    for (int layer = 0; layer < 4 && ok; ++layer) {
      const uint32_t K = layer == 0 ? kFeatureWidth : kMlpHidden;
      const uint32_t Nn = layer == 3 ? kW4Rows : kMlpHidden;
      fenceAsyncShared();
      tcFenceBefore();
      __syncthreads();
      tcFenceAfter();
      if (tid == 0) {
        const uint32_t idesc = instrDesc(kTcRows, Nn);
        for (uint32_t ks = 0; ks < K / 16; ++ks) {
          const uint64_t a = smemDesc(sA[cur] + ks * 256u, 128u, K * 16u);
          const uint64_t b = smemDesc(sW[layer] + ks * 256u, 128u, K * 16u);
          mmaBf16(tmem, a, b, idesc, ks > 0 ? 1u : 0u);
        }
        commitTo(mbar);
      }
      const bool landed = waitParity(mbar, phase);
      if (!__syncthreads_and(landed)) {  // one decision for the whole block
        ok = false;
        if (tid == 0) atomicOr(errFlag, kErrMmaTimeout);
        break;
      }
      phase ^= 1u;
      tcFenceAfter();
      if (layer < 3) {
        const float* b = bias + layer * kMlpHidden;
        unsigned char* dst = sm + (cur == 0 ? kOffA1 : kOffA0);
        const int c0 = cb * 32;
        float v[32];
        tmemLoad32(laneBase + static_cast<uint32_t>(c0), v);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          uint4 q;
          const int c = c0 + 8 * j;
          q.x = packBf16(fmaxf(v[8 * j] + b[c], 0.f), fmaxf(v[8 * j + 1] + b[c + 1], 0.f));
          q.y = packBf16(fmaxf(v[8 * j + 2] + b[c + 2], 0.f), fmaxf(v[8 * j + 3] + b[c + 3], 0.f));
          q.z = packBf16(fmaxf(v[8 * j + 4] + b[c + 4], 0.f), fmaxf(v[8 * j + 5] + b[c + 5], 0.f));
          q.w = packBf16(fmaxf(v[8 * j + 6] + b[c + 6], 0.f), fmaxf(v[8 * j + 7] + b[c + 7], 0.f));
          *reinterpret_cast<uint4*>(dst + coreOffset(static_cast<uint32_t>(myRow), static_cast<uint32_t>(c),
                                                     kMlpHidden)) = q;
        }
        cur ^= 1;
      } else if (cb == 0) {
        float v[4];
        tmemLoad4(laneBase, v);
        const uint64_t pos = tile * kTcRows + static_cast<uint64_t>(myRow);
        if (pos < rows) {
          const uint64_t row = rowAt(pos, N, order);
          const float* b4 = bias + 3 * kMlpHidden;
          for (int c = 0; c < 3; ++c) {
            const float y = v[c] + b4[c];
            out[3 * row + c] = residual ? stats[row * kFeatureStats + c] + y : y;
          }
        }
      }
    }
  }
  if (!ok && tid == 0) waitParity(mbar, phase);  // let a late commit land before the TMEM is freed
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

}  // namespace

cudaError_t inferDenoiserTc(const float* stats, const float4* omm, const int* nb, uint32_t N, uint32_t P,
                            const MlpWeights& w, float* out, uint32_t* errFlag, cudaStream_t stream, bool residual,
                            const uint32_t* order) {
  const uint64_t rows = static_cast<uint64_t>(N) * P;
  if (rows == 0) return cudaSuccess;
  static int smCount = 0;
  static bool attrSet = false;
  if (!attrSet) {
    cudaError_t e = cudaFuncSetAttribute(inferTcKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(kTcSmem));
    if (e != cudaSuccess) return e;
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smCount, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    attrSet = true;
  }
  const uint64_t tiles = (rows + kTcRows - 1) / kTcRows;
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(tiles, static_cast<uint64_t>(smCount)));
  inferTcKernel<<<grid, kTcThreads, kTcSmem, stream>>>(stats, omm, nb, N, rows, w, residual, out, errFlag, order);
  return cudaGetLastError();
}

}  // namespace cr
