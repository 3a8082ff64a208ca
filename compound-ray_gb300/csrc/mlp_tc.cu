// Fused denoiser inference on the 5th-generation tensor cores (tcgen05).
//
// Same function as inferKernel in mlp.cu (feature rows from the feature-render
// statistics, 112 -> 128 -> 128 -> 128 -> 8 network with bf16 operands and
// fp32 accumulation, bias + ReLU between layers, residual add), laid out for
// sm_103a's MMA unit as a two-role pipeline in one persistent block of 768
// threads per SM:
//   * all weights are staged once in shared memory as K-major UMMA operands
//     (transposed to [out][in]) in the canonical no-swizzle layout: 8-row x
//     16-byte core matrices, core matrices along K 128 bytes apart (leading
//     byte offset) and 8-row groups K*16 bytes apart (stride byte offset);
//   * feature warps 0-15 build the 112 features of each row of a 128-row
//     tile (four threads per row: own block + neighbour 0 / neighbours 1-2 /
//     3-4 / 5 + padding) from statistics derived once per row (deriveKernel:
//     three float4) and unit axes (axesKernel), into one of two tile
//     buffers, and signal it full on an mbarrier;
//   * network warps 16-23 take the full buffer: one elected thread issues
//     each layer's tcgen05.mma instructions (M = 128, N = 128, K = 16 each)
//     into a 128-column TMEM accumulator and commits them to an mbarrier.
//     Warps 16 + q and 20 + q read accumulator lanes 32 q .. +31, columns
//     0-63 and 64-127, with tcgen05.ld, add the bias, apply ReLU, round to
//     bf16 and write the next layer's operand into the same tile buffer (the
//     MMAs that read it are done);
//     the last layer (N padded to 16) adds the residual base and writes the
//     output, and its commit hands the buffer back to the feature warps.
// So the feature warps gather tile i + 1 (and i + 2) while the network warps
// run tile i.  Every mbarrier wait is bounded: on timeout the waiting side
// records an error bit and stops; the other side then times out too, the
// network warps wait (bounded) for their last commit, and the TMEM is freed.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "device_api.hpp"
#include "features.cuh"

namespace cr {
namespace {

constexpr int kTcRows = 128;
constexpr int kFeatThreads = 512;  // feature warps 0-15: four threads per row
constexpr int kNetThreads = 256;   // network warps 16-23: two per accumulator lane quarter
constexpr int kTcThreads = kFeatThreads + kNetThreads;
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

// Two floats to a bf16 pair, round to nearest even: one paired conversion
// (the conversion pipe's throughput limited the epilogue with two single
// ones).
__device__ __forceinline__ uint32_t packBf16(float lo, float hi) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&p);
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
// Two tile buffers: features (K = 112 layout), then in place the hidden
// activations of layers 1-3 (K = 128 layout).  Small enough that the rest of
// the SM's 256 KB stays L1 cache for the feature gathers.
constexpr uint32_t kOffB0 = kOffW4 + kW4Bytes;
constexpr uint32_t kOffB1 = kOffB0 + kActBytes;
constexpr uint32_t kOffBias = kOffB1 + kActBytes;                   // 3 x 128 + 16 floats
constexpr uint32_t kOffBar = kOffBias + (3 * kMlpHidden + 16) * 4;  // 5 mbarriers (8 B each) + TMEM address
constexpr uint32_t kTcSmem = kOffBar + 48 + 128;                    // + alignment slack
static_assert(kTcSmem <= 227 * 1024, "shared memory plan exceeds a block's limit");

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

// Derived statistics of every row and unit axes of every ommatidium for
// featureRowDerived.
__global__ void deriveKernel(const float* __restrict__ stats, uint64_t rows, float4* __restrict__ derived) {
  const uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  feat::deriveStats(stats + r * kFeatureStats, derived + 3 * r);
}

__global__ void axesKernel(const float4* __restrict__ omm, uint32_t N, float4* __restrict__ axes) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= N) return;
  float aa;
  const float3 d = feat::ommAxis(omm, o, aa);
  axes[o] = make_float4(d.x, d.y, d.z, aa);
}

__device__ __forceinline__ void mbarInit(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbarArrive(uint32_t mbar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(mbar) : "memory");
}

// AND of `v` over the network threads (named barrier 1).
__device__ __forceinline__ bool netAll(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, 1, %2, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}\n"
      : "=r"(r)
      : "r"(v ? 1u : 0u), "n"(kNetThreads)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void netSync() { asm volatile("bar.sync 1, %0;" ::"n"(kNetThreads) : "memory"); }

__global__ void __launch_bounds__(kTcThreads, 1)
    inferTcKernel(const float4* __restrict__ derived, const float4* __restrict__ axes, const int* __restrict__ nb,
                  uint32_t N, uint64_t rows, MlpWeights w, bool residual, float* __restrict__ out,
                  uint32_t* errFlag, const uint32_t* __restrict__ order) {
  extern __shared__ __align__(128) unsigned char smemRaw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smemRaw) + 127) & ~uintptr_t(127));
  float* bias = reinterpret_cast<float*>(sm + kOffBias);  // b1 | b2 | b3 | b4 (16)
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kOffBar);  // full0, full1, empty0, empty1, mma
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(sm + kOffBar + 40);
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
  const uint32_t fullBar[2] = {smemAddr(bars), smemAddr(bars + 1)};
  const uint32_t emptyBar[2] = {smemAddr(bars + 2), smemAddr(bars + 3)};
  const uint32_t mmaBar = smemAddr(bars + 4);
  if (tid == 0) {
    mbarInit(fullBar[0], kFeatThreads);
    mbarInit(fullBar[1], kFeatThreads);
    mbarInit(emptyBar[0], 1);
    mbarInit(emptyBar[1], 1);
    mbarInit(mmaBar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kFeatThreads / 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(tmemSlot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fenceAsyncShared();
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint64_t tiles = (rows + kTcRows - 1) / kTcRows;

  if (tid < kFeatThreads) {
    // Feature warps: tile i of this block into buffer i & 1.
    const uint32_t r = static_cast<uint32_t>(tid >> 2), q = static_cast<uint32_t>(tid & 3);
    static constexpr int kBegin[4] = {0, 1, 3, 5}, kEnd[4] = {1, 3, 5, kNeighbours};
    uint32_t i = 0;
    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++i) {
      const uint32_t b = i & 1u;
      if (i >= 2 && !waitParity(emptyBar[b], ((i >> 1) - 1u) & 1u)) {
        atomicOr(errFlag, kErrMmaTimeout);
        break;
      }
      unsigned char* fb = sm + (b ? kOffB1 : kOffB0);
      auto put = [fb, r](int k, __nv_bfloat16 v) {
        *reinterpret_cast<__nv_bfloat16*>(fb + coreOffset(r, static_cast<uint32_t>(k), kFeatureWidth)) = v;
      };
      const uint64_t fpos = tile * kTcRows + r;
      if (fpos < rows) {
        feat::featureRowDerived(derived, axes, nb, N, rowAt(fpos, N, order), q == 0, kBegin[q], kEnd[q], put);
      } else {
        for (int k = static_cast<int>(q); k < kFeatureWidth; k += 4) put(k, __float2bfloat16(0.f));
      }
      fenceAsyncShared();  // the tensor cores read the buffer through the async proxy
      mbarArrive(fullBar[b]);
    }
  } else {
    // Network warps: the four layers of tile i from buffer i & 1.
    const uint32_t tmem = *tmemSlot;
    const int lq = warp & 3;                               // TMEM lane quarter this warp may read
    const int half = (warp - kFeatThreads / 32) >> 2;      // columns 64 half .. +63
    const int m = lq * 32 + (tid & 31);                    // accumulator lane = tile row
    const uint32_t laneBase = tmem + (static_cast<uint32_t>(lq * 32) << 16);
    const bool issuer = tid == kFeatThreads;
    const uint32_t sW[4] = {smemAddr(sm + kOffW1), smemAddr(sm + kOffW2), smemAddr(sm + kOffW3),
                            smemAddr(sm + kOffW4)};
    const uint32_t sB[2] = {smemAddr(sm + kOffB0), smemAddr(sm + kOffB1)};
    uint32_t phase = 0;
    bool ok = true, pending = false;  // pending: a commit to mmaBar not yet waited for
    uint32_t i = 0;
    for (uint64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x, ++i) {
      const uint32_t b = i & 1u;
      if (!netAll(waitParity(fullBar[b], (i >> 1) & 1u))) {
        ok = false;
        if (issuer) atomicOr(errFlag, kErrMmaTimeout);
        break;
      }
      tcFenceAfter();
      unsigned char* h = sm + (b ? kOffB1 : kOffB0);
      for (int layer = 0; layer < 4; ++layer) {
        const uint32_t K = layer == 0 ? kFeatureWidth : kMlpHidden;
        const uint32_t Nn = layer == 3 ? kW4Rows : kMlpHidden;
        if (issuer) {
          const uint32_t idesc = instrDesc(kTcRows, Nn);
          for (uint32_t ks = 0; ks < K / 16; ++ks) {
            const uint64_t a = smemDesc(sB[b] + ks * 256u, 128u, K * 16u);
            const uint64_t bd = smemDesc(sW[layer] + ks * 256u, 128u, K * 16u);
            mmaBf16(tmem, a, bd, idesc, ks > 0 ? 1u : 0u);
          }
          if (layer == 3) commitTo(emptyBar[b]);  // the tile buffer is free once these MMAs are done
          commitTo(mmaBar);
        }
        pending = true;
        if (!netAll(waitParity(mmaBar, phase))) {
          ok = false;
          if (issuer) atomicOr(errFlag, kErrMmaTimeout);
          break;
        }
        pending = false;
        phase ^= 1u;
        tcFenceAfter();
        if (layer < 3) {
          const float* bl = bias + layer * kMlpHidden;
#pragma unroll 1
          for (int c0 = 64 * half; c0 < 64 * half + 64; c0 += 32) {
            float v[32];
            tmemLoad32(laneBase + static_cast<uint32_t>(c0), v);
            // the chunk's 32 biases first, then the values, then the stores
            float bb[32];
            const uint32_t bs = smemAddr(bl + c0);
#pragma unroll
            for (int k = 0; k < 8; ++k)
              asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                           : "=f"(bb[4 * k]), "=f"(bb[4 * k + 1]), "=f"(bb[4 * k + 2]), "=f"(bb[4 * k + 3])
                           : "r"(bs + 16u * k));
            uint32_t qs[16];
#pragma unroll
            for (int k = 0; k < 16; ++k)
              qs[k] = packBf16(fmaxf(v[2 * k] + bb[2 * k], 0.f), fmaxf(v[2 * k + 1] + bb[2 * k + 1], 0.f));
            const uint32_t hs = smemAddr(h);
#pragma unroll
            for (int j = 0; j < 4; ++j)
              asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(
                               hs + coreOffset(static_cast<uint32_t>(m), static_cast<uint32_t>(c0 + 8 * j), kMlpHidden)),
                           "r"(qs[4 * j]), "r"(qs[4 * j + 1]), "r"(qs[4 * j + 2]), "r"(qs[4 * j + 3])
                           : "memory");
          }
        } else if (half == 0) {
          float v[4];
          tmemLoad4(laneBase, v);
          const uint64_t pos = tile * kTcRows + static_cast<uint64_t>(m);
          if (pos < rows) {
            const uint64_t row = rowAt(pos, N, order);
            const float* b4 = bias + 3 * kMlpHidden;
            const float4 mc = __ldg(derived + 3 * row);  // the mean colour, as the statistics hold it
            const float mean[3] = {mc.x, mc.y, mc.z};
            for (int c = 0; c < 3; ++c) {
              const float y = v[c] + b4[c];
              out[3 * row + c] = residual ? mean[c] + y : y;
            }
          }
        }
        // The next MMA reads h (async proxy) and overwrites the accumulator
        // that every network thread has just read.
        fenceAsyncShared();
        tcFenceBefore();
        netSync();
        tcFenceAfter();
      }
    }
    if (!ok && pending && issuer) waitParity(mmaBar, phase);  // let a late commit land before the TMEM is freed
  }
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == kFeatThreads / 32) {
    const uint32_t tmem = *tmemSlot;
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// The bounded wait, on an mbarrier that nothing arrives on.
__global__ void waitProbeKernel(uint32_t polls, uint32_t* errFlag) {
  __shared__ uint64_t bar;
  const uint32_t mbar = smemAddr(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  bool landed = false;
  for (uint32_t i = 0; i < polls && !landed; ++i) landed = tryWait(mbar, 0);
  if (!landed && threadIdx.x == 0) atomicOr(errFlag, kErrMmaTimeout);
}

// ---------------------------------------------------------------------------
// Training GEMMs on the tcgen05 tensor cores: C[M x N] = sum_k a(m, k) b(n, k)
// with the operand conventions of gemmBf16 (mlp.cu):
//   a(m, k) = aTrans ? A[k * lda + m] : A[m * lda + k],
//   b(n, k) = bTrans ? B[n * ldb + k] : B[k * ldb + n],
// and its epilogues (0 fp32 store, 1 bias + ReLU to bf16 and the fp32
// pre-activation, 2 ReLU-derivative mask to bf16, 3 bias to fp32).
// One 256-thread block per 128 x 128 output tile (N padded to a multiple of
// 16 for the MMA), K in chunks of 64 staged by the threads into shared
// memory in the canonical K-major no-swizzle layout, 16 bytes per load; one
// thread issues the chunk's four tcgen05.mma (K 16 each) into the TMEM
// accumulator and commits them; warps w and w + 4 read accumulator lanes
// 32 w .. +31, columns 0-63 and 64-127.  grid.z > 1 splits
// K into slices that write partial tiles (ldc = N) for a reduction in slice
// order.  Waits are bounded; a timeout sets g_tcGemmErr.
// ---------------------------------------------------------------------------
constexpr int kGemmTile = 128;
constexpr int kGemmChunk = 64;
constexpr uint32_t kGemmStage = kGemmTile * kGemmChunk * 2;  // bytes per operand stage
// Dynamic shared memory per block, sized so that at most four blocks share
// an SM: their four 128-column accumulators fill its 512 TMEM columns, and
// no block ever waits in tcgen05.alloc.
constexpr uint32_t kGemmSmem = 56 * 1024;
static_assert(2 * kGemmStage + 128 <= kGemmSmem, "staging exceeds the block's shared memory");
constexpr uint32_t kGemmMaskOff = 8 * 32 * 33 * 4;  // after the eight warps' fp32 epilogue tiles
constexpr int kGemmMaskLd = 40;                     // bf16 per mask row: 80 bytes, 16-byte aligned rows
static_assert(kGemmMaskOff % 16 == 0, "mask tiles must start 16-byte aligned");
static_assert(kGemmMaskOff + 8 * 32 * kGemmMaskLd * 2 + 128 <= kGemmSmem,
              "epilogue tiles exceed the block's shared memory");
__device__ uint32_t g_tcGemmErr;

constexpr int kGemmThreads = 256;  // eight warps: two per accumulator lane quarter

// Stages rows [0, rowsValid) x chunk columns of an operand whose element
// (r, c) is at P[(row0 + r) * ld + k0 + c] (K contiguous: 8 elements per
// 16-byte load) or, when `kMajorInMemory` is false, at
// P[(k0 + c) * ld + row0 + r] (rows contiguous: 8 rows per 16-byte load,
// scattered to their core-matrix rows); zero outside rowsValid and kEnd.
__device__ __forceinline__ void stageOperand(unsigned char* dst, const __nv_bfloat16* __restrict__ P, int ld,
                                             bool kMajorInMemory, int row0, int rowsValid, int rowsPadded, int k0,
                                             int kEnd, int tid) {
  const bool vec = (reinterpret_cast<uintptr_t>(P) & 15) == 0 && (ld & 7) == 0;
  if (kMajorInMemory) {
    // groups of 8 consecutive k of one row
    for (int e = tid; e < rowsPadded * (kGemmChunk / 8); e += kGemmThreads) {
      const int r = e / (kGemmChunk / 8), c = (e % (kGemmChunk / 8)) * 8;
      const int k = k0 + c;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (r < rowsValid) {
        const __nv_bfloat16* src = P + static_cast<size_t>(row0 + r) * ld + k;
        if (vec && k + 8 <= kEnd) {
          v = *reinterpret_cast<const uint4*>(src);
        } else {
          uint16_t t[8];
          for (int j = 0; j < 8; ++j) t[j] = k + j < kEnd ? __bfloat16_as_ushort(src[j]) : 0;
          v = make_uint4(t[0] | (uint32_t(t[1]) << 16), t[2] | (uint32_t(t[3]) << 16), t[4] | (uint32_t(t[5]) << 16),
                         t[6] | (uint32_t(t[7]) << 16));
        }
      }
      *reinterpret_cast<uint4*>(dst + coreOffset(static_cast<uint32_t>(r), static_cast<uint32_t>(c), kGemmChunk)) = v;
    }
  } else {
    // 8 x 8 blocks (8 rows x 8 k), one per group of eight lanes: lane l8
    // loads the block's 8 rows at k = 8 kg + l8 (16 bytes, rows contiguous in
    // memory), the group transposes the block in three exchange rounds, and
    // lane l8 stores row l8's 8 k as one 16-byte row of a core matrix, so the
    // eight lanes of a store phase fill 128 contiguous bytes.
    const int lane = tid & 31, q = lane >> 3, l8 = lane & 7;
    const int groups = rowsPadded / 8, nBlocks = groups * (kGemmChunk / 8);  // nBlocks: a multiple of 4
    for (int base = (tid >> 5) * 4; base < nBlocks; base += kGemmThreads / 8) {
      const int b = base + q;  // < nBlocks for every lane: the warp runs each round whole
      const int g = b % groups, kg = b / groups;
      const int r = g * 8, k = k0 + kg * 8 + l8;
      uint32_t w0 = 0u, w1 = 0u, w2 = 0u, w3 = 0u;
      if (k < kEnd) {
        const __nv_bfloat16* src = P + static_cast<size_t>(k) * ld + row0 + r;
        if (vec && r + 8 <= rowsValid) {
          const uint4 v = *reinterpret_cast<const uint4*>(src);
          w0 = v.x; w1 = v.y; w2 = v.z; w3 = v.w;
        } else {
          uint32_t t[8];
          for (int j = 0; j < 8; ++j) t[j] = r + j < rowsValid ? __bfloat16_as_ushort(src[j]) : 0u;
          w0 = t[0] | (t[1] << 16); w1 = t[2] | (t[3] << 16); w2 = t[4] | (t[5] << 16); w3 = t[6] | (t[7] << 16);
        }
      }
      // Round 1, lanes l8 ^ 4: elements 4-7 of the low lanes for 0-3 of the high ones.
      {
        const bool hi = l8 & 4;
        const uint32_t r0 = __shfl_xor_sync(0xffffffffu, hi ? w0 : w2, 4);
        const uint32_t r1 = __shfl_xor_sync(0xffffffffu, hi ? w1 : w3, 4);
        if (hi) { w0 = r0; w1 = r1; } else { w2 = r0; w3 = r1; }
      }
      // Round 2, lanes l8 ^ 2: element pairs {2,3}, {6,7} against {0,1}, {4,5}.
      {
        const bool hi = l8 & 2;
        const uint32_t r0 = __shfl_xor_sync(0xffffffffu, hi ? w0 : w1, 2);
        const uint32_t r1 = __shfl_xor_sync(0xffffffffu, hi ? w2 : w3, 2);
        if (hi) { w0 = r0; w2 = r1; } else { w1 = r0; w3 = r1; }
      }
      // Round 3, lanes l8 ^ 1: odd elements of the even lane for even
      // elements of the odd lane, two per exchanged word.
      {
        const bool hi = l8 & 1;
        const uint32_t s0 = hi ? __byte_perm(w0, w1, 0x5410) : __byte_perm(w0, w1, 0x7632);
        const uint32_t s1 = hi ? __byte_perm(w2, w3, 0x5410) : __byte_perm(w2, w3, 0x7632);
        const uint32_t r0 = __shfl_xor_sync(0xffffffffu, s0, 1);
        const uint32_t r1 = __shfl_xor_sync(0xffffffffu, s1, 1);
        if (hi) {
          w0 = __byte_perm(r0, w0, 0x7610); w1 = __byte_perm(r0, w1, 0x7632);
          w2 = __byte_perm(r1, w2, 0x7610); w3 = __byte_perm(r1, w3, 0x7632);
        } else {
          w0 = __byte_perm(w0, r0, 0x5410); w1 = __byte_perm(w1, r0, 0x7610);
          w2 = __byte_perm(w2, r1, 0x5410); w3 = __byte_perm(w3, r1, 0x7610);
        }
      }
      *reinterpret_cast<uint4*>(dst + coreOffset(static_cast<uint32_t>(r + l8), static_cast<uint32_t>(kg * 8),
                                                 kGemmChunk)) = make_uint4(w0, w1, w2, w3);
    }
  }
}

template <int kMode>
__global__ void __launch_bounds__(kGemmThreads, 1)
    gemmTcKernel(int M, int N, int K, const __nv_bfloat16* __restrict__ A, int lda, bool aTrans,
                 const __nv_bfloat16* __restrict__ B, int ldb, bool bTrans, float* __restrict__ Cf,
                 __nv_bfloat16* __restrict__ Hb, int ldc, const float* __restrict__ bias,
                 const __nv_bfloat16* __restrict__ mask, int kSlice) {
  extern __shared__ __align__(128) unsigned char gemmSmem[];
  unsigned char* stage =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(gemmSmem) + 127) & ~uintptr_t(127));
  __shared__ uint64_t bar;
  __shared__ uint32_t tmemSlot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kGemmTile, n0 = blockIdx.x * kGemmTile;
  const int Mt = min(kGemmTile, M - m0);
  const int Nt = min(kGemmTile, N - n0);
  const uint32_t Nn = static_cast<uint32_t>((Nt + 15) & ~15);  // MMA N: a multiple of 16
  const int kBeg = kSlice ? static_cast<int>(blockIdx.z) * kSlice : 0;
  const int kEnd = kSlice ? min(K, kBeg + kSlice) : K;
  if (kSlice) Cf += static_cast<size_t>(blockIdx.z) * M * N;
  unsigned char* sA = stage;
  unsigned char* sB = stage + kGemmStage;
  const uint32_t mbar = smemAddr(&bar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(&tmemSlot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  const uint32_t tmem = tmemSlot;
  uint32_t phase = 0;
  bool ok = true, pending = false;
  for (int k0 = kBeg; k0 < kEnd && ok; k0 += kGemmChunk) {
    // a(m, k): K contiguous unless aTrans; b(n, k): K contiguous when bTrans.
    stageOperand(sA, A, lda, !aTrans, m0, Mt, kGemmTile, k0, kEnd, tid);
    stageOperand(sB, B, ldb, bTrans, n0, Nt, static_cast<int>(Nn), k0, kEnd, tid);
    fenceAsyncShared();
    tcFenceBefore();
    __syncthreads();
    tcFenceAfter();
    if (tid == 0) {
      const uint32_t idesc = instrDesc(kGemmTile, Nn);
      for (uint32_t ks = 0; ks < kGemmChunk / 16; ++ks) {
        const uint64_t a = smemDesc(smemAddr(sA) + ks * 256u, 128u, kGemmChunk * 16u);
        const uint64_t b = smemDesc(smemAddr(sB) + ks * 256u, 128u, kGemmChunk * 16u);
        mmaBf16(tmem, a, b, idesc, (k0 > kBeg || ks > 0) ? 1u : 0u);
      }
      commitTo(mbar);
    }
    pending = true;
    if (!__syncthreads_and(waitParity(mbar, phase))) {
      ok = false;
      if (tid == 0) atomicOr(&g_tcGemmErr, kErrMmaTimeout);
      break;
    }
    pending = false;
    phase ^= 1u;
    tcFenceAfter();
  }
  if (ok) {
    // Each warp turns its 32 rows x 32 columns through shared memory (the
    // staging area is free once the MMAs are done), so that a store writes
    // 32 consecutive columns of one row.
    const int lq = warp & 3, half = warp >> 2;  // lane quarter, and columns 64 half .. +63
    const uint32_t laneBase = tmem + (static_cast<uint32_t>(lq * 32) << 16);
    const bool empty = kEnd <= kBeg;  // no chunk ran: the accumulator holds nothing
    float* t = reinterpret_cast<float*>(stage) + warp * (32 * 33);
    // kMode 2: the warp's 32 x 32 block of the mask, read in 16-byte pieces
    // while the accumulators load, then turned through shared memory too.
    __nv_bfloat16* mt = reinterpret_cast<__nv_bfloat16*>(stage + kGemmMaskOff) + warp * (32 * kGemmMaskLd);
    const bool maskVec = kMode == 2 && (reinterpret_cast<uintptr_t>(mask) & 15) == 0 && (ldc & 7) == 0;
    for (int c0 = 64 * half; c0 < min(Nt, 64 * half + 64); c0 += 32) {
      uint4 mq[4];
      if (kMode == 2) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int m = m0 + lq * 32 + (lane >> 2) + 8 * i, cc = c0 + (lane & 3) * 8;
          mq[i] = make_uint4(0u, 0u, 0u, 0u);
          if (m < M) {
            const __nv_bfloat16* src = mask + static_cast<size_t>(m) * ldc + n0 + cc;
            if (maskVec && cc + 8 <= Nt) {
              mq[i] = __ldg(reinterpret_cast<const uint4*>(src));
            } else {
              uint16_t e[8];
              for (int j = 0; j < 8; ++j) e[j] = cc + j < Nt ? __bfloat16_as_ushort(src[j]) : 0;
              mq[i] = make_uint4(e[0] | (uint32_t(e[1]) << 16), e[2] | (uint32_t(e[3]) << 16),
                                 e[4] | (uint32_t(e[5]) << 16), e[6] | (uint32_t(e[7]) << 16));
            }
          }
        }
      }
      float v[32];
      if (!empty) tmemLoad32(laneBase + static_cast<uint32_t>(c0), v);
      else
        for (int j = 0; j < 32; ++j) v[j] = 0.f;
#pragma unroll
      for (int j = 0; j < 32; ++j) t[lane * 33 + j] = v[j];  // row `lane`, column j
      if (kMode == 2) {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          *reinterpret_cast<uint4*>(mt + ((lane >> 2) + 8 * i) * kGemmMaskLd + (lane & 3) * 8) = mq[i];
      }
      __syncwarp();
      const int n = n0 + c0 + lane;
      const bool colOk = c0 + lane < Nt;
      const float bn = (kMode == 1 || kMode == 3) && colOk ? bias[n] : 0.f;
#pragma unroll
      for (int r = 0; r < 32; ++r) {
        const int m = m0 + lq * 32 + r;
        if (m >= M || !colOk) continue;
        const size_t o = static_cast<size_t>(m) * ldc + n;
        const float acc = t[r * 33 + lane];
        if (kMode == 0) {
          Cf[o] = acc;
        } else if (kMode == 1) {
          const float z = acc + bn;
          Cf[o] = z;
          Hb[o] = __float2bfloat16(fmaxf(z, 0.f));
        } else if (kMode == 2) {
          Hb[o] = __float2bfloat16(__bfloat162float(mt[r * kGemmMaskLd + lane]) > 0.f ? acc : 0.f);
        } else {
          Cf[o] = acc + bn;
        }
      }
      __syncwarp();
    }
  }
  if (!ok && pending && tid == 0) waitParity(mbar, phase);  // let a late commit land before the TMEM is freed
  tcFenceBefore();
  __syncthreads();
  tcFenceAfter();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

__global__ void tcSplitReduceKernel(const float* __restrict__ part, int slices, int M, int N, float* __restrict__ C,
                                    int ldc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * N) return;
  const int m = i / N, n = i % N;
  float s = 0.f;
  for (int k = 0; k < slices; ++k) s += part[static_cast<size_t>(k) * M * N + i];
  C[static_cast<size_t>(m) * ldc + n] = s;
}

float* g_tcSplit = nullptr;
size_t g_tcSplitFloats = 0;

}  // namespace

cudaError_t gemmBf16Tc(int mode, int M, int N, int K, const void* A, int lda, bool aTrans, const void* B, int ldb,
                       bool bTrans, float* Cf, void* Hb, int ldc, const float* bias, const void* mask,
                       cudaStream_t stream) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  if (mode < 0 || mode > 3) return cudaErrorInvalidValue;
  const unsigned gx = static_cast<unsigned>((N + kGemmTile - 1) / kGemmTile);
  const unsigned gy = static_cast<unsigned>((M + kGemmTile - 1) / kGemmTile);
  auto a = static_cast<const __nv_bfloat16*>(A);
  auto b = static_cast<const __nv_bfloat16*>(B);
  auto h = static_cast<__nv_bfloat16*>(Hb);
  auto mk = static_cast<const __nv_bfloat16*>(mask);
  // Weight gradients: a long K over the minibatch and one or two output
  // tiles; K is split into slices of 128 summed afterwards in slice order.
  static bool attrSet = false;
  if (!attrSet) {
    const void* fns[4] = {reinterpret_cast<const void*>(gemmTcKernel<0>), reinterpret_cast<const void*>(gemmTcKernel<1>),
                          reinterpret_cast<const void*>(gemmTcKernel<2>), reinterpret_cast<const void*>(gemmTcKernel<3>)};
    for (const void* f : fns) {
      const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
      if (e != cudaSuccess) return e;
    }
    attrSet = true;
  }
  if (mode == 0 && K >= 1024 && gx * gy < 64) {
    const int slice = 128, slices = (K + slice - 1) / slice;
    const size_t need = static_cast<size_t>(slices) * M * N;
    if (need > g_tcSplitFloats) {
      if (g_tcSplit) cudaFree(g_tcSplit);
      g_tcSplit = nullptr;
      g_tcSplitFloats = 0;
      const cudaError_t e = cudaMalloc(&g_tcSplit, need * sizeof(float));
      if (e != cudaSuccess) return e;
      g_tcSplitFloats = need;
    }
    gemmTcKernel<0><<<dim3(gx, gy, slices), kGemmThreads, kGemmSmem, stream>>>(M, N, K, a, lda, aTrans, b, ldb, bTrans,
                                                                       g_tcSplit, nullptr, N, nullptr, nullptr, slice);
    tcSplitReduceKernel<<<(M * N + 255) / 256, 256, 0, stream>>>(g_tcSplit, slices, M, N, Cf, ldc);
    return cudaGetLastError();
  }
  const dim3 grid(gx, gy);
  switch (mode) {
    case 0: gemmTcKernel<0><<<grid, kGemmThreads, kGemmSmem, stream>>>(M, N, K, a, lda, aTrans, b, ldb, bTrans, Cf, h, ldc, bias, mk, 0); break;
    case 1: gemmTcKernel<1><<<grid, kGemmThreads, kGemmSmem, stream>>>(M, N, K, a, lda, aTrans, b, ldb, bTrans, Cf, h, ldc, bias, mk, 0); break;
    case 2: gemmTcKernel<2><<<grid, kGemmThreads, kGemmSmem, stream>>>(M, N, K, a, lda, aTrans, b, ldb, bTrans, Cf, h, ldc, bias, mk, 0); break;
    default: gemmTcKernel<3><<<grid, kGemmThreads, kGemmSmem, stream>>>(M, N, K, a, lda, aTrans, b, ldb, bTrans, Cf, h, ldc, bias, mk, 0); break;
  }
  return cudaGetLastError();
}

cudaError_t takeTcGemmError(uint32_t* flags) {
  cudaError_t e = cudaMemcpyFromSymbol(flags, g_tcGemmErr, sizeof(uint32_t));
  if (e != cudaSuccess) return e;
  const uint32_t zero = 0;
  return cudaMemcpyToSymbol(g_tcGemmErr, &zero, sizeof(uint32_t));
}

cudaError_t launchWaitProbe(uint32_t polls, uint32_t* errFlag, cudaStream_t stream) {
  waitProbeKernel<<<1, 32, 0, stream>>>(polls, errFlag);
  return cudaGetLastError();
}

cudaError_t deriveFeatureStats(const float* stats, const float4* omm, uint32_t N, uint32_t P, float4* derived,
                               float4* axes, cudaStream_t stream) {
  const uint64_t rows = static_cast<uint64_t>(N) * P;
  if (rows == 0) return cudaSuccess;
  deriveKernel<<<static_cast<unsigned>((rows + 255) / 256), 256, 0, stream>>>(stats, rows, derived);
  axesKernel<<<(N + 255) / 256, 256, 0, stream>>>(omm, N, axes);
  return cudaGetLastError();
}

cudaError_t inferDenoiserTc(const float4* derived, const float4* axes, const int* nb, uint32_t N, uint32_t P,
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
  inferTcKernel<<<grid, kTcThreads, kTcSmem, stream>>>(derived, axes, nb, N, rows, w, residual, out, errFlag, order);
  return cudaGetLastError();
}

}  // namespace cr
