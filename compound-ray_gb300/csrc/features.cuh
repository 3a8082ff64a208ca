// Denoiser feature rows, shared by the feature-row kernel, the mma.sync
// inference kernel (mlp.cu) and the tcgen05 inference kernel (mlp_tc.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "device_api.hpp"

namespace cr {
namespace feat {

// Feature rows.  Block 0 describes the ommatidium itself:
//   0-2 mean colour, 3-5 colour standard deviation x 4, 6 hit fraction,
//   7 log(1 + mean hit distance) / 4, 8-10 mean facing normal, 11-13 axis
//   direction (eye frame), 14 acceptance angle x 10 (radians).
// Blocks 1..6 describe the neighbours relative to it:
//   0-2 (neighbour mean - own mean) x 4, 3-5 neighbour deviation x 4,
//   6 hit-fraction difference, 7 log-distance difference, 8-10 neighbour
//   normal, 11-12 neighbour axis offset in the own axis' tangent frame and
//   13 its length, all in units of the own acceptance angle, 14 acceptance
//   angle ratio.
// Colour differences are formed in fp32 before the bf16 rounding.
struct OmmStats {
  float m[3], sd[3], hit, logDepth, n[3];
};

__device__ __forceinline__ OmmStats ommStats(const float* __restrict__ s) {
  OmmStats r;
  for (int k = 0; k < 3; ++k) {
    r.m[k] = s[k];
    r.sd[k] = sqrtf(fmaxf(s[3 + k] - s[k] * s[k], 0.f));
    r.n[k] = s[8 + k];
  }
  r.hit = s[6];
  const float depth = r.hit > 0.f ? s[7] / r.hit : 0.f;
  r.logDepth = log1pf(depth) * 0.25f;
  return r;
}

__device__ __forceinline__ float3 ommAxis(const float4* __restrict__ omm, uint32_t o, float& aa) {
  const float4 a = omm[2 * o], b = omm[2 * o + 1];
  const float il = rsqrtf(fmaxf(a.w * a.w + b.x * b.x + b.y * b.y, 1e-30f));
  aa = b.z;
  return make_float3(a.w * il, b.x * il, b.y * il);
}

// One feature row (row = pose * N + ommatidium): the own block when
// `withSelf`, neighbour blocks [jBegin, jEnd) and, when jEnd is the last
// neighbour, the zero padding; the residual base (own mean colour) when
// `base` is given.
// `put(k, v)` stores feature k of the row.
template <typename Put>
__device__ __forceinline__ void featureRowTo(const float* __restrict__ stats, const float4* __restrict__ omm,
                                             const int* __restrict__ nb, uint32_t N, size_t row, bool withSelf,
                                             int jBegin, int jEnd, Put put, float* __restrict__ base) {
  const uint32_t p = static_cast<uint32_t>(row / N), o = static_cast<uint32_t>(row % N);
  const float* sp = stats + static_cast<size_t>(p) * N * kFeatureStats;
  const OmmStats me = ommStats(sp + static_cast<size_t>(o) * kFeatureStats);
  float aa;
  const float3 d = ommAxis(omm, o, aa);
  float f[kFeatBlock];
  if (withSelf) {
    for (int k = 0; k < 3; ++k) {
      f[k] = me.m[k];
      f[3 + k] = me.sd[k] * 4.0f;
      f[8 + k] = me.n[k];
    }
    f[6] = me.hit;
    f[7] = me.logDepth;
    f[11] = d.x;
    f[12] = d.y;
    f[13] = d.z;
    f[14] = aa * 10.0f;
    for (int k = 0; k < kFeatBlock; ++k) put(k, __float2bfloat16(f[k]));
  }
  if (base) {
    base[3 * row] = me.m[0];
    base[3 * row + 1] = me.m[1];
    base[3 * row + 2] = me.m[2];
  }
  if (jBegin >= jEnd) return;
  const float inva = 1.0f / fmaxf(aa, 1e-6f);
  // tangent frame of the own axis
  float3 t1 = fabsf(d.y) < 0.9f ? make_float3(d.z, 0.f, -d.x) : make_float3(0.f, -d.z, d.y);
  const float il = rsqrtf(fmaxf(t1.x * t1.x + t1.y * t1.y + t1.z * t1.z, 1e-30f));
  t1 = make_float3(t1.x * il, t1.y * il, t1.z * il);
  const float3 t2 = make_float3(d.y * t1.z - d.z * t1.y, d.z * t1.x - d.x * t1.z, d.x * t1.y - d.y * t1.x);
  for (int j = jBegin; j < jEnd; ++j) {
    const uint32_t q = static_cast<uint32_t>(nb[kNeighbours * o + j]);
    const OmmStats ns = ommStats(sp + static_cast<size_t>(q) * kFeatureStats);
    float qa;
    const float3 e = ommAxis(omm, q, qa);
    for (int k = 0; k < 3; ++k) {
      f[k] = (ns.m[k] - me.m[k]) * 4.0f;
      f[3 + k] = ns.sd[k] * 4.0f;
      f[8 + k] = ns.n[k];
    }
    f[6] = ns.hit - me.hit;
    f[7] = ns.logDepth - me.logDepth;
    const float3 g = make_float3(e.x - d.x, e.y - d.y, e.z - d.z);
    const float u = (g.x * t1.x + g.y * t1.y + g.z * t1.z) * inva, v = (g.x * t2.x + g.y * t2.y + g.z * t2.z) * inva;
    f[11] = u;
    f[12] = v;
    f[13] = sqrtf(u * u + v * v);
    f[14] = qa * inva;
    for (int k = 0; k < kFeatBlock; ++k) put(kFeatBlock * (j + 1) + k, __float2bfloat16(f[k]));
  }
  if (jEnd == kNeighbours)
    for (int k = kFeatBlock * (kNeighbours + 1); k < kFeatureWidth; ++k) put(k, __float2bfloat16(0.f));
}

// The per-(pose, ommatidium) values a feature row reads, derived once:
// three float4 (m0, m1, m2, 4 sd0), (4 sd1, 4 sd2, hit, logDepth),
// (n0, n1, n2, 0), the same float operations as ommStats.
__device__ __forceinline__ void deriveStats(const float* __restrict__ s, float4* __restrict__ out) {
  const OmmStats r = ommStats(s);
  out[0] = make_float4(r.m[0], r.m[1], r.m[2], r.sd[0] * 4.0f);
  out[1] = make_float4(r.sd[1] * 4.0f, r.sd[2] * 4.0f, r.hit, r.logDepth);
  out[2] = make_float4(r.n[0], r.n[1], r.n[2], 0.f);
}

// Stores a block of kFeatBlock features from k0 on, converting them to bf16
// in pairs (the same round-to-nearest-even values as one at a time).
template <typename Put>
__device__ __forceinline__ void putBlock(int k0, const float* f, Put put) {
#pragma unroll
  for (int k = 0; k + 1 < kFeatBlock; k += 2) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(f[k], f[k + 1]);
    put(k0 + k, p.x);
    put(k0 + k + 1, p.y);
  }
  if (kFeatBlock & 1) put(k0 + kFeatBlock - 1, __float2bfloat16(f[kFeatBlock - 1]));
}

// featureRowTo from derived statistics (deriveStats, three float4 per row)
// and unit axes ((axis, acceptance angle) per ommatidium, as ommAxis gives
// them): the same feature values with vector loads and no transcendental
// functions per gathered ommatidium.
template <typename Put>
__device__ __forceinline__ void featureRowDerived(const float4* __restrict__ derived, const float4* __restrict__ axes,
                                                  const int* __restrict__ nb, uint32_t N, size_t row, bool withSelf,
                                                  int jBegin, int jEnd, Put put) {
  const uint32_t p = static_cast<uint32_t>(row / N), o = static_cast<uint32_t>(row % N);
  const float4* dp = derived + static_cast<size_t>(p) * N * 3;
  const float4 a0 = __ldg(dp + 3 * o), a1 = __ldg(dp + 3 * o + 1);
  const float4 ax = __ldg(axes + o);
  const float aa = ax.w;
  const float3 d = make_float3(ax.x, ax.y, ax.z);
  if (withSelf) {
    const float4 a2 = __ldg(dp + 3 * o + 2);
    const float f[kFeatBlock] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w, a2.x, a2.y, a2.z,
                                 d.x,  d.y,  d.z,  aa * 10.0f};
    putBlock(0, f, put);
  }
  if (jBegin >= jEnd) return;
  const float inva = 1.0f / fmaxf(aa, 1e-6f);
  float3 t1 = fabsf(d.y) < 0.9f ? make_float3(d.z, 0.f, -d.x) : make_float3(0.f, -d.z, d.y);
  const float il = rsqrtf(fmaxf(t1.x * t1.x + t1.y * t1.y + t1.z * t1.z, 1e-30f));
  t1 = make_float3(t1.x * il, t1.y * il, t1.z * il);
  const float3 t2 = make_float3(d.y * t1.z - d.z * t1.y, d.z * t1.x - d.x * t1.z, d.x * t1.y - d.y * t1.x);
  for (int j = jBegin; j < jEnd; ++j) {
    const uint32_t q = static_cast<uint32_t>(__ldg(nb + kNeighbours * o + j));
    const float4 b0 = __ldg(dp + 3 * q), b1 = __ldg(dp + 3 * q + 1), b2 = __ldg(dp + 3 * q + 2);
    const float4 e = __ldg(axes + q);
    const float3 g = make_float3(e.x - d.x, e.y - d.y, e.z - d.z);
    const float u = (g.x * t1.x + g.y * t1.y + g.z * t1.z) * inva, v = (g.x * t2.x + g.y * t2.y + g.z * t2.z) * inva;
    const float f[kFeatBlock] = {(b0.x - a0.x) * 4.0f, (b0.y - a0.y) * 4.0f, (b0.z - a0.z) * 4.0f,
                                 b0.w, b1.x, b1.y, b1.z - a1.z, b1.w - a1.w, b2.x, b2.y, b2.z,
                                 u, v, sqrtf(u * u + v * v), e.w * inva};
    putBlock(kFeatBlock * (j + 1), f, put);
  }
  if (jEnd == kNeighbours)
    for (int k = kFeatBlock * (kNeighbours + 1); k < kFeatureWidth; ++k) put(k, __float2bfloat16(0.f));
}

// The row into a linear bf16 array x[kFeatureWidth].
__device__ __forceinline__ void featureRow(const float* __restrict__ stats, const float4* __restrict__ omm,
                                           const int* __restrict__ nb, uint32_t N, size_t row, bool withSelf,
                                           int jBegin, int jEnd, __nv_bfloat16* __restrict__ x,
                                           float* __restrict__ base) {
  featureRowTo(stats, omm, nb, N, row, withSelf, jBegin, jEnd, [x](int k, __nv_bfloat16 v) { x[k] = v; }, base);
}

}  // namespace feat
}  // namespace cr
