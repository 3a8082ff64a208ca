// Compound-eye render kernels for sm_103a.
//
// One fused kernel per batch of poses: every warp owns up to 32 samples of
// one ommatidium (or several whole ommatidia when spp < 32), keeps their
// XORWOW states in registers across all poses of the batch, and per pose
//   1. draws one normal and one uniform number per sample (cuRAND, as
//      libEyeRenderer3/shaders.cu:680-695),
//   2. builds the splayed ray (shaders.cu:648-709),
//   3. finds the closest triangle in the BVH2 (replaces optixTrace,
//      shaders.cu:110-137),
//   4. shades it with the lighting-off whitted closest-hit program or the
//      miss program (shaders.cu:740-811, cuda/LocalGeometry.h:55-156),
//   5. scales by 1/spp (shaders.cu:730) and reduces the warp's samples with
//      shuffles, replacing the per-sample compound buffer and the second
//      summing launch (shaders.cu:341-347, 396-406).
//
// This translation unit is compiled with --use_fast_math, as the reference's
// shaders are (CMakeLists.txt:154-159, 193), so the random draws, ray
// directions and shading follow the same approximate maths.  The triangle
// test alone runs on explicitly rounded PTX (add/mul/fma/div .rn without
// .ftz) so that a CPU implementation can repeat it bit for bit.
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <cstdint>
#include <type_traits>

#include "device_api.hpp"

namespace cr {
namespace {

// ---------------------------------------------------------------------------
// Small float3 algebra with the operator forms of the reference shaders.
// ---------------------------------------------------------------------------
struct v3 {
  float x, y, z;
};
__device__ __forceinline__ v3 mk(float x, float y, float z) { return v3{x, y, z}; }
__device__ __forceinline__ v3 operator+(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ v3 operator-(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ v3 operator*(float s, v3 a) { return mk(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ v3 operator*(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3 cross(v3 a, v3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ v3 normalize(v3 v) {
  const float invLen = 1.0f / sqrtf(dot(v, v));
  return v * invLen;
}

// cos/sin of a float argument; with --use_fast_math these are the fast
// hardware approximations, as in the reference build.
__device__ __forceinline__ v3 rotatePoint(v3 point, float angle, v3 axis) {
  return cosf(angle) * point + sinf(angle) * cross(axis, point) + (1 - cosf(angle)) * dot(axis, point) * axis;
}

// ---------------------------------------------------------------------------
// Explicitly rounded single-precision operations (no FTZ, no contraction).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float xadd(float a, float b) {
  float r;
  asm("add.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float xsub(float a, float b) {
  float r;
  asm("sub.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float xmul(float a, float b) {
  float r;
  asm("mul.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float xfma(float a, float b, float c) {
  float r;
  asm("fma.rn.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float xdiv(float a, float b) {
  float r;
  asm("div.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float xsqrt(float a) {
  float r;
  asm("sqrt.rn.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}
__device__ __forceinline__ float xneg(float a) { return __int_as_float(__float_as_int(a) ^ 0x80000000); }

__device__ __forceinline__ float sel3(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

// Ray set up for the watertight triangle test (Woop, Benthin, Wald,
// "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013) and the slab test.
//
// Child boxes are stored as centre c and half-extent e.  Per axis the entry
// and exit distances are
//   mid = c * idir + nox            (nox = -origin * idir, one fma)
//   half = e * |idir| + slack       (one fma, |.| is an operand modifier)
//   near = mid - half, far = mid + half
// which puts the slab test on the fma pipe instead of min/max on the ALU pipe.
// idir comes from the hardware reciprocal approximation (<= 1 ulp).  All
// rounding (idir, nox, the two fmas, the add) stays within 5 ulp of
// (|c| + |e| + |origin|) * |idir|; every plane of the scene lies within
// `extent` of the world origin, so
//   slack = (extent + |origin|) * |idir| * 2^-21   (8 ulp of that bound)
// makes every computed box interval a superset of the exact one: no box
// holding a hit the triangle test would accept is ever culled.
struct Ray {
  float idx, idy, idz;
  float nox, noy, noz;
  float slx, sly, slz;
  int kx, ky, kz;
  float nSx, nSy, Sz;  // -Sx, -Sy, Sz of the shear
  float okx, oky, okz;
};

__device__ __forceinline__ float rcpApprox(float d) {
  const float tiny = 1e-20f;
  const float dd = fabsf(d) < tiny ? copysignf(tiny, d) : d;
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(dd));
  return r;
}

__device__ __forceinline__ Ray setupRay(v3 o, v3 d, float extent) {
  Ray r;
  r.idx = rcpApprox(d.x);
  r.idy = rcpApprox(d.y);
  r.idz = rcpApprox(d.z);
  r.nox = -o.x * r.idx;
  r.noy = -o.y * r.idy;
  r.noz = -o.z * r.idz;
  r.slx = (extent + fabsf(o.x)) * fabsf(r.idx) * 4.76837158e-07f;
  r.sly = (extent + fabsf(o.y)) * fabsf(r.idy) * 4.76837158e-07f;
  r.slz = (extent + fabsf(o.z)) * fabsf(r.idz) * 4.76837158e-07f;
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = 0;
  float m = ax;
  if (ay > m) {
    kz = 1;
    m = ay;
  }
  if (az > m) kz = 2;
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  const float dkz = sel3(d.x, d.y, d.z, kz);
  if (dkz < 0.0f) {
    const int t = kx;
    kx = ky;
    ky = t;
  }
  r.kx = kx;
  r.ky = ky;
  r.kz = kz;
  r.Sz = xdiv(1.0f, dkz);
  r.nSx = xneg(xmul(sel3(d.x, d.y, d.z, kx), r.Sz));
  r.nSy = xneg(xmul(sel3(d.x, d.y, d.z, ky), r.Sz));
  r.okx = sel3(o.x, o.y, o.z, kx);
  r.oky = sel3(o.x, o.y, o.z, ky);
  r.okz = sel3(o.x, o.y, o.z, kz);
  return r;
}

struct Hit {
  float t;
  uint32_t id;   // original triangle id, 0xffffffff = none
  uint32_t pos;  // BVH position of the triangle
  float U, V, W, det;
};

// Watertight test of one triangle; updates `h` when the hit is closer in the
// (t, id) order and lies in [tmin, h.t].
__device__ __forceinline__ void testTriangle(const Ray& r, float4 v0, float4 v1, float4 v2, uint32_t pos, float tmin,
                                             Hit& h) {
  const float Akx = xsub(sel3(v0.x, v0.y, v0.z, r.kx), r.okx);
  const float Aky = xsub(sel3(v0.x, v0.y, v0.z, r.ky), r.oky);
  const float Akz = xsub(sel3(v0.x, v0.y, v0.z, r.kz), r.okz);
  const float Bkx = xsub(sel3(v1.x, v1.y, v1.z, r.kx), r.okx);
  const float Bky = xsub(sel3(v1.x, v1.y, v1.z, r.ky), r.oky);
  const float Bkz = xsub(sel3(v1.x, v1.y, v1.z, r.kz), r.okz);
  const float Ckx = xsub(sel3(v2.x, v2.y, v2.z, r.kx), r.okx);
  const float Cky = xsub(sel3(v2.x, v2.y, v2.z, r.ky), r.oky);
  const float Ckz = xsub(sel3(v2.x, v2.y, v2.z, r.kz), r.okz);
  const float Ax = xfma(r.nSx, Akz, Akx);
  const float Ay = xfma(r.nSy, Akz, Aky);
  const float Bx = xfma(r.nSx, Bkz, Bkx);
  const float By = xfma(r.nSy, Bkz, Bky);
  const float Cx = xfma(r.nSx, Ckz, Ckx);
  const float Cy = xfma(r.nSy, Ckz, Cky);
  float U = xfma(Cx, By, xneg(xmul(Cy, Bx)));
  float V = xfma(Ax, Cy, xneg(xmul(Ay, Cx)));
  float W = xfma(Bx, Ay, xneg(xmul(By, Ax)));
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    const double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
    const double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
    const double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
    U = __double2float_rn(__dsub_rn(CxBy, CyBx));
    V = __double2float_rn(__dsub_rn(AxCy, AyCx));
    W = __double2float_rn(__dsub_rn(BxAy, ByAx));
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return;
  const float det = xadd(xadd(U, V), W);
  if (det == 0.0f) return;
  const float Az = xmul(r.Sz, Akz);
  const float Bz = xmul(r.Sz, Bkz);
  const float Cz = xmul(r.Sz, Ckz);
  const float T = xfma(U, Az, xfma(V, Bz, xmul(W, Cz)));
  const float t = xdiv(T, det);
  if (!(t >= tmin && t <= h.t)) return;
  const uint32_t id = __float_as_uint(v0.w);
  if (t == h.t && id >= h.id) return;
  h.t = t;
  h.id = id;
  h.pos = pos;
  h.U = U;
  h.V = V;
  h.W = W;
  h.det = det;
}

constexpr int kStackSize = 64;

__device__ __forceinline__ float max3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Entry/exit distances of one child box given as centre and half-extent.
__device__ __forceinline__ void childSpan(const Ray& r, float cx, float cy, float cz, float ex, float ey, float ez,
                                          float tmin, float tmax, float& tn, float& tf) {
  const float mx = fmaf(cx, r.idx, r.nox), hx = fmaf(ex, fabsf(r.idx), r.slx);
  const float my = fmaf(cy, r.idy, r.noy), hy = fmaf(ey, fabsf(r.idy), r.sly);
  const float mz = fmaf(cz, r.idz, r.noz), hz = fmaf(ez, fabsf(r.idz), r.slz);
  tn = max3(mx - hx, my - hy, fmaxf(mz - hz, tmin));
  tf = min3(mx + hx, my + hy, fminf(mz + hz, tmax));
}

// Traversal loop over the BVH2 from `node`, with `sp` deferred entries
// already on the stack; updates the closest hit `h`.  restart: when the
// stack runs empty and the hit is not within `guard` (distance, t * dlen),
// go on once more from the root (the near-field cut's second phase, in the
// same loop so the code is not inlined twice).
template <bool kCount, bool kAnyHit = false>
__device__ __forceinline__ void traverseFrom(const DevScene& sc, const Ray& r, float tmin, Hit& h, int* stack, int sp,
                                             int node, uint32_t* errFlag, uint32_t& nodeVisits, uint32_t& triTests,
                                             bool restart = false, float guard = 0.f, float dlen = 0.f) {
  for (;;) {
    if (node >= 0) {
      if (kCount) ++nodeVisits;
      const float4* n = sc.nodes + 4 * node;
      const float4 n0 = __ldg(n + 0);
      const float4 n1 = __ldg(n + 1);
      const float4 n2 = __ldg(n + 2);
      const int4 n3 = __ldg(reinterpret_cast<const int4*>(n + 3));
      float tn0, tf0, tn1, tf1;
      childSpan(r, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, tmin, h.t, tn0, tf0);
      childSpan(r, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, tmin, h.t, tn1, tf1);
      const bool hit0 = tn0 <= tf0;
      const bool hit1 = tn1 <= tf1;
      if (hit0 && hit1) {
        int first = n3.x, second = n3.y;
        if (tn1 < tn0) {
          first = n3.y;
          second = n3.x;
        }
        if (sp >= kStackSize) {
          atomicOr(errFlag, kErrStackOverflow);
          return;
        }
        stack[sp++] = second;
        node = first;
        continue;
      }
      if (hit0) {
        node = n3.x;
        continue;
      }
      if (hit1) {
        node = n3.y;
        continue;
      }
    } else {
      const uint32_t code = ~static_cast<uint32_t>(node);
      const uint32_t first = code >> 3;
      const uint32_t count = (code & 7u) + 1u;
      if (kCount) triTests += count;
      for (uint32_t k = 0; k < count; ++k) {
        const float4* t = sc.tris + 3 * (first + k);
        testTriangle(r, __ldg(t), __ldg(t + 1), __ldg(t + 2), first + k, tmin, h);
      }
      if (kAnyHit && h.id != 0xffffffffu) return;  // occlusion query: any hit will do
    }
    if (sp == 0) {
      if (restart) {
        restart = false;
        if (!(h.id != 0xffffffffu && h.t * dlen <= guard)) {
          node = 0;
          continue;
        }
      }
      return;
    }
    node = stack[--sp];
  }
}

// ---------------------------------------------------------------------------
// Wide BVH traversal (4 or 8 children per node, 8-bit quantised child boxes;
// layout in wbvh.hpp).  Per node and axis the ray's entry and exit distances
// to child k's planes p + q * s are fma(q, s * idir, p * idir - o * idir),
// the byte q turned into a float exactly through the mantissa (0x4B000000 |
// q is the float 2^23 + q); the slack of the BVH2 slab test (see setupRay)
// is folded into the per-node offsets and covers the same rounding, since
// every plane lies within the scene's extent.  Hit children are ordered
// near to far by a sorting network; the nearest is entered, the rest pushed
// far first.
// ---------------------------------------------------------------------------
constexpr int kWideStackSize = kWideStackEntries;

__device__ __forceinline__ float byteAsFloat(uint32_t w, int k) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, static_cast<uint32_t>(k) | 0x7650u)) - 8388608.0f;
}

// Compare-exchange of (key, ref) pairs: the smaller key first.
__device__ __forceinline__ void cex(float& ka, int& ra, float& kb, int& rb) {
  const bool sw = kb < ka;
  const float k = sw ? kb : ka;
  kb = sw ? ka : kb;
  ka = k;
  const int r = sw ? rb : ra;
  rb = sw ? ra : rb;
  ra = r;
}

template <int W>
__device__ __forceinline__ void sortChildren(float* key, int* ref) {
  if (W == 4) {
    cex(key[0], ref[0], key[1], ref[1]);
    cex(key[2], ref[2], key[3], ref[3]);
    cex(key[0], ref[0], key[2], ref[2]);
    cex(key[1], ref[1], key[3], ref[3]);
    cex(key[1], ref[1], key[2], ref[2]);
  } else {
    // 19 comparators, depth 6 (checked exhaustively on 0/1 inputs)
    cex(key[0], ref[0], key[2], ref[2]);
    cex(key[1], ref[1], key[3], ref[3]);
    cex(key[4], ref[4], key[6], ref[6]);
    cex(key[5], ref[5], key[7], ref[7]);
    cex(key[0], ref[0], key[4], ref[4]);
    cex(key[1], ref[1], key[5], ref[5]);
    cex(key[2], ref[2], key[6], ref[6]);
    cex(key[3], ref[3], key[7], ref[7]);
    cex(key[0], ref[0], key[1], ref[1]);
    cex(key[2], ref[2], key[3], ref[3]);
    cex(key[4], ref[4], key[5], ref[5]);
    cex(key[6], ref[6], key[7], ref[7]);
    cex(key[2], ref[2], key[4], ref[4]);
    cex(key[3], ref[3], key[5], ref[5]);
    cex(key[1], ref[1], key[4], ref[4]);
    cex(key[3], ref[3], key[6], ref[6]);
    cex(key[1], ref[1], key[2], ref[2]);
    cex(key[3], ref[3], key[4], ref[4]);
    cex(key[5], ref[5], key[6], ref[6]);
  }
}

// Traversal of the W-wide BVH from `node` with `sp` deferred entries, for at
// most `budget` node visits or leaves; returns true when the search is over
// (h holds the closest hit), false when the budget ran out (node and sp hold
// the position to go on from).
template <int W>
__device__ __forceinline__ bool traverseWide(const DevScene& sc, const Ray& r, float tmin, Hit& h, int* stack, int& sp,
                                             int& node, uint32_t* errFlag, uint32_t& nodeVisits, uint32_t& triTests,
                                             bool count, int budget) {
  constexpr int F = W == 8 ? 6 : 4;  // float4 per node
  const bool negX = r.idx < 0.f, negY = r.idy < 0.f, negZ = r.idz < 0.f;
  for (int it = 0; it < budget; ++it) {
    if (node >= 0) {
      if (count) ++nodeVisits;
      const float4* n = sc.wnodes + static_cast<size_t>(F) * node;
      const float4 n0 = __ldg(n);
      const uint32_t meta = __float_as_uint(n0.w);
      const int cnt = static_cast<int>(meta >> 24);
      const float sx = __uint_as_float((meta & 0xFFu) << 23) * r.idx;
      const float sy = __uint_as_float(((meta >> 8) & 0xFFu) << 23) * r.idy;
      const float sz = __uint_as_float(((meta >> 16) & 0xFFu) << 23) * r.idz;
      const float bx = fmaf(n0.x, r.idx, r.nox), by = fmaf(n0.y, r.idy, r.noy), bz = fmaf(n0.z, r.idz, r.noz);
      const float nbx = bx - r.slx, fbx = bx + r.slx;
      const float nby = by - r.sly, fby = by + r.sly;
      const float nbz = bz - r.slz, fbz = bz + r.slz;
      uint32_t lo[3][W / 4], hi[3][W / 4];
      int ref[W];
      if (W == 4) {
        const uint4 a = __ldg(reinterpret_cast<const uint4*>(n + 1));
        const uint4 b = __ldg(reinterpret_cast<const uint4*>(n + 2));
        const int4 c = __ldg(reinterpret_cast<const int4*>(n + 3));
        lo[0][0] = a.x;
        lo[1][0] = a.y;
        lo[2][0] = a.z;
        hi[0][0] = a.w;
        hi[1][0] = b.x;
        hi[2][0] = b.y;
        ref[0] = c.x;
        ref[1] = c.y;
        ref[2] = c.z;
        ref[3] = c.w;
      } else {
        const uint4 a = __ldg(reinterpret_cast<const uint4*>(n + 1));
        const uint4 b = __ldg(reinterpret_cast<const uint4*>(n + 2));
        const uint4 c = __ldg(reinterpret_cast<const uint4*>(n + 3));
        const int4 d = __ldg(reinterpret_cast<const int4*>(n + 4));
        const int4 e = __ldg(reinterpret_cast<const int4*>(n + 5));
        lo[0][0] = a.x;
        lo[0][W / 8] = a.y;
        lo[1][0] = a.z;
        lo[1][W / 8] = a.w;
        lo[2][0] = b.x;
        lo[2][W / 8] = b.y;
        hi[0][0] = b.z;
        hi[0][W / 8] = b.w;
        hi[1][0] = c.x;
        hi[1][W / 8] = c.y;
        hi[2][0] = c.z;
        hi[2][W / 8] = c.w;
        ref[0] = d.x;
        ref[1] = d.y;
        ref[2] = d.z;
        ref[3] = d.w;
        ref[W / 2] = e.x;
        ref[W / 2 + 1] = e.y;
        ref[W / 2 + 2] = e.z;
        ref[W / 2 + 3] = e.w;
      }
      // near planes: the lower ones along positive direction components
      uint32_t wn[3][W / 4], wf[3][W / 4];
#pragma unroll
      for (int j = 0; j < W / 4; ++j) {
        wn[0][j] = negX ? hi[0][j] : lo[0][j];
        wf[0][j] = negX ? lo[0][j] : hi[0][j];
        wn[1][j] = negY ? hi[1][j] : lo[1][j];
        wf[1][j] = negY ? lo[1][j] : hi[1][j];
        wn[2][j] = negZ ? hi[2][j] : lo[2][j];
        wf[2][j] = negZ ? lo[2][j] : hi[2][j];
      }
      float key[W];
      int nHit = 0;
#pragma unroll
      for (int k = 0; k < W; ++k) {
        const int j = k >> 2, b = k & 3;
        const float tnx = fmaf(byteAsFloat(wn[0][j], b), sx, nbx), tfx = fmaf(byteAsFloat(wf[0][j], b), sx, fbx);
        const float tny = fmaf(byteAsFloat(wn[1][j], b), sy, nby), tfy = fmaf(byteAsFloat(wf[1][j], b), sy, fby);
        const float tnz = fmaf(byteAsFloat(wn[2][j], b), sz, nbz), tfz = fmaf(byteAsFloat(wf[2][j], b), sz, fbz);
        const float tn = max3(tnx, tny, fmaxf(tnz, tmin));
        const float tf = min3(tfx, tfy, fminf(tfz, h.t));
        const bool hit = k < cnt && tn <= tf;
        key[k] = hit ? tn : INFINITY;
        nHit += hit ? 1 : 0;
      }
      if (nHit > 0) {
        sortChildren<W>(key, ref);
        if (sp + nHit - 1 > kWideStackSize) {
          atomicOr(errFlag, kErrStackOverflow);
          return true;
        }
#pragma unroll
        for (int k = W - 1; k >= 1; --k)
          if (k < nHit) stack[sp++] = ref[k];
        node = ref[0];
        continue;
      }
    } else {
      const uint32_t code = ~static_cast<uint32_t>(node);
      const uint32_t first = code >> 3;
      const uint32_t tcount = (code & 7u) + 1u;
      if (count) triTests += tcount;
      for (uint32_t k = 0; k < tcount; ++k) {
        const float4* t = sc.tris + 3 * (first + k);
        testTriangle(r, __ldg(t), __ldg(t + 1), __ldg(t + 2), first + k, tmin, h);
      }
    }
    if (sp == 0) return true;
    node = stack[--sp];
  }
  return false;
}

// Closest hit over the BVH2; returns the hit in `h` (h.id == ~0u on a miss).
// cut: null, or the pose's near-field cut (cutKernel): the subtrees whose
// boxes meet a ball around the eye are searched first, and a hit found there
// within the ball's guaranteed radius (in distance, hence t * dlen with dlen
// = |direction|) is final: every triangle nearer than it lies in the ball and
// so in one of those subtrees.  Otherwise the search continues from the root
// with the hit found so far.  Either way the result is the closest hit.
//
// beginTrace sets up that search (the hit, the stack with the cut entries,
// the start node) for traverseFrom; it returns false when the scene is empty
// (the ray misses).
__device__ __forceinline__ bool beginTrace(const DevScene& sc, const Ray& r, float tmin, float tmax, Hit& h,
                                           int* stack, int& sp, int& node, bool& restart, float& guard,
                                           const float4* __restrict__ cut) {
  h.t = tmax;
  h.id = 0xffffffffu;
  h.pos = 0;
  sp = 0;
  node = 0;
  restart = false;
  guard = 0.f;
  if (sc.triCount == 0) return false;
  if (cut) {
    const float4 hdr = __ldg(cut);
    const int count = __float_as_int(hdr.x);
    // Entries are stored far to near; the nearest hit box is entered first.
    // When no cut box is hit the search starts at the root directly.
    for (int k = 0; k < count; ++k) {
      const float4 a = __ldg(cut + 1 + 2 * k), b = __ldg(cut + 2 + 2 * k);
      float tn, tf;
      childSpan(r, a.x, a.y, a.z, b.x, b.y, b.z, tmin, h.t, tn, tf);
      if (tn <= tf) {
        if (restart) stack[sp++] = node;
        node = __float_as_int(a.w);
        restart = true;
      }
    }
    guard = hdr.y;
  }
  return true;
}

template <bool kCount>
__device__ __forceinline__ void traceClosest(const DevScene& sc, const Ray& r, float tmin, float tmax, Hit& h,
                                             uint32_t* errFlag, uint32_t& nodeVisits, uint32_t& triTests,
                                             const float4* __restrict__ cut = nullptr, float dlen = 0.f) {
  int stack[kStackSize];
  int sp, node;
  bool restart;
  float guard;
  if (!beginTrace(sc, r, tmin, tmax, h, stack, sp, node, restart, guard, cut)) return;
  traverseFrom<kCount>(sc, r, tmin, h, stack, sp, node, errFlag, nodeVisits, triTests, restart, guard, dlen);
}

// traverseFrom in bursts: at most `budget` steps (node visits or leaves)
// from the saved position (node, sp, restart; the stack holds the deferred
// entries), which is updated in place.  Returns true when the search is over
// (h holds the closest hit), false when the budget ran out first.  Lets a
// warp stop every few steps to hand finished lanes new rays.  Each lane
// visits the nodes and leaves in traverseFrom's order, but the loop is
// "while-while" (Aila and Laine, "Understanding the Efficiency of Ray
// Traversal on GPUs", HPG 2009): a lane descends inner nodes until it holds
// a leaf, and the warp tests leaves together, so lanes at inner nodes and
// lanes at leaves do not alternate step by step.  On the adaptive kernel's
// rays this is about 5% faster than the single-loop form; on the plain
// kernel's coherent rays it was not (its traverseFrom keeps one loop).
__device__ __forceinline__ bool traverseBurst(const DevScene& sc, const Ray& r, float tmin, Hit& h, int* stack,
                                              int& sp, int& node, bool& restart, float guard, float dlen,
                                              uint32_t* errFlag, int budget) {
  int it = 0;
  for (;;) {
    // Inner nodes until this lane reaches a leaf, the end of the search or
    // the budget.
    while (node >= 0) {
      if (it >= budget) return false;
      ++it;
      const float4* n = sc.nodes + 4 * node;
      const float4 n0 = __ldg(n + 0);
      const float4 n1 = __ldg(n + 1);
      const float4 n2 = __ldg(n + 2);
      const int4 n3 = __ldg(reinterpret_cast<const int4*>(n + 3));
      float tn0, tf0, tn1, tf1;
      childSpan(r, n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, tmin, h.t, tn0, tf0);
      childSpan(r, n1.z, n1.w, n2.x, n2.y, n2.z, n2.w, tmin, h.t, tn1, tf1);
      const bool hit0 = tn0 <= tf0;
      const bool hit1 = tn1 <= tf1;
      if (hit0 && hit1) {
        int first = n3.x, second = n3.y;
        if (tn1 < tn0) {
          first = n3.y;
          second = n3.x;
        }
        if (sp >= kStackSize) {
          atomicOr(errFlag, kErrStackOverflow);
          return true;
        }
        stack[sp++] = second;
        node = first;
        continue;
      }
      if (hit0) {
        node = n3.x;
        continue;
      }
      if (hit1) {
        node = n3.y;
        continue;
      }
      if (sp == 0) {
        if (restart) {
          restart = false;
          if (!(h.id != 0xffffffffu && h.t * dlen <= guard)) {
            node = 0;
            continue;
          }
        }
        return true;
      }
      node = stack[--sp];
    }
    if (it >= budget) return false;
    ++it;
    {
      const uint32_t code = ~static_cast<uint32_t>(node);
      const uint32_t first = code >> 3;
      const uint32_t count = (code & 7u) + 1u;
      for (uint32_t k = 0; k < count; ++k) {
        const float4* t = sc.tris + 3 * (first + k);
        testTriangle(r, __ldg(t), __ldg(t + 1), __ldg(t + 2), first + k, tmin, h);
      }
    }
    if (sp == 0) {
      if (restart) {
        restart = false;
        if (!(h.id != 0xffffffffu && h.t * dlen <= guard)) {
          node = 0;
          continue;
        }
      }
      return true;
    }
    node = stack[--sp];
  }
}

// Near-field cut of one pose: at most kCutEntries BVH subtrees (box + ref)
// covering every box that meets the ball of radius R around the pose
// position, grown from the root's children by repeatedly splitting the
// largest entry while the count allows; entries that miss the ball are
// dropped.  Header: (count, guaranteed radius, 0, 0) where the guaranteed
// radius R - rEye (rEye bounds how far ray origins lie from the pose
// position: maxRel times the sum of the pose axes' lengths) is shrunk by
// 1e-4 relative.  Entries sorted far to near by box distance.
__device__ __forceinline__ float boxDist2(float px, float py, float pz, float cx, float cy, float cz, float ex,
                                          float ey, float ez) {
  const float dx = fmaxf(fabsf(px - cx) - ex, 0.f), dy = fmaxf(fabsf(py - cy) - ey, 0.f),
              dz = fmaxf(fabsf(pz - cz) - ez, 0.f);
  return dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ void buildCut(const DevScene& sc, const float4* __restrict__ pose, float R, float maxRel,
                                         float4* __restrict__ out) {
  const float4 P0 = pose[0], X = pose[1], Y = pose[2], Z = pose[3];
  const float rEye = maxRel * (sqrtf(X.x * X.x + X.y * X.y + X.z * X.z) + sqrtf(Y.x * Y.x + Y.y * Y.y + Y.z * Y.z) +
                               sqrtf(Z.x * Z.x + Z.y * Z.y + Z.z * Z.z));
  const float rGuard = R - rEye;
  float c[kCutEntries][3], e[kCutEntries][3];
  int ref[kCutEntries];
  bool frozen[kCutEntries];
  int count = 0;
  const float R2 = R * R * 1.0002f;  // the ball test errs on the side of keeping a box
  if (rGuard > 0.f && sc.triCount > 0) {
    auto meets = [&](float cx, float cy, float cz, float ex, float ey, float ez) {
      return boxDist2(P0.x, P0.y, P0.z, cx, cy, cz, ex, ey, ez) <= R2;
    };
    auto children = [&](int node, float (*cc)[3], float (*ce)[3], int* cr, int& nc) {
      const float4* n = sc.nodes + 4 * node;
      const float4 n0 = n[0], n1 = n[1], n2 = n[2];
      const int4 n3 = reinterpret_cast<const int4*>(n)[3];
      nc = 0;
      if (meets(n0.x, n0.y, n0.z, n0.w, n1.x, n1.y)) {
        cc[nc][0] = n0.x; cc[nc][1] = n0.y; cc[nc][2] = n0.z;
        ce[nc][0] = n0.w; ce[nc][1] = n1.x; ce[nc][2] = n1.y;
        cr[nc++] = n3.x;
      }
      if (meets(n1.z, n1.w, n2.x, n2.y, n2.z, n2.w)) {
        cc[nc][0] = n1.z; cc[nc][1] = n1.w; cc[nc][2] = n2.x;
        ce[nc][0] = n2.y; ce[nc][1] = n2.z; ce[nc][2] = n2.w;
        cr[nc++] = n3.y;
      }
    };
    float cc[2][3], ce[2][3];
    int cr[2], nc;
    children(0, cc, ce, cr, nc);
    for (int k = 0; k < nc; ++k) {
      for (int a = 0; a < 3; ++a) {
        c[count][a] = cc[k][a];
        e[count][a] = ce[k][a];
      }
      ref[count] = cr[k];
      frozen[count] = false;
      ++count;
    }
    for (int iter = 0; iter < 4 * kCutEntries; ++iter) {
      int best = -1;
      float size = -1.f;
      for (int k = 0; k < count; ++k) {
        if (ref[k] < 0 || frozen[k]) continue;
        const float s = fmaxf(e[k][0], fmaxf(e[k][1], e[k][2]));
        if (s > size) {
          size = s;
          best = k;
        }
      }
      if (best < 0) break;
      children(ref[best], cc, ce, cr, nc);
      if (count - 1 + nc > kCutEntries) {
        frozen[best] = true;
        continue;
      }
      if (nc == 0) {  // the box meets the ball but neither child does
        --count;
        for (int a = 0; a < 3; ++a) {
          c[best][a] = c[count][a];
          e[best][a] = e[count][a];
        }
        ref[best] = ref[count];
        frozen[best] = frozen[count];
        continue;
      }
      for (int a = 0; a < 3; ++a) {
        c[best][a] = cc[0][a];
        e[best][a] = ce[0][a];
      }
      ref[best] = cr[0];
      frozen[best] = false;
      if (nc == 2) {
        for (int a = 0; a < 3; ++a) {
          c[count][a] = cc[1][a];
          e[count][a] = ce[1][a];
        }
        ref[count] = cr[1];
        frozen[count] = false;
        ++count;
      }
    }
    // far to near
    for (int i = 1; i < count; ++i)
      for (int j = i; j > 0; --j) {
        const float dj = boxDist2(P0.x, P0.y, P0.z, c[j][0], c[j][1], c[j][2], e[j][0], e[j][1], e[j][2]);
        const float dk =
            boxDist2(P0.x, P0.y, P0.z, c[j - 1][0], c[j - 1][1], c[j - 1][2], e[j - 1][0], e[j - 1][1], e[j - 1][2]);
        if (dj <= dk) break;
        for (int a = 0; a < 3; ++a) {
          const float tc = c[j][a], te = e[j][a];
          c[j][a] = c[j - 1][a];
          e[j][a] = e[j - 1][a];
          c[j - 1][a] = tc;
          e[j - 1][a] = te;
        }
        const int tr = ref[j];
        ref[j] = ref[j - 1];
        ref[j - 1] = tr;
      }
  }
  out[0] = make_float4(__int_as_float(count), rGuard * (1.0f - 1e-4f), 0.f, 0.f);
  for (int k = 0; k < count; ++k) {
    out[1 + 2 * k] = make_float4(c[k][0], c[k][1], c[k][2], __int_as_float(ref[k]));
    out[2 + 2 * k] = make_float4(e[k][0], e[k][1], e[k][2], 0.f);
  }
}

__global__ void cutKernel(DevScene sc, const float4* __restrict__ poses, uint32_t P, float R, float maxRel,
                          float4* __restrict__ cuts) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  buildCut(sc, poses + 4 * p, R, maxRel, cuts + static_cast<size_t>(p) * kCutStride);
}

// ---------------------------------------------------------------------------
// Shading (lighting off): closest hit and miss programs.
// ---------------------------------------------------------------------------
__device__ __forceinline__ v3 linearize(v3 c) { return mk(powf(c.x, 2.2f), powf(c.y, 2.2f), powf(c.z, 2.2f)); }

// One wrapped texel index along an axis of n texels.
__device__ __forceinline__ int wrapIndex(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// Texel-space position along one axis: wrap to [0, 1] (frac), scale, move to
// texel centres; i = first texel, A = weight of the second in 1/256 steps,
// rounded half up (the texture unit's 8-bit fractional filter weight).
__device__ __forceinline__ void texAxis(float u, int n, int& i, int& A) {
  float f = __fsub_rn(u, floorf(u));
  if (!(f >= 0.0f && f <= 1.0f)) f = 0.0f;  // NaN / infinite coordinates
  const float xb = __fsub_rn(__fmul_rn(f, static_cast<float>(n)), 0.5f);
  const float fl = floorf(xb);
  i = static_cast<int>(fl);
  A = static_cast<int>(floorf(__fadd_rn(__fmul_rn(__fsub_rn(xb, fl), 256.0f), 0.5f)));
}

// x / 256 rounded to the nearest integer, ties to even.
__device__ __forceinline__ uint32_t div256Even(uint32_t x) {
  const uint32_t q = x >> 8, r = x & 255u;
  return q + ((r > 128u || (r == 128u && (q & 1u))) ? 1u : 0u);
}

// Bilinear lookup in integer arithmetic: the four corner weights are the
// products of the per-axis weights rounded to 1/256, the result
// sum(w * texel) / (256 * 255) rounded once to float.
__device__ __forceinline__ float4 sampleTexture(const uint32_t* __restrict__ tx, int4 t, float u, float v) {
  int i, j, A, B;
  texAxis(u, t.y, i, A);
  texAxis(v, t.z, j, B);
  const int i0 = wrapIndex(i, t.y), i1 = wrapIndex(i + 1, t.y);
  const int j0 = wrapIndex(j, t.z), j1 = wrapIndex(j + 1, t.z);
  const uint32_t* row0 = tx + static_cast<uint32_t>(t.x) + static_cast<uint32_t>(j0) * static_cast<uint32_t>(t.y);
  const uint32_t* row1 = tx + static_cast<uint32_t>(t.x) + static_cast<uint32_t>(j1) * static_cast<uint32_t>(t.y);
  const uint32_t T00 = __ldg(row0 + i0), T10 = __ldg(row0 + i1), T01 = __ldg(row1 + i0), T11 = __ldg(row1 + i1);
  const uint32_t a = static_cast<uint32_t>(A), b = static_cast<uint32_t>(B);
  const uint32_t w00 = div256Even((256u - a) * (256u - b)), w10 = div256Even(a * (256u - b));
  const uint32_t w01 = div256Even((256u - a) * b), w11 = div256Even(a * b);
  float r[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t s = 8u * k;
    const uint32_t acc = w00 * ((T00 >> s) & 255u) + w10 * ((T10 >> s) & 255u) + w01 * ((T01 >> s) & 255u) +
                         w11 * ((T11 >> s) & 255u);
    r[k] = __fdiv_rn(static_cast<float>(acc), 65280.0f);
  }
  return make_float4(r[0], r[1], r[2], r[3]);
}

// Barycentric interpolation of one texture coordinate, (1-b1-b2) p0 + b1 p1
// + b2 p2 evaluated left to right with rounded operations.
__device__ __forceinline__ float lerpUv(float w0, float b1, float b2, float p0, float p1, float p2) {
  return __fadd_rn(__fadd_rn(__fmul_rn(w0, p0), __fmul_rn(b1, p1)), __fmul_rn(b2, p2));
}

__device__ __forceinline__ v3 shadeHit(const DevScene& sc, uint32_t pos, float b1, float b2) {
  const float4* s = sc.shade + 3 * pos;
  const float4 c0 = __ldg(s);
  if (c0.w == 0.0f) return mk(c0.x, c0.y, c0.z);  // material base colour
  const float4 c1 = __ldg(s + 1);
  const float4 c2 = __ldg(s + 2);
  const float w0 = 1.0f - b1 - b2;
  if (c0.w == 2.0f) {  // base colour texture at the interpolated (u, v)
    const float u = lerpUv(w0, b1, b2, c0.x, c1.x, c2.x);
    const float v = lerpUv(w0, b1, b2, c0.y, c1.y, c2.y);
    const float4 T = sampleTexture(sc.texels, __ldg(sc.texTable + static_cast<int>(c0.z)), u, v);
    return linearize(mk(T.x, T.y, T.z));
  }
  const v3 C = mk(w0 * c0.x + b1 * c1.x + b2 * c2.x, w0 * c0.y + b1 * c1.y + b2 * c2.y, w0 * c0.z + b1 * c1.z + b2 * c2.z);
  return linearize(C);
}

#define CR_PI_F 3.14159265358979323846f

// ---------------------------------------------------------------------------
// Lighting-on closest hit (shaders.cu:812-880): GGX/Smith shading of four
// point lights with shadow rays, from the base colour above.
// ---------------------------------------------------------------------------
__device__ __forceinline__ v3 vmul(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }

// shaders.cu:67-90
__device__ __forceinline__ v3 schlick(v3 spec, float VdH) {
  const float f = powf(1.0f - VdH, 5.0f);
  return spec + vmul(mk(1.0f, 1.0f, 1.0f) - spec, mk(f, f, f));
}
__device__ __forceinline__ float smithVis(float NdL, float NdV, float alpha) {
  const float a2 = alpha * alpha;
  const float ggx0 = NdL * sqrtf(NdV * NdV * (1.0f - a2) + a2);
  const float ggx1 = NdV * sqrtf(NdL * NdL * (1.0f - a2) + a2);
  return 2.0f * NdL * NdV / (ggx0 + ggx1);
}
__device__ __forceinline__ float ggxNormal(float NdH, float alpha) {
  const float a2 = alpha * alpha;
  const float x = NdH * NdH * (a2 - 1.0f) + 1.0f;
  return a2 / (CR_PI_F * x * x);
}

// Occlusion query (shaders.cu:140-163): any triangle in [tmin, tmax].
__device__ __forceinline__ bool occluded(const DevScene& sc, v3 o, v3 d, float tmin, float tmax, uint32_t* errFlag) {
  const Ray r = setupRay(o, d, sc.extent);
  Hit h;
  h.t = tmax;
  h.id = 0xffffffffu;
  h.pos = 0;
  int stack[kStackSize];
  uint32_t nv = 0, tt = 0;
  traverseFrom<false, true>(sc, r, tmin, h, stack, 0, 0, errFlag, nv, tt);
  return h.id != 0xffffffffu;
}

__device__ v3 shadeLit(const DevScene& sc, const Hit& h, float b1, float b2, v3 dir, v3 base, uint32_t* errFlag) {
  const float4* L = sc.light + 5 * static_cast<size_t>(h.id);
  const float4 l0 = __ldg(L), l1 = __ldg(L + 1), l2 = __ldg(L + 2), l3 = __ldg(L + 3), l4 = __ldg(L + 4);
  const float4* t = sc.tris + 3 * h.pos;
  const float4 q0 = __ldg(t), q1 = __ldg(t + 1), q2 = __ldg(t + 2);
  const v3 P0 = mk(q0.x, q0.y, q0.z), P1 = mk(q1.x, q1.y, q1.z), P2 = mk(q2.x, q2.y, q2.z);
  const float w0 = 1.0f - b1 - b2;
  const v3 P = P0 * w0 + P1 * b1 + P2 * b2;
  const int flags = static_cast<int>(l4.w);
  const v3 Ng = normalize(cross(P1 - P0, P2 - P0));
  v3 N = Ng;
  if (flags & 1) N = normalize(mk(l0.x, l0.y, l0.z) * w0 + mk(l0.w, l1.x, l1.y) * b1 + mk(l1.z, l1.w, l2.x) * b2);
  const float u0 = l2.y, v0 = l2.z, u1 = l2.w, v1 = l3.x, u2 = l3.y, v2 = l3.z;
  float U = b1, Vt = b2;  // without TEXCOORD_0 the coordinates are the barycentrics (LocalGeometry.h:99-102)
  if (flags & 2) {
    U = w0 * u0 + b1 * u1 + b2 * u2;
    Vt = w0 * v0 + b1 * v1 + b2 * v2;
  }
  float metallic = l3.w, roughness = l4.x;
  const int mrTex = static_cast<int>(l4.y), nTex = static_cast<int>(l4.z);
  if (mrTex >= 0) {  // (occlusion, roughness, metallic)
    const float4 mr = sampleTexture(sc.texels, __ldg(sc.texTable + mrTex), U, Vt);
    roughness *= mr.y;
    metallic *= mr.z;
  }
  const float F0 = 0.04f;
  const v3 diff = base * ((1.0f - F0) * (1.0f - metallic));
  const v3 spec = mk(F0, F0, F0) + (base - mk(F0, F0, F0)) * metallic;
  const float alpha = roughness * roughness;
  if (nTex >= 0) {
    const float4 T = sampleTexture(sc.texels, __ldg(sc.texTable + nTex), U, Vt);
    const float du1 = u0 - u2, du2 = u1 - u2, dv1 = v0 - v2, dv2 = v1 - v2;
    const v3 dp1 = P0 - P2, dp2 = P1 - P2;
    const float invdet = 1.f / (du1 * dv2 - dv1 * du2);
    const v3 dpdu = (dp1 * dv2 - dp2 * dv1) * invdet;
    const v3 dpdv = (dp1 * -du2 + dp2 * du1) * invdet;
    N = normalize(normalize(dpdu) * (2.0f * T.x - 1.0f) + normalize(dpdv) * (2.0f * T.y - 1.0f) + N * (2.0f * T.z - 1.0f));
  }
  const v3 V = normalize(dir) * -1.0f;
  v3 result = mk(0.f, 0.f, 0.f);
  for (int i = 0; i < 4; ++i) {
    const float4 lp = sc.lightPos[i], lc = sc.lightCol[i];
    const v3 Lv = mk(lp.x, lp.y, lp.z) - P;
    const float Ldist = sqrtf(dot(Lv, Lv));
    const v3 Ld = Lv * (1.0f / Ldist);
    const v3 H = normalize(Ld + V);
    const float NdL = dot(N, Ld), NdV = dot(N, V), NdH = dot(N, H), VdH = dot(V, H);
    if (NdL > 0.0f && NdV > 0.0f && !occluded(sc, P, Ld, 0.001f, Ldist - 0.001f, errFlag)) {
      const v3 F = schlick(spec, VdH);
      const float G = smithVis(NdL, NdV, alpha);
      const float D = ggxNormal(NdH, alpha);
      const v3 d = vmul(mk(1.0f, 1.0f, 1.0f) - F, diff) * (1.0f / CR_PI_F);
      const v3 s = F * (G * D);
      result = result + vmul(mk(lc.x, lc.y, lc.z) * (lp.w * NdL), d + s);
    }
  }
  return result;
}

__device__ __forceinline__ v3 shadeMiss(int miss, v3 dirIn) {
  const v3 dir = normalize(dirIn);
  if (miss == 1) {
    const float mix = fminf(fmaxf(0.0f, (asinf(dir.y) * 2.0f) / CR_PI_F), 1.0f);
    const v3 upper = mk(1.0f / 255.0f, 31.0f / 255.0f, 117.0f / 255.0f);
    const v3 lower = mk(143.0f / 255.0f * 0.8f, 179.0f / 255.0f * 0.8f, 203.0f / 255.0f * 0.8f);
    return lower * (1.0f - mix) + upper * mix;
  }
  v3 c = mk((atan2f(dir.z, dir.x) + CR_PI_F) / (CR_PI_F * 2.0f), (asinf(dir.y) + CR_PI_F / 2.0f) / CR_PI_F, 0.0f);
  const float border = 0.01f;
  if (fabsf(dir.x) < border || fabsf(dir.y) < border || fabsf(dir.z) < border) c = mk(0.f, 0.f, 0.f);
  return c;
}

// ---------------------------------------------------------------------------
// Generator state transfer (structure of arrays, see DevEye).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void loadState(const uint32_t* rng, size_t plane, size_t idx, curandState& st) {
  st.d = rng[idx];
  st.v[0] = rng[plane + idx];
  st.v[1] = rng[2 * plane + idx];
  st.v[2] = rng[3 * plane + idx];
  st.v[3] = rng[4 * plane + idx];
  st.v[4] = rng[5 * plane + idx];
  st.boxmuller_flag = static_cast<int>(rng[6 * plane + idx]);
  st.boxmuller_flag_double = 0;
  st.boxmuller_extra = __uint_as_float(rng[7 * plane + idx]);
  st.boxmuller_extra_double = 0.0;
}
__device__ __forceinline__ void storeState(uint32_t* rng, size_t plane, size_t idx, const curandState& st) {
  rng[idx] = st.d;
  rng[plane + idx] = st.v[0];
  rng[2 * plane + idx] = st.v[1];
  rng[3 * plane + idx] = st.v[2];
  rng[4 * plane + idx] = st.v[3];
  rng[5 * plane + idx] = st.v[4];
  rng[6 * plane + idx] = static_cast<uint32_t>(st.boxmuller_flag);
  rng[7 * plane + idx] = __float_as_uint(st.boxmuller_extra);
}

__global__ void rngInitKernel(DevEye eye, uint32_t* errFlag) {
  const size_t total = static_cast<size_t>(eye.N) * eye.spp;
  const size_t idx = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const uint32_t o = static_cast<uint32_t>(idx / eye.spp);
  const uint32_t s = static_cast<uint32_t>(idx % eye.spp);
  // Same stream as the reference's id = launch_dims.x * launch_idx.y + launch_idx.x.
  const int id = static_cast<int>(eye.N * s + o);
  curandState st;
  curand_init(42, id, 0, &st);
  if (st.boxmuller_flag_double != 0) atomicOr(errFlag, kErrRngDoubleFlag);
  storeState(eye.rng, total, idx, st);
}

// The random numbers of P consecutive frames for every (ommatidium, sample)
// stream, in the order the render kernel would draw them (one normal, then
// one uniform per frame), into draws[(p * N + o) * spp + s]; the states
// advance by P frames, exactly as a render of the P poses would leave them.
__global__ void drawsKernel(DevEye eye, uint32_t P) {
  const size_t total = static_cast<size_t>(eye.N) * eye.spp;
  const size_t idx = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  curandState st;
  loadState(eye.rng, total, idx, st);
  for (uint32_t p = 0; p < P; ++p) {
    const float nd = curand_normal(&st);
    const float ud = curand_uniform(&st);
    eye.draws[static_cast<size_t>(p) * total + idx] = make_float2(nd, ud);
  }
  storeState(eye.rng, total, idx, st);
}

// SplitMix64's output function (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014): a bijective 64-bit mix.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Draws of sample k of an entry (the adaptive render's (pose, ommatidium)
// entries; a feature render's (frame, ommatidium)): point k of the
// two-dimensional Sobol' sequence (dimension 1 the van der Corput sequence in
// base 2, i.e. k bit-reversed; dimension 2 the generator matrix whose
// columns start at 2^31 and follow v <- v ^ (v >> 1)) with a random digital
// shift per entry (both coordinates XORed with mix64 of the seed and the
// entry).  The first 2^m points of this (0, 2)-sequence form a (0, m, 2)-net,
// and a digital shift keeps that, so an entry's 2^m samples are stratified
// in every elementary interval of area 2^-m and each is still uniform, so
// the estimate stays unbiased.  Coordinate 1 -> the normal draw through the
// inverse normal distribution at the midpoint of its 2^-23 cell (23 bits,
// so that the midpoint is exact in float: with 24 the top cell's midpoint
// rounds to 1 and its draw to infinity), coordinate 2 -> the uniform draw in
// (0, 1].
__device__ __forceinline__ float2 netDraw(unsigned long long seed, unsigned long long entry, uint32_t k) {
  const unsigned long long h = mix64(seed + (entry + 1ull) * 0x9E3779B97F4A7C15ull);
  uint32_t x2 = 0u;
  for (uint32_t v = 0x80000000u, b = k; b != 0u; b >>= 1, v ^= v >> 1)
    if (b & 1u) x2 ^= v;
  const uint32_t x1 = __brev(k) ^ static_cast<uint32_t>(h);
  x2 ^= static_cast<uint32_t>(h >> 32);
  float2 d;
  d.x = normcdfinvf((static_cast<float>(x1 >> 9) + 0.5f) * (1.0f / 8388608.0f));
  d.y = 1.0f - static_cast<float>(x2 >> 8) * (1.0f / 16777216.0f);
  return d;
}

__constant__ float FWHM_SD_RATIO = 2.35482004503094938202313865291f;

// In-block chunk sums keep the partials of kInBlockPoses poses at a time in
// shared memory: [ommatidium slot of the block][pose of the group][chunk][3].
constexpr uint32_t kInBlockPoses = 16;

// Sums the block's chunk partials of poses pg0 .. pg0 + count - 1 in chunk
// order into out (P x N x 3), between two barriers: every warp of the block
// has written its partials of these poses before, and none overwrites them
// before the sums are read.  Called by every thread of the block.
__device__ __forceinline__ void flushChunkSums(const float* __restrict__ part, const WarpPlan& plan,
                                               const DevEye& eye, float* __restrict__ out, uint32_t pg0,
                                               uint32_t count) {
  __syncthreads();
  const uint32_t perBlock = plan.groupsPerBlock * plan.ommPerWarp;  // ommatidium slots of the block
  for (uint32_t item = threadIdx.x; item < perBlock * count; item += blockDim.x) {
    const uint32_t gs = item / count, pp = item - gs * count;
    const uint64_t slot = static_cast<uint64_t>(blockIdx.x) * perBlock + gs;
    if (slot >= eye.N) continue;
    const uint32_t o = eye.order ? __ldg(eye.order + slot) : static_cast<uint32_t>(slot);
    const float* src = part + (static_cast<size_t>(gs) * kInBlockPoses + pp) * plan.chunks * 3;
    float x = 0.f, y = 0.f, z = 0.f;
    for (uint32_t c = 0; c < plan.chunks; ++c) {
      x += src[3 * c];
      y += src[3 * c + 1];
      z += src[3 * c + 2];
    }
    float* dst = out + (static_cast<size_t>(pg0 + pp) * eye.N + o) * 3;
    dst[0] = x;
    dst[1] = y;
    dst[2] = z;
  }
  __syncthreads();
}

// kMode: 0 = render, 1 = render and record every ray, 2 = render and count
// node visits / triangle tests into stats[0..1].  kMinBlocks: resident
// 128-thread blocks per SM the register allocation is sized for (the
// autotuner's occupancy knob).
// One warp task: up to 32 samples of one ommatidium (or whole ommatidia when
// spp < 32) for all P poses.  Called by whole warps.
// part: null, or (plan.inBlock) the block's shared-memory chunk partials,
// [group in block][ommatidium in warp][pose of the group][chunk][3] floats
// for kInBlockPoses poses at a time; with it every thread of the block
// calls this function with the same poses (flushChunkSums has barriers).
// kWidth: 2 searches the BVH2 (with the near-field cut when eye.cuts is
// set), 4 or 8 the wide BVH of that width (no cut).
template <int kMode, int kWidth = 2>
__device__ __forceinline__ void renderTask(const DevScene& sc, const DevEye& eye, const float4* __restrict__ poses,
                                           uint32_t P, const WarpPlan& plan, uint64_t task, float* __restrict__ out,
                                           float* __restrict__ scratch, uint32_t* errFlag,
                                           RayRecord* __restrict__ rec, uint32_t& nodeVisits, uint32_t& triTests,
                                           float* __restrict__ part = nullptr) {
  constexpr bool kRecord = (kMode & 3) == 1;
  constexpr bool kFeat = (kMode & 3) == 3;
  constexpr bool kCount = (kMode & 3) == 2 || kFeat;  // feature mode: the per-entry traversal cost
  constexpr bool kLit = (kMode & 4) != 0;  // lighting-on shading (modes 4 render, 5 record)
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t p0 = 0, p1 = P;
  if (plan.poseSplits > 1) {
    const uint64_t perSplit = plan.tasks / plan.poseSplits;
    const uint32_t split = static_cast<uint32_t>(task / perSplit);
    task %= perSplit;
    p0 = split * plan.posesPerSplit;
    p1 = min(P, p0 + plan.posesPerSplit);
  }
  const uint32_t group = static_cast<uint32_t>(task / plan.chunks);
  const uint32_t chunk = static_cast<uint32_t>(task % plan.chunks);
  const uint32_t slot = group * plan.ommPerWarp + lane / plan.segWidth;
  const uint32_t o = (eye.order && slot < eye.N) ? __ldg(eye.order + slot) : slot;
  const uint32_t s = chunk * plan.segWidth + lane % plan.segWidth;
  const bool valid = slot < eye.N && s < eye.spp;
  const size_t plane = static_cast<size_t>(eye.N) * eye.spp;
  const size_t sidx = static_cast<size_t>(o) * eye.spp + s;
  // Where a segment leader writes pose p's sum (or chunk partial): dst0 + p *
  // dstStride, one of the output, the scratch partials or the block's shared
  // partials (render and record modes).
  float* dst0;
  size_t dstStride;
  if (plan.chunks == 1) {
    dst0 = out + static_cast<size_t>(o) * 3;
    dstStride = static_cast<size_t>(eye.N) * 3;
  } else if (part) {  // pose p's partial at (p - p0) % kInBlockPoses of the group
    const uint32_t gs = (group % plan.groupsPerBlock) * plan.ommPerWarp + lane / plan.segWidth;
    dst0 = part + (static_cast<size_t>(gs) * kInBlockPoses * plan.chunks + chunk) * 3;
    dstStride = static_cast<size_t>(plan.chunks) * 3;
  } else {
    dst0 = scratch + (static_cast<size_t>(o) * plan.chunks + chunk) * 3;
    dstStride = static_cast<size_t>(eye.N) * plan.chunks * 3;
  }

  curandState st;
  v3 axis = mk(0.f, 1.f, 0.f), relPos = mk(0.f, 0.f, 0.f), perp = mk(0.f, 0.f, 1.f);
  float sd = 0.f, fpo = 0.f;
  if (valid) {
    if (!kFeat && !eye.draws) loadState(eye.rng, plane, sidx, st);
    const float4 a = __ldg(eye.omm + 2 * o);
    const float4 b = __ldg(eye.omm + 2 * o + 1);
    axis = mk(a.w, b.x, b.y);
    const v3 pos = mk(a.x, a.y, a.z);
    fpo = b.w;
    sd = b.z / FWHM_SD_RATIO;
    // generateOffsetRay's perpendicular axis (shaders.cu:655-657), including
    // its test on the component sum.
    perp = cross(mk(0.0f, 1.0f, 0.0f), axis);
    perp = (perp.x + perp.y + perp.z == 0.0f) ? mk(0.0f, 0.0f, 1.0f) : normalize(perp);
    relPos = pos - normalize(axis) * fpo;
  }
  const float invSpp = 1.0f / static_cast<float>(eye.spp);

  for (uint32_t p = p0; p < p1; ++p) {
    v3 col = mk(0.f, 0.f, 0.f);
    // Feature mode: per-sample squared colour, hit flag, hit distance and the
    // hit triangle's normal in the eye's frame (facing the ray), all / spp.
    float f2x = 0.f, f2y = 0.f, f2z = 0.f, fHit = 0.f, fT = 0.f, fnx = 0.f, fny = 0.f, fnz = 0.f, fCost = 0.f;
    const uint32_t steps0 = nodeVisits + triTests;
    if (valid) {
      const float4* pp = poses + 4 * p;
      const float4 P0 = __ldg(pp), X = __ldg(pp + 1), Y = __ldg(pp + 2), Z = __ldg(pp + 3);
      float nd, ud;
      if (kFeat) {  // feature renders: each ommatidium's samples a net (launchFeatures requires eye.netDraws)
        const float2 dr = netDraw(eye.drawSeed, (eye.frame0 + p) * eye.N + o, s);
        nd = dr.x;
        ud = dr.y;
      } else if (eye.draws) {
        const float2 dr = eye.draws[(static_cast<size_t>(p) * eye.N + o) * eye.spp + s];
        nd = dr.x;
        ud = dr.y;
      } else {
        nd = curand_normal(&st);
        ud = curand_uniform(&st);
      }
      const float splayAngle = nd * sd;
      const float axisAngle = ud * CR_PI_F;
      const v3 splayed = rotatePoint(axis, splayAngle, perp);
      const v3 rel = rotatePoint(splayed, axisAngle, axis);
      const v3 org = mk(P0.x, P0.y, P0.z) + mk(X.x, X.y, X.z) * relPos.x + mk(Y.x, Y.y, Y.z) * relPos.y +
                     mk(Z.x, Z.y, Z.z) * relPos.z;
      const v3 dir = mk(X.x, X.y, X.z) * rel.x + mk(Y.x, Y.y, Y.z) * rel.y + mk(Z.x, Z.y, Z.z) * rel.z;
      const Ray ray = setupRay(org, dir, sc.extent);
      Hit h;
      if (kWidth != 2) {
        h.t = 1e16f;
        h.id = 0xffffffffu;
        h.pos = 0;
        if (sc.triCount > 0) {
          int wstack[kWideStackSize];
          int wsp = 0, wnode = 0;
          traverseWide<kWidth == 8 ? 8 : 4>(sc, ray, fpo, h, wstack, wsp, wnode, errFlag, nodeVisits, triTests, kCount,
                                             0x7fffffff);
        }
      } else if (eye.cuts) {
        traceClosest<kCount>(sc, ray, fpo, 1e16f, h, errFlag, nodeVisits, triTests,
                             eye.cuts + static_cast<size_t>(p) * kCutStride, sqrtf(dot(dir, dir)));
      } else {
        traceClosest<kCount>(sc, ray, fpo, 1e16f, h, errFlag, nodeVisits, triTests);
      }
      v3 c;
      float b1 = 0.f, b2 = 0.f;
      if (h.id != 0xffffffffu) {
        b1 = xdiv(h.V, h.det);
        b2 = xdiv(h.W, h.det);
        c = shadeHit(sc, h.pos, b1, b2);
        if (kLit) c = shadeLit(sc, h, b1, b2, dir, c, errFlag);
      } else {
        c = shadeMiss(sc.miss, dir);
      }
      if (kRecord) {
        RayRecord& R = rec[(static_cast<size_t>(p) * eye.N + o) * eye.spp + s];
        R.normalDraw = nd;
        R.uniformDraw = ud;
        R.ox = org.x;
        R.oy = org.y;
        R.oz = org.z;
        R.dx = dir.x;
        R.dy = dir.y;
        R.dz = dir.z;
        R.t = h.id != 0xffffffffu ? h.t : -1.0f;
        R.b1 = b1;
        R.b2 = b2;
        R.hitId = h.id != 0xffffffffu ? static_cast<int32_t>(h.id) : -1;
        R.r = c.x;
        R.g = c.y;
        R.b = c.z;
        R.pad = 0.f;
      }
      col = c * invSpp;
      if (kFeat) {
        fCost = static_cast<float>(nodeVisits + triTests - steps0) * invSpp;
        f2x = c.x * c.x * invSpp;
        f2y = c.y * c.y * invSpp;
        f2z = c.z * c.z * invSpp;
        if (h.id != 0xffffffffu) {
          fHit = invSpp;
          fT = h.t * invSpp;
          const float4* t = sc.tris + 3 * h.pos;
          const float4 a = __ldg(t), b = __ldg(t + 1), cc = __ldg(t + 2);
          v3 n = normalize(cross(mk(b.x - a.x, b.y - a.y, b.z - a.z), mk(cc.x - a.x, cc.y - a.y, cc.z - a.z)));
          if (dot(n, dir) > 0.f) n = n * -1.0f;
          fnx = dot(n, mk(X.x, X.y, X.z)) * invSpp;
          fny = dot(n, mk(Y.x, Y.y, Y.z)) * invSpp;
          fnz = dot(n, mk(Z.x, Z.y, Z.z)) * invSpp;
        }
      }
    }
    // Segmented butterfly reduction over the samples of each ommatidium.
    for (uint32_t m = plan.segWidth >> 1; m >= 1u; m >>= 1) {
      col.x += __shfl_xor_sync(0xffffffffu, col.x, static_cast<int>(m));
      col.y += __shfl_xor_sync(0xffffffffu, col.y, static_cast<int>(m));
      col.z += __shfl_xor_sync(0xffffffffu, col.z, static_cast<int>(m));
      if (kFeat) {
        f2x += __shfl_xor_sync(0xffffffffu, f2x, static_cast<int>(m));
        f2y += __shfl_xor_sync(0xffffffffu, f2y, static_cast<int>(m));
        f2z += __shfl_xor_sync(0xffffffffu, f2z, static_cast<int>(m));
        fHit += __shfl_xor_sync(0xffffffffu, fHit, static_cast<int>(m));
        fT += __shfl_xor_sync(0xffffffffu, fT, static_cast<int>(m));
        fnx += __shfl_xor_sync(0xffffffffu, fnx, static_cast<int>(m));
        fny += __shfl_xor_sync(0xffffffffu, fny, static_cast<int>(m));
        fnz += __shfl_xor_sync(0xffffffffu, fnz, static_cast<int>(m));
        fCost += __shfl_xor_sync(0xffffffffu, fCost, static_cast<int>(m));
      }
    }
    if (kFeat) {
      if ((lane % plan.segWidth) == 0u && o < eye.N) {
        float* dst = out + (static_cast<size_t>(p) * eye.N + o) * kFeatureStats;
        dst[0] = col.x;
        dst[1] = col.y;
        dst[2] = col.z;
        dst[3] = f2x;
        dst[4] = f2y;
        dst[5] = f2z;
        dst[6] = fHit;
        dst[7] = fT;
        dst[8] = fnx;
        dst[9] = fny;
        dst[10] = fnz;
        dst[kCostStat] = fCost;
      }
      continue;
    }
    if ((lane % plan.segWidth) == 0u && o < eye.N) {
      float* dst = dst0 + (part ? (p - p0) % kInBlockPoses : p) * dstStride;
      dst[0] = col.x;
      dst[1] = col.y;
      dst[2] = col.z;
    }
    // In-block sums: after each group of kInBlockPoses poses (and the last),
    // the block sums the group's partials (every warp of the block runs the
    // same poses, so all of them reach these barriers).
    if (part && ((p - p0 + 1) % kInBlockPoses == 0 || p + 1 == p1)) {
      const uint32_t pg0 = p0 + (p - p0) / kInBlockPoses * kInBlockPoses;
      flushChunkSums(part, plan, eye, out, pg0, p + 1 - pg0);
    }
  }
  if (!kFeat && valid && !eye.draws) storeState(eye.rng, plane, sidx, st);
}

// kRegs: registers per thread the kernel is compiled for (the autotuner's
// occupancy knob: 96, 80 or 64 allow 640, 768 or 1024 resident threads per
// SM), independent of the block size, which the plan sets (128-512 threads).
// With plan.inBlock every block holds all chunk warps of plan.groupsPerBlock
// ommatidium groups (tasks padded to whole blocks): each warp leaves its
// per-pose chunk partial in shared memory, and after every kInBlockPoses
// poses the block sums each (ommatidium, pose) of the group over its chunks
// in chunk order (flushChunkSums), so the buffer holds 16 poses at a time.
template <int kMode, int kRegs, int kWidth = 2, bool kInBlock = false>
__global__ void __maxnreg__(kRegs) renderKernel(DevScene sc, DevEye eye, const float4* __restrict__ poses, uint32_t P,
                                                WarpPlan plan, float* __restrict__ out, float* __restrict__ scratch,
                                                uint32_t* errFlag, RayRecord* __restrict__ rec,
                                                unsigned long long* stats) {
  extern __shared__ float chunkPart[];
  constexpr bool kCount = kMode == 2;
  uint32_t nodeVisits = 0, triTests = 0;
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t task = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (task >= plan.tasks) return;  // whole warps exit together (never with inBlock: whole blocks)
  renderTask<kMode, kWidth>(sc, eye, poses, P, plan, task, out, scratch, errFlag, rec, nodeVisits, triTests,
                            kInBlock ? chunkPart : nullptr);
  if (kCount) {
    unsigned long long nv = nodeVisits, tt = triTests;
    for (int m = 16; m >= 1; m >>= 1) {
      nv += __shfl_xor_sync(0xffffffffu, nv, m);
      tt += __shfl_xor_sync(0xffffffffu, tt, m);
    }
    if (lane == 0) {
      atomicAdd(stats, nv);
      atomicAdd(stats + 1, tt);
    }
  }
}

// Sums the per-chunk partials of each (pose, ommatidium) in chunk order.
__global__ void combineChunksKernel(const float* __restrict__ scratch, uint32_t chunks, size_t count,
                                    float* __restrict__ out) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float* src = scratch + i * chunks * 3;
  float x = 0.f, y = 0.f, z = 0.f;
  for (uint32_t c = 0; c < chunks; ++c) {
    x += src[3 * c];
    y += src[3 * c + 1];
    z += src[3 * c + 2];
  }
  out[3 * i] = x;
  out[3 * i + 1] = y;
  out[3 * i + 2] = z;
}

__device__ __forceinline__ uchar4 makeColour(float r, float g, float b) {
  // make_color (shaders.cu:180-189): clamp, gamma 1/2.2 (a double constant
  // narrowed to float), scale to 255 and truncate.
  const float invGamma = static_cast<float>(1.0 / static_cast<double>(2.2f));
  return make_uchar4(static_cast<uint8_t>(powf(fminf(fmaxf(r, 0.0f), 1.0f), invGamma) * 255.0f),
                     static_cast<uint8_t>(powf(fminf(fmaxf(g, 0.0f), 1.0f), invGamma) * 255.0f),
                     static_cast<uint8_t>(powf(fminf(fmaxf(b, 0.0f), 1.0f), invGamma) * 255.0f), 255u);
}

__global__ void projectKernel(const float* __restrict__ sums, uint32_t N, uchar4* frame, int w, int h, int mode) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= w || y >= h) return;
  if (mode == 0) {
    // single_dimension_fast (shaders.cu:396-406): only row 0, x < N.
    if (y > 0 || static_cast<uint32_t>(x) >= N) return;
    frame[x] = makeColour(sums[3 * x], sums[3 * x + 1], sums[3 * x + 2]);
    return;
  }
  // single_dimension (shaders.cu:375-390): every pixel, ommatidium x*N/w.
  if (N == 0) return;
  const uint32_t o = static_cast<uint32_t>((static_cast<uint64_t>(x) * N) / static_cast<uint64_t>(w));
  frame[static_cast<size_t>(y) * w + x] = makeColour(sums[3 * o], sums[3 * o + 1], sums[3 * o + 2]);
}

// Spherical projections (shaders.cu:412-640): every pixel maps to a point on
// the unit sphere and shows the ommatidium whose position (or direction)
// makes the smallest angle with it, the first such ommatidium on ties.
//  kind 0 positionwise, 1 orientationwise, 2 split orientationwise (the left
//  half of the image considers only ommatidia with position.x < 0, the right
//  half those with x > 0; ommatidium 0 is the starting candidate either way),
//  3 orientationwise ids, 4 positionwise ids (index in RGBA, base 256).
// The candidate lengths are precomputed per ommatidium (len), identical to
// recomputing them per pixel.

// Point on the sphere of pixel (x, y) and its horizontal image coordinate.
__device__ __forceinline__ v3 sphericalPixel(int x, int y, int w, int h, int kind, float& ux) {
  ux = static_cast<float>(x) / static_cast<float>(w);
  const float uy = static_cast<float>(y) / static_cast<float>(h);
  float dx, dy;
  if (kind == 2) {
    const float sx = ux * 2.0f;
    const float sub = sx > 1.0f ? 1.0f : 0.f;
    dx = (sx - sub) * 2.0f - 1.0f;
    dy = uy * 2.0f - 1.0f;
  } else {
    dx = 2.0f * ux - 1.0f;
    dy = 2.0f * uy - 1.0f;
  }
  const float ax = dx * -CR_PI_F + CR_PI_F / 2.0f, ay = dy * (CR_PI_F / 2.0f);
  const float cosY = cosf(ay);
  return mk(cosf(ax) * cosY, sinf(ay), sinf(ax) * cosY);
}

// The compared quantity: angle between candidate i's vector and the pixel's
// point, as the reference computes it.
__device__ __forceinline__ float sphericalAngle(const float4* __restrict__ omm, const float* __restrict__ len,
                                                uint32_t N, bool byPos, uint32_t i, v3 p, float lp) {
  const float4 a = __ldg(omm + 2 * i), b = __ldg(omm + 2 * i + 1);
  const v3 v = byPos ? mk(a.x, a.y, a.z) : mk(a.w, b.x, b.y);
  return acosf(dot(v, p) / (__ldg(len + (byPos ? i : N + i)) * lp));
}

__device__ __forceinline__ void sphericalWrite(uint32_t bi, int kind, const float* __restrict__ sums, uchar4* frame,
                                               size_t px) {
  uchar4 c;
  if (kind >= 3) c = make_uchar4(static_cast<uint8_t>(bi >> 24), static_cast<uint8_t>((bi >> 16) & 0xff),
                                 static_cast<uint8_t>((bi >> 8) & 0xff), static_cast<uint8_t>(bi & 0xff));
  else c = makeColour(sums[3 * bi], sums[3 * bi + 1], sums[3 * bi + 2]);
  frame[px] = c;
}

// Exhaustive form: every candidate in index order, as the reference does.
__global__ void sphericalKernel(const float4* __restrict__ omm, const float* __restrict__ len, uint32_t N,
                                const float* __restrict__ sums, uchar4* frame, int w, int h, int kind) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= w || y >= h || N == 0) return;
  float ux;
  const v3 p = sphericalPixel(x, y, w, h, kind, ux);
  const float lp = sqrtf(dot(p, p));
  const bool byPos = (kind == 0 || kind == 4);
  float best = sphericalAngle(omm, len, N, byPos, 0, p, lp);
  uint32_t bi = 0;
  for (uint32_t i = 1; i < N; ++i) {
    const float ang = sphericalAngle(omm, len, N, byPos, i, p, lp);
    bool ok = ang < best;
    if (kind == 2) {
      const float px = __ldg(omm + 2 * i).x;
      ok = ok && ((px > 0.f && ux > 0.5f) || (px < 0.f && ux < 0.5f));
    }
    if (ok) {
      best = ang;
      bi = i;
    }
  }
  sphericalWrite(bi, kind, sums, frame, static_cast<size_t>(y) * w + x);
}

// Grid form, same result.  The candidates i >= 1 of the pixel's set are
// binned by their unit vector into a G^3 grid over [-1, 1]^3 (SphereGrid).
// Candidate 0 starts, as in the exhaustive form; cells are searched in boxes
// around the pixel's unit point q that grow (one cell, then doubling radii)
// until the box holds every point within chord distance
// 2 sin((best + margin) / 2) of q.  Candidates compare by (angle, index), so
// the smallest index wins among equal angles.  margin (0.01 rad) bounds twice
// the difference between a computed angle and the true one, so every
// candidate left outside the box has a computed angle above the best.
// A NaN angle never wins; a NaN angle of candidate 0 makes 0 the answer.
__global__ void sphericalGridKernel(const float4* __restrict__ omm, const float* __restrict__ len, uint32_t N,
                                    SphereGridSet grids, const float* __restrict__ sums, uchar4* frame, int w, int h,
                                    int kind) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= w || y >= h || N == 0) return;
  float ux;
  const v3 p = sphericalPixel(x, y, w, h, kind, ux);
  const float lp = sqrtf(dot(p, p));
  const bool byPos = (kind == 0 || kind == 4);
  float best = sphericalAngle(omm, len, N, byPos, 0, p, lp);
  uint32_t bi = 0;
  const SphereGridView* g = nullptr;
  if (kind == 2) {
    if (ux < 0.5f) g = &grids.g[2];
    else if (ux > 0.5f) g = &grids.g[3];
  } else {
    g = &grids.g[byPos ? 0 : 1];
  }
  if (best == best && g && g->G > 0) {
    const int G = g->G;
    const float cell = 2.0f / static_cast<float>(G);
    const float inv = 1.0f / lp;
    const float q[3] = {p.x * inv, p.y * inv, p.z * inv};
    auto cellOf = [&](float c) { return min(G - 1, max(0, static_cast<int>(floorf((c + 1.0f) / cell)))); };
    int vlo[3] = {1, 1, 1}, vhi[3] = {0, 0, 0};  // visited box (empty)
    float r = cell;
    for (;;) {
      int lo[3], hi[3];
      for (int a = 0; a < 3; ++a) {
        lo[a] = cellOf(q[a] - r - 1e-5f);
        hi[a] = cellOf(q[a] + r + 1e-5f);
      }
      for (int cz = lo[2]; cz <= hi[2]; ++cz)
        for (int cy = lo[1]; cy <= hi[1]; ++cy)
          for (int cx = lo[0]; cx <= hi[0]; ++cx) {
            if (cx >= vlo[0] && cx <= vhi[0] && cy >= vlo[1] && cy <= vhi[1] && cz >= vlo[2] && cz <= vhi[2]) continue;
            const uint32_t c = (static_cast<uint32_t>(cz) * G + cy) * G + cx;
            const uint32_t e = __ldg(g->start + c + 1);
            for (uint32_t k = __ldg(g->start + c); k < e; ++k) {
              const uint32_t i = __ldg(g->items + k);
              const float ang = sphericalAngle(omm, len, N, byPos, i, p, lp);
              if (ang < best || (ang == best && i < bi)) {
                best = ang;
                bi = i;
              }
            }
          }
      for (int a = 0; a < 3; ++a) {
        vlo[a] = lo[a];
        vhi[a] = hi[a];
      }
      const float reach = best + 0.01f;
      const float need = reach >= CR_PI_F ? 2.0f : 2.0f * sinf(0.5f * reach);
      if (r >= need) break;
      bool whole = true;
      for (int a = 0; a < 3; ++a) whole = whole && lo[a] == 0 && hi[a] == G - 1;
      if (whole) break;
      r = fminf(2.0f * r, need);
    }
  }
  sphericalWrite(bi, kind, sums, frame, static_cast<size_t>(y) * w + x);
}

__global__ void lengthsKernel(const float4* __restrict__ omm, uint32_t N, float* len) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const float4 a = omm[2 * i], b = omm[2 * i + 1];
  const v3 pos = mk(a.x, a.y, a.z), dir = mk(a.w, b.x, b.y);
  len[i] = sqrtf(dot(pos, pos));
  len[N + i] = sqrtf(dot(dir, dir));
}

// raw_ommatidial_samples (shaders.cu:354-369): pixel (x, y) with x < N and
// y < spp shows sample y of ommatidium x, scaled by 1/spp.
__global__ void rawSamplesKernel(const RayRecord* __restrict__ rec, uint32_t N, uint32_t spp, uchar4* frame, int w,
                                 int h) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= w || y >= h) return;
  if (static_cast<uint32_t>(y) >= spp || static_cast<uint32_t>(x) >= N) return;
  const RayRecord& r = rec[static_cast<size_t>(x) * spp + y];
  const float inv = 1.0f / static_cast<float>(spp);
  frame[static_cast<size_t>(y) * w + x] = makeColour(r.r * inv, r.g * inv, r.b * inv);
}

// ---------------------------------------------------------------------------
// Batched rendering of many eyes in one persistent launch.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long globalTimerNs() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Index of the last entry with base <= key in an ascending table.
template <typename T>
__device__ __forceinline__ uint32_t lastAtMost(const T* base, uint32_t n, uint64_t key) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (static_cast<uint64_t>(base[mid]) <= key) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Persistent kernel over the warp tasks of every eye of a batch: each warp
// takes the next task from a global counter until none are left.  Task t
// belongs to the last eye whose taskBase <= t; the eyes' tasks are laid out
// one eye after another.  ctrl[0] = task counter, ctrl[1] = earliest start
// (ns), ctrl[2 + e] = completion time of eye e's last task (ns).
template <int kRegs, int kWidth = 2>
__global__ void __maxnreg__(kRegs) batchKernel(DevScene sc, const BatchEye* __restrict__ eyes,
                                                               const unsigned long long* __restrict__ taskBase,
                                                               uint32_t nEyes, unsigned long long totalTasks,
                                                               unsigned long long* ctrl, uint32_t* errFlag) {
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t nv = 0, tt = 0;
  bool first = true;
  for (;;) {
    unsigned long long task = 0;
    if (lane == 0) task = atomicAdd(&ctrl[0], 1ull);
    task = __shfl_sync(0xffffffffu, task, 0);
    if (task >= totalTasks) break;
    if (first && lane == 0) atomicMin(&ctrl[1], globalTimerNs());
    first = false;
    const uint32_t e = lastAtMost(taskBase, nEyes, task);
    const BatchEye be = eyes[e];
    renderTask<0, kWidth>(sc, be.eye, be.poses, be.P, be.plan, task - taskBase[e], be.out, be.scratch, errFlag, nullptr, nv,
                  tt);
    if (lane == 0) atomicMax(&ctrl[2 + e], globalTimerNs());
  }
}

// Near-field cuts of every eye of a batch: thread i builds the cut of pose
// i % P of eye i / P (each eye has P poses) when that eye has a cut buffer.
__global__ void batchCutKernel(DevScene sc, const BatchEye* __restrict__ eyes, uint32_t nEyes, uint32_t P) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= static_cast<uint64_t>(nEyes) * P) return;
  const uint32_t e = static_cast<uint32_t>(i / P), p = static_cast<uint32_t>(i % P);
  const DevEye& de = eyes[e].eye;
  if (!de.cuts || p >= eyes[e].P) return;
  buildCut(sc, eyes[e].poses + 4 * p, de.cutRadius, de.maxRel, de.cuts + static_cast<size_t>(p) * kCutStride);
}

// Chunk sums of every eye with more than 32 samples: cell c belongs to the
// last eye whose cellBase <= c.
__global__ void batchCombineKernel(const BatchEye* __restrict__ eyes, const unsigned long long* __restrict__ cellBase,
                                   uint32_t nEyes, unsigned long long totalCells) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= totalCells) return;
  const uint32_t e = lastAtMost(cellBase, nEyes, i);
  const BatchEye& be = eyes[e];
  const unsigned long long local = i - cellBase[e];
  const uint32_t chunks = be.plan.chunks;
  const float* src = be.scratch + local * chunks * 3;
  float x = 0.f, y = 0.f, z = 0.f;
  for (uint32_t c = 0; c < chunks; ++c) {
    x += src[3 * c];
    y += src[3 * c + 1];
    z += src[3 * c + 2];
  }
  be.out[3 * local] = x;
  be.out[3 * local + 1] = y;
  be.out[3 * local + 2] = z;
}

// The render kernel's texture filter and the hardware sampler side by side.
__global__ void textureCheckKernel(const uint32_t* __restrict__ tx, int4 t, cudaTextureObject_t obj,
                                   const float2* __restrict__ uv, int n, float4* __restrict__ soft,
                                   float4* __restrict__ hard) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float2 c = uv[k];
  soft[k] = sampleTexture(tx, t, c.x, c.y);
  hard[k] = tex2D<float4>(obj, c.x, c.y);
}

}  // namespace

cudaError_t sampleTextureBoth(const uint32_t* texels, int width, int height, const float* uv, int n, float* rgbaSoft,
                              float* rgbaHard) {
  if (width <= 0 || height <= 0 || n < 0 || !texels || (n > 0 && (!uv || !rgbaSoft || !rgbaHard)))
    return cudaErrorInvalidValue;
  if (n == 0) return cudaSuccess;
  const size_t texBytes = static_cast<size_t>(width) * static_cast<size_t>(height) * 4;
  uint32_t* dTex = nullptr;
  float2* dUv = nullptr;
  float4* dOut = nullptr;
  cudaArray_t arr = nullptr;
  cudaTextureObject_t obj = 0;
  cudaError_t e = cudaMalloc(&dTex, texBytes);
  if (e == cudaSuccess) e = cudaMalloc(&dUv, static_cast<size_t>(n) * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&dOut, static_cast<size_t>(n) * 2 * sizeof(float4));
  if (e == cudaSuccess) e = cudaMemcpy(dTex, texels, texBytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dUv, uv, static_cast<size_t>(n) * sizeof(float2), cudaMemcpyHostToDevice);
  // The reference's texture: a uchar4 array behind a sampler with wrap
  // addressing, linear filtering, normalised-float reads and normalised
  // coordinates (MulticamScene.cpp:753-833).
  const cudaChannelFormatDesc cd = cudaCreateChannelDesc<uchar4>();
  if (e == cudaSuccess) e = cudaMallocArray(&arr, &cd, static_cast<size_t>(width), static_cast<size_t>(height));
  if (e == cudaSuccess)
    e = cudaMemcpy2DToArray(arr, 0, 0, texels, static_cast<size_t>(width) * 4, static_cast<size_t>(width) * 4,
                            static_cast<size_t>(height), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td = {};
    td.addressMode[0] = cudaAddressModeWrap;
    td.addressMode[1] = cudaAddressModeWrap;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeNormalizedFloat;
    td.normalizedCoords = 1;
    td.maxAnisotropy = 1;
    td.maxMipmapLevelClamp = 99;
    td.minMipmapLevelClamp = 0;
    td.mipmapFilterMode = cudaFilterModePoint;
    td.borderColor[0] = 1.0f;
    td.sRGB = 0;
    e = cudaCreateTextureObject(&obj, &rd, &td, nullptr);
  }
  if (e == cudaSuccess) {
    const int4 t = make_int4(0, width, height, 0);
    textureCheckKernel<<<(n + 127) / 128, 128>>>(dTex, t, obj, dUv, n, dOut, dOut + n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(rgbaSoft, dOut, static_cast<size_t>(n) * sizeof(float4), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(rgbaHard, dOut + n, static_cast<size_t>(n) * sizeof(float4), cudaMemcpyDeviceToHost);
  if (obj) cudaDestroyTextureObject(obj);
  if (arr) cudaFreeArray(arr);
  cudaFree(dOut);
  cudaFree(dUv);
  cudaFree(dTex);
  return e;
}

WarpPlan planWarps(uint32_t N, uint32_t spp) {
  WarpPlan p;
  if (spp >= 32) {
    p.segWidth = 32;
    p.ommPerWarp = 1;
    p.chunks = (spp + 31) / 32;
  } else {
    uint32_t w = 1;
    while (w < spp) w <<= 1;
    p.segWidth = w;
    p.ommPerWarp = 32 / w;
    p.chunks = 1;
  }
  const uint64_t groups = (static_cast<uint64_t>(N) + p.ommPerWarp - 1) / p.ommPerWarp;
  p.tasks = groups * p.chunks;
  return p;
}

static uint32_t g_blockThreads = 0, g_samplesPerWarp = 0;

void setRenderLayout(uint32_t blockThreads, uint32_t samplesPerWarp) {
  g_blockThreads = (blockThreads == 128 || blockThreads == 256 || blockThreads == 512) ? blockThreads : 0;
  g_samplesPerWarp = (samplesPerWarp == 8 || samplesPerWarp == 16) ? samplesPerWarp : 0;
}
void renderLayout(uint32_t* blockThreads, uint32_t* samplesPerWarp) {
  *blockThreads = g_blockThreads;
  *samplesPerWarp = g_samplesPerWarp;
}

namespace {
constexpr uint64_t kFillWarps = 16384;  // warps that keep every SM busy (152 SMs x 8 blocks x 4 warps, x3)
constexpr size_t kChunkSmemMax = 96 * 1024;  // shared memory for in-block chunk sums, per block

// The plain render's plan under the process-wide layout: the segment width,
// then the block size, and whether the chunk partials of P poses are summed
// in shared memory (possible when a block holds whole ommatidium groups and
// their partials fit kChunkSmemMax).
WarpPlan planRender(uint32_t N, uint32_t spp, uint32_t P, bool forceScratch, bool inBlockAllowed = true) {
  WarpPlan p = planWarps(N, spp);
  if (g_samplesPerWarp && g_samplesPerWarp < p.segWidth) {
    p.segWidth = g_samplesPerWarp;
    p.ommPerWarp = 32 / p.segWidth;
    p.chunks = (spp + p.segWidth - 1) / p.segWidth;
    p.tasks = (static_cast<uint64_t>(N) + p.ommPerWarp - 1) / p.ommPerWarp * p.chunks;
  }
  uint32_t bw = g_blockThreads / 32;
  if (bw == 0) {
    bw = 4;
    if (p.chunks > 1 && !forceScratch && inBlockAllowed)
      for (uint32_t c : {4u, 8u, 16u})
        if (p.chunks <= c && c % p.chunks == 0) {
          bw = c;
          break;
        }
  }
  p.blockWarps = bw;
  // A small eye's launch may spread its poses over more warps (pre-drawn
  // random numbers, splitPoses): that plan keeps the chunk partials in scratch.
  const bool maySplit = P >= 2 && p.tasks < kFillWarps / 2;
  if (p.chunks > 1 && !forceScratch && inBlockAllowed && !maySplit && bw % p.chunks == 0) {
    const uint32_t G = bw / p.chunks;
    const size_t bytes = static_cast<size_t>(G) * p.ommPerWarp * kInBlockPoses * p.chunks * 3 * sizeof(float);
    if (bytes <= kChunkSmemMax) {
      p.inBlock = 1;
      p.groupsPerBlock = G;
      const uint64_t groups = p.tasks / p.chunks;
      p.tasks = (groups + G - 1) / G * G * p.chunks;
    }
  }
  return p;
}


// Cuts the poses of a pre-drawn launch into ranges so that about kFillWarps
// warp tasks exist.
WarpPlan splitPoses(WarpPlan plan, uint32_t P, uint64_t fill = kFillWarps) {
  if (P < 2 || plan.tasks >= fill / 2) return plan;
  uint64_t S = (fill + plan.tasks - 1) / plan.tasks;
  if (S > P) S = P;
  const uint32_t pps = static_cast<uint32_t>((P + S - 1) / S);
  plan.posesPerSplit = pps;
  plan.poseSplits = (P + pps - 1) / pps;
  plan.tasks *= plan.poseSplits;
  return plan;
}
}  // namespace

size_t renderDrawBytes(uint32_t N, uint32_t spp, uint32_t P) {
  const WarpPlan plan = splitPoses(planWarps(N, spp), P);
  if (plan.poseSplits <= 1) return 0;
  return static_cast<size_t>(P) * N * spp * sizeof(float2);
}

WarpPlan planBatch(uint32_t N, uint32_t spp) {
  WarpPlan p = planRender(N, spp, 1, true);
  p.blockWarps = batchBlockThreads() / 32;
  return p;
}

uint32_t batchBlockThreads() { return g_blockThreads ? g_blockThreads : 128u; }

// In-block chunk sums are built for the plain and recording renders on the
// two-wide BVH only.
static bool inBlockAllowed(const DevScene& scene, bool rec, bool stats) {
  return !stats && !scene.lighting && (scene.width == 2 || rec);
}

size_t renderScratchFloats(const DevScene& scene, uint32_t N, uint32_t spp, uint32_t P, bool rec, bool stats,
                           bool forceScratch) {
  const WarpPlan p = planRender(N, spp, P, forceScratch, inBlockAllowed(scene, rec, stats));
  if (p.chunks == 1 || p.inBlock) return 0;
  return static_cast<size_t>(P) * N * p.chunks * 3;
}

// Occupancy variant of the plain render kernel: 0, 1, 2 = register budgets
// for 5, 6 and 8 resident 128-thread blocks per SM.
static int g_renderVariant = 0;

int renderVariantCount() { return 3; }
void setRenderVariant(int v) { g_renderVariant = (v >= 0 && v < 3) ? v : 0; }
int renderVariant() { return g_renderVariant; }

cudaError_t launchRngInit(const DevEye& eye, uint32_t* errFlag, cudaStream_t stream) {
  const size_t total = static_cast<size_t>(eye.N) * eye.spp;
  if (total == 0) return cudaSuccess;
  const unsigned blocks = static_cast<unsigned>((total + 255) / 256);
  rngInitKernel<<<blocks, 256, 0, stream>>>(eye, errFlag);
  return cudaGetLastError();
}

namespace {
// One launch of renderKernel<kMode, kRegs> with the plan's block size and,
// for in-block chunk sums, the shared memory of the partials.
// Launch of the kernel instance with (kInBlock) or without in-block chunk sums.
template <int kMode, int kRegs, int kWidth, bool kInBlock>
cudaError_t runRenderKernel(const DevScene& scene, const DevEye& eye, const float4* poses, uint32_t P,
                            const WarpPlan& plan, float* out, float* scratch, uint32_t* errFlag, RayRecord* rec,
                            unsigned long long* stats, cudaStream_t stream) {
  const unsigned block = 32u * plan.blockWarps;
  const uint64_t blocks = (plan.tasks + plan.blockWarps - 1) / plan.blockWarps;
  if (blocks > 0x7fffffffULL) return cudaErrorInvalidConfiguration;
  size_t smem = 0;
  if (kInBlock) {
    smem = static_cast<size_t>(plan.groupsPerBlock) * plan.ommPerWarp * kInBlockPoses * plan.chunks * 3 * sizeof(float);
    if (smem > 48 * 1024) {
      const cudaError_t e = cudaFuncSetAttribute(renderKernel<kMode, kRegs, kWidth, kInBlock>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 static_cast<int>(kChunkSmemMax));
      if (e != cudaSuccess) return e;
    }
  }
  renderKernel<kMode, kRegs, kWidth, kInBlock><<<static_cast<unsigned>(blocks), block, smem, stream>>>(
      scene, eye, poses, P, plan, out, scratch, errFlag, rec, stats);
  return cudaGetLastError();
}

// In-block chunk sums exist for the plain and recording renders on the
// two-wide BVH (planRender offers them only there, see inBlockAllowed).
template <int kMode, int kRegs, int kWidth = 2>
cudaError_t runRender(const DevScene& scene, const DevEye& eye, const float4* poses, uint32_t P,
                      const WarpPlan& plan, float* out, float* scratch, uint32_t* errFlag, RayRecord* rec,
                      unsigned long long* stats, cudaStream_t stream) {
  constexpr bool kHasInBlock = (kMode == 0 || kMode == 1) && kWidth == 2;
  if (plan.inBlock) {
    if (!kHasInBlock) return cudaErrorInvalidValue;
    return runRenderKernel<kMode, kRegs, kWidth, kHasInBlock>(scene, eye, poses, P, plan, out, scratch, errFlag,
                                                              rec, stats, stream);
  }
  return runRenderKernel<kMode, kRegs, kWidth, false>(scene, eye, poses, P, plan, out, scratch, errFlag, rec,
                                                      stats, stream);
}

// The plain render (mode 0) or the counting render (mode 2) of the scene's
// BVH width.
template <int kMode, int kRegs>
cudaError_t runRenderWidth(const DevScene& scene, const DevEye& eye, const float4* poses, uint32_t P,
                           const WarpPlan& plan, float* out, float* scratch, uint32_t* errFlag,
                           unsigned long long* stats, cudaStream_t stream) {
  switch (scene.width) {
    case 4:
      return runRender<kMode, kRegs, 4>(scene, eye, poses, P, plan, out, scratch, errFlag, nullptr, stats, stream);
    case 8:
      return runRender<kMode, kRegs, 8>(scene, eye, poses, P, plan, out, scratch, errFlag, nullptr, stats, stream);
    default:
      return runRender<kMode, kRegs, 2>(scene, eye, poses, P, plan, out, scratch, errFlag, nullptr, stats, stream);
  }
}
}  // namespace

cudaError_t launchRender(const DevScene& scene, const DevEye& eye, const float4* poses, uint32_t P, float* out,
                         float* scratch, uint32_t* errFlag, RayRecord* rec, cudaStream_t stream,
                         unsigned long long* stats, bool forceScratch) {
  if (P == 0 || eye.N == 0) return cudaSuccess;
  WarpPlan plan = planRender(eye.N, eye.spp, P, forceScratch, inBlockAllowed(scene, rec != nullptr, stats != nullptr));
  if (plan.chunks > 1 && !plan.inBlock && scratch == nullptr) return cudaErrorInvalidValue;
  if (eye.draws) {
    if (plan.inBlock) return cudaErrorInvalidValue;  // planRender keeps splittable launches out of shared memory
    const size_t total = static_cast<size_t>(eye.N) * eye.spp;
    drawsKernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, stream>>>(eye, P);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    plan = splitPoses(plan, P);
  }
  if (eye.cuts && (scene.width == 2 || rec || scene.lighting)) {  // the wide BVH searches without a cut
    if (!(eye.cutRadius > 0.f)) return cudaErrorInvalidValue;
    cutKernel<<<(P + 63) / 64, 64, 0, stream>>>(scene, poses, P, eye.cutRadius, eye.maxRel, eye.cuts);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  cudaError_t e;
  if (scene.lighting && !stats) {
    if (!scene.light) return cudaErrorInvalidValue;
    e = rec ? runRender<5, 96>(scene, eye, poses, P, plan, out, scratch, errFlag, rec, nullptr, stream)
            : runRender<4, 96>(scene, eye, poses, P, plan, out, scratch, errFlag, nullptr, nullptr, stream);
  } else if (rec) {
    e = runRender<1, 96>(scene, eye, poses, P, plan, out, scratch, errFlag, rec, nullptr, stream);
  } else if (stats) {
    e = runRenderWidth<2, 96>(scene, eye, poses, P, plan, out, scratch, errFlag, stats, stream);
  } else {
    switch (g_renderVariant) {
      case 1:
        e = runRenderWidth<0, 80>(scene, eye, poses, P, plan, out, scratch, errFlag, nullptr, stream);
        break;
      case 2:
        e = runRenderWidth<0, 64>(scene, eye, poses, P, plan, out, scratch, errFlag, nullptr, stream);
        break;
      default:
        e = runRenderWidth<0, 96>(scene, eye, poses, P, plan, out, scratch, errFlag, nullptr, stream);
        break;
    }
  }
  if (e != cudaSuccess || plan.chunks == 1 || plan.inBlock) return e;
  const size_t count = static_cast<size_t>(P) * eye.N;
  combineChunksKernel<<<static_cast<unsigned>((count + 255) / 256), 256, 0, stream>>>(scratch, plan.chunks, count, out);
  return cudaGetLastError();
}

cudaError_t launchFeatures(const DevScene& scene, const DevEye& eye, const float4* poses, uint32_t P, float* stats,
                           uint32_t* errFlag, cudaStream_t stream, bool cutsReady) {
  if (P == 0 || eye.N == 0) return cudaSuccess;
  WarpPlan plan = planWarps(eye.N, eye.spp);
  if (plan.chunks != 1) return cudaErrorInvalidValue;  // feature renders use at most 32 samples
  if (!eye.netDraws) return cudaErrorInvalidValue;  // feature renders draw from shifted nets
  // Counter-based draws: spread the poses over enough warps for about a
  // dozen waves, so that the last one costs little.
  plan = splitPoses(plan, P, 4 * kFillWarps);
  if (eye.cuts && !cutsReady) {
    if (!(eye.cutRadius > 0.f)) return cudaErrorInvalidValue;
    cutKernel<<<(P + 63) / 64, 64, 0, stream>>>(scene, poses, P, eye.cutRadius, eye.maxRel, eye.cuts);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  switch (g_renderVariant) {
    case 1: return runRender<3, 80>(scene, eye, poses, P, plan, stats, nullptr, errFlag, nullptr, nullptr, stream);
    case 2: return runRender<3, 64>(scene, eye, poses, P, plan, stats, nullptr, errFlag, nullptr, nullptr, stream);
    default: return runRender<3, 96>(scene, eye, poses, P, plan, stats, nullptr, errFlag, nullptr, nullptr, stream);
  }
}

int batchBlocksPerSM(int variant) {
  int blocks = 0;
  cudaError_t e;
  const int bt = static_cast<int>(batchBlockThreads());
  switch (variant) {
    case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, batchKernel<80>, bt, 0); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, batchKernel<64>, bt, 0); break;
    default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, batchKernel<96>, bt, 0); break;
  }
  return e == cudaSuccess ? blocks : 0;
}

cudaError_t launchBatch(const DevScene& scene, const BatchEye* eyes, const unsigned long long* taskBase,
                        const unsigned long long* cellBase, uint32_t nEyes, unsigned long long totalTasks,
                        unsigned long long totalCells, unsigned long long* ctrl, uint32_t* errFlag, int variant,
                        int gridBlocks, uint32_t cutPoses, cudaStream_t stream) {
  if (nEyes == 0 || gridBlocks <= 0) return cudaSuccess;
  if (cutPoses) {
    const uint64_t n = static_cast<uint64_t>(nEyes) * cutPoses;
    batchCutKernel<<<static_cast<unsigned>((n + 63) / 64), 64, 0, stream>>>(scene, eyes, nEyes, cutPoses);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const unsigned bt = batchBlockThreads();
  auto run = [&](auto regsTag) {
    constexpr int R = decltype(regsTag)::value;
    switch (scene.width) {
      case 4: batchKernel<R, 4><<<gridBlocks, bt, 0, stream>>>(scene, eyes, taskBase, nEyes, totalTasks, ctrl, errFlag); break;
      case 8: batchKernel<R, 8><<<gridBlocks, bt, 0, stream>>>(scene, eyes, taskBase, nEyes, totalTasks, ctrl, errFlag); break;
      default: batchKernel<R, 2><<<gridBlocks, bt, 0, stream>>>(scene, eyes, taskBase, nEyes, totalTasks, ctrl, errFlag); break;
    }
  };
  switch (variant) {
    case 1: run(std::integral_constant<int, 80>{}); break;
    case 2: run(std::integral_constant<int, 64>{}); break;
    default: run(std::integral_constant<int, 96>{}); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || totalCells == 0) return e;
  batchCombineKernel<<<static_cast<unsigned>((totalCells + 255) / 256), 256, 0, stream>>>(eyes, cellBase, nEyes,
                                                                                            totalCells);
  return cudaGetLastError();
}

cudaError_t launchSpherical(const float4* omm, float* lenScratch, uint32_t N, const float* sums, uchar4* frame, int w,
                            int h, int kind, const SphereGridSet* grids, cudaStream_t stream) {
  if (w <= 0 || h <= 0 || N == 0) return cudaSuccess;
  if (kind < 0 || kind > 4) return cudaErrorInvalidValue;
  lengthsKernel<<<(N + 255) / 256, 256, 0, stream>>>(omm, N, lenScratch);
  dim3 grid((w + 127) / 128, h);
  if (grids)
    sphericalGridKernel<<<grid, 128, 0, stream>>>(omm, lenScratch, N, *grids, sums, frame, w, h, kind);
  else
    sphericalKernel<<<grid, 128, 0, stream>>>(omm, lenScratch, N, sums, frame, w, h, kind);
  return cudaGetLastError();
}

cudaError_t launchRawSamples(const RayRecord* rec, uint32_t N, uint32_t spp, uchar4* frame, int w, int h,
                             cudaStream_t stream) {
  if (w <= 0 || h <= 0) return cudaSuccess;
  dim3 grid((w + 127) / 128, h);
  rawSamplesKernel<<<grid, 128, 0, stream>>>(rec, N, spp, frame, w, h);
  return cudaGetLastError();
}

cudaError_t launchProject(const float* sums, uint32_t N, uchar4* frame, int w, int h, int mode, cudaStream_t stream) {
  if (w <= 0 || h <= 0) return cudaSuccess;
  dim3 grid((w + 127) / 128, h);
  projectKernel<<<grid, 128, 0, stream>>>(sums, N, frame, w, h, mode);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Adaptive sampling: entries (pose, ommatidium) rendered at per-entry sample
// counts, grouped into buckets of one power-of-two count each.
// ---------------------------------------------------------------------------
namespace {

// Sort key of a sample by where its ray leaves the acceptance cone: the
// splay (in standard deviations) and the turn about the axis, as a point of
// the cone's cross-section, in a 2D Morton order of 16-bit cells over
// [-4, 4]^2.  Samples with neighbouring keys leave in neighbouring directions.
__device__ __forceinline__ uint32_t coneKey(float nd, float ud) {
  float sn, cs;
  __sincosf(ud * CR_PI_F, &sn, &cs);
  auto cell = [](float v) {
    const float q = fminf(fmaxf((v + 4.0f) * (65535.0f / 8.0f), 0.0f), 65535.0f);
    uint32_t x = static_cast<uint32_t>(q);
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
  };
  return (cell(nd * cs) << 1) | cell(nd * sn);
}

// One warp task of a bucket: up to 32 samples of one entry, or several whole
// entries when the bucket's count is below 32 (the render kernel's plan);
// with more than 32 samples per entry a task is spl rounds of 32 samples of
// one entry (chunks of 32 * spl samples when the count is larger still).
//
// A warp takes a pool of consecutive tasks of one bucket, up to kPoolRounds
// rounds of 32 sample slots, and works through it with ray refill (warp-level
// ray compaction):
//   1. the random numbers of every slot of the pool are drawn first, all 32
//      lanes busy (netDraw: sample s of entry e is point s of a digitally
//      shifted Sobol' net, so an entry's samples are stratified over its
//      cone; O(1) set-up per sample).  With more than 32 samples
//      per task, on scenes whose traversals are long and vary from ray to ray
//      (at least kAdaptiveSortMinTris triangles), each task's samples are
//      sorted by where they leave the cone (coneKey, bitonic sort in shared
//      memory), so that neighbouring slots trace neighbouring directions;
//   2. each lane traces one slot at a time.  The warp traverses in bursts of
//      `steps` BVH steps; between bursts, lanes whose ray has finished shade
//      it and store its colour in shared memory, and once at least
//      `refillIdle` lanes are idle they all take the next slots of the pool.
//      So lanes do not wait for the longest ray of a round of 32, and a new
//      ray's set-up runs on many lanes at once;
//   3. each task is summed in a fixed order that does not depend on the
//      scheduling: lane L adds the colours of slot L of the task's rounds in
//      round order (fma with 1/spp), then the segmented butterfly over the
//      lanes of an entry.  Results are deterministic.
// Every sample is traced once with its own random numbers.
constexpr uint32_t kAdaptiveSortMinTris = 16384;

constexpr uint32_t kPoolRounds = 8;
constexpr uint32_t kPoolSlots = 32 * kPoolRounds;
constexpr uint32_t kAdaptiveWarps = 4;  // warps per 128-thread block

__device__ __forceinline__ uint32_t lanesBelow(uint32_t lane) { return (1u << lane) - 1u; }

template <int kWidth, int kMinBlocks = 5>
__global__ void __launch_bounds__(128, kMinBlocks)
    adaptiveKernel(DevScene sc, const float4* __restrict__ omm, uint32_t N, const float4* __restrict__ poses,
                   AdaptiveLaunch L, unsigned long long seed, float* __restrict__ sums, uint32_t* errFlag,
                   RayRecord* __restrict__ rec, const float4* __restrict__ cuts) {
  __shared__ uint32_t sortIdx[kAdaptiveWarps][kPoolSlots];
  __shared__ float2 slotDraw[kAdaptiveWarps][kPoolSlots];  // by sample position k within its task segment
  // Unscaled colour of every slot; its red plane holds the sort keys first
  // (the keys are dead once sorted, before any colour is written), so that
  // the block needs 24 KB and 8 blocks fit on an SM.
  __shared__ float slotCol[kAdaptiveWarps][3][kPoolSlots];
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  const uint32_t pool = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // totalPools < 2^26 (checked at launch)
  if (pool >= L.totalPools) return;  // whole warps
  uint32_t bi = 0;
  while (bi + 1 < L.nBuckets && pool >= L.b[bi + 1].poolBase) ++bi;
  const AdaptiveBucket B = L.b[bi];
  const uint32_t spp = B.spp;
  const uint32_t segWidth = spp < 32u ? spp : 32u;
  const uint32_t perWarp = 32u / segWidth;
  const uint32_t spl = adaptiveSamplesPerLane(spp);  // rounds per task
  const uint32_t chunks = adaptiveChunks(spp);
  // segWidth, spl and chunks are powers of two (spp is): their logarithms
  // turn the slot arithmetic below into shifts and masks.
  const uint32_t lsw = __ffs(segWidth) - 1, lspl = __ffs(spl) - 1, lch = __ffs(chunks) - 1;
  const uint32_t tpp = kPoolRounds / spl;  // tasks per pool
  const uint64_t task0 = static_cast<uint64_t>(pool - B.poolBase) * tpp;
  const uint64_t left = B.tasks - task0;
  const uint32_t nTasks = left < tpp ? static_cast<uint32_t>(left) : tpp;
  const uint32_t nSlots = nTasks * spl * 32u;
  const bool sorted = spl > 1 && sc.triCount >= kAdaptiveSortMinTris;
  uint32_t* key = reinterpret_cast<uint32_t*>(slotCol[w][0]);
  uint32_t* idx = sortIdx[w];
  float2* draw = slotDraw[w];
  float* colR = slotCol[w][0];
  float* colG = slotCol[w][1];
  float* colB = slotCol[w][2];
  const float invSpp = 1.0f / static_cast<float>(spp);

  // Slot j of the pool: round r = j / 32 of task q = r / spl, lane position
  // j % 32.  Entry (index within the bucket) and sample of a slot:
  auto slotEntry = [&](uint32_t j) -> uint32_t {
    const uint64_t t = task0 + ((j >> 5) >> lspl);
    const uint64_t group = t >> lch;
    return static_cast<uint32_t>(group * perWarp + ((j & 31u) >> lsw));
  };
  // Sample position k within the task's segment (slot j's draws are draw[seg + k]).
  auto slotK = [&](uint32_t j) -> uint32_t {
    const uint32_t seg = j & ~((32u << lspl) - 1u), pos = j - seg;
    return spl > 1 ? (sorted ? idx[seg + pos] : pos) : (j & (segWidth - 1u));
  };
  auto slotSample = [&](uint32_t j, uint32_t k) -> uint32_t {
    const uint64_t t = task0 + ((j >> 5) >> lspl);
    const uint32_t chunk = static_cast<uint32_t>(t) & (chunks - 1u);
    return (chunk << (5 + lspl)) + k;
  };

  // 1. Random numbers (and sort keys) of every slot.
  for (uint32_t j = lane; j < nSlots; j += 32u) {
    const uint32_t i = slotEntry(j);
    const uint32_t seg = j & ~((32u << lspl) - 1u);
    const uint32_t k = spl > 1 ? j - seg : (j & (segWidth - 1u));
    float2 d = make_float2(0.f, 0.f);
    if (i < B.count) d = netDraw(seed, B.entries[i], slotSample(j, k));
    draw[spl > 1 ? seg + k : j] = d;
    if (sorted) {
      key[j] = coneKey(d.x, d.y);
      idx[j] = k;
    }
  }
  __syncwarp();
  if (sorted) {  // bitonic sort of each task's (key, position) pairs, ascending
    const uint32_t n = 32u * spl, lhalf = 4 + lspl;  // n / 2 = 2^lhalf compare-exchanges per task
    for (uint32_t size = 2; size <= n; size <<= 1)
      for (uint32_t ls = __ffs(size) - 2, stride = size >> 1; stride > 0; stride >>= 1, --ls) {
        for (uint32_t m = lane; m < nSlots / 2; m += 32u) {
          const uint32_t seg = (m >> lhalf) << (lhalf + 1), mm = m & ((1u << lhalf) - 1u);
          const uint32_t lo = seg + (((mm >> ls) << ls) << 1) + (mm & (stride - 1u)), hi = lo + stride;
          const bool up = ((lo - seg) & size) == 0u;
          const uint32_t ka = key[lo], kb = key[hi];
          if ((ka > kb) == up) {
            key[lo] = kb;
            key[hi] = ka;
            const uint32_t t2 = idx[lo];
            idx[lo] = idx[hi];
            idx[hi] = t2;
          }
        }
        __syncwarp();
      }
  }

  // 2. Trace with refill.
  int stack[kWidth == 2 ? kStackSize : kWideStackSize];
  int sp = 0, node = 0;
  bool restart = false, live = false;
  float guard = 0.f, dlen = 0.f, fpo = 0.f;
  int slot = -1;  // the slot this lane traces, -1 when idle
  v3 dir = mk(0.f, 0.f, 0.f), org = mk(0.f, 0.f, 0.f);
  float nd = 0.f, ud = 0.f;
  Hit h;
  h.t = 0.f;
  h.id = 0xffffffffu;
  h.pos = 0;
  Ray ray = setupRay(mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 1.f), sc.extent);
  uint32_t next = 0;  // next slot of the pool to hand out (warp-uniform)
  for (;;) {
    // Shade the rays that finished in the last burst.
    if (slot >= 0 && !live) {
      v3 c;
      float b1 = 0.f, b2 = 0.f;
      if (h.id != 0xffffffffu) {
        b1 = xdiv(h.V, h.det);
        b2 = xdiv(h.W, h.det);
        c = shadeHit(sc, h.pos, b1, b2);
      } else {
        c = shadeMiss(sc.miss, dir);
      }
      const uint32_t j = static_cast<uint32_t>(slot);
      colR[j] = c.x;
      colG[j] = c.y;
      colB[j] = c.z;
      if (rec) {
        RayRecord& R = rec[static_cast<size_t>(slotEntry(j)) * spp + slotSample(j, slotK(j))];
        R.normalDraw = nd;
        R.uniformDraw = ud;
        R.ox = org.x;
        R.oy = org.y;
        R.oz = org.z;
        R.dx = dir.x;
        R.dy = dir.y;
        R.dz = dir.z;
        R.t = h.id != 0xffffffffu ? h.t : -1.0f;
        R.b1 = b1;
        R.b2 = b2;
        R.hitId = h.id != 0xffffffffu ? static_cast<int32_t>(h.id) : -1;
        R.r = c.x;
        R.g = c.y;
        R.b = c.z;
        R.pad = 0.f;
      }
      slot = -1;
    }
    // Refill once enough lanes are idle (or all are).
    const uint32_t idle = __ballot_sync(0xffffffffu, slot < 0);
    const uint32_t nIdle = __popc(idle);
    if (next < nSlots && (nIdle >= L.refillIdle || nIdle == 32u)) {
      if (slot < 0) {
        const uint32_t j = next + __popc(idle & lanesBelow(lane));
        if (j < nSlots) {
          const uint32_t i = slotEntry(j);
          if (i < B.count) {
            slot = static_cast<int>(j);
            const uint32_t e = B.entries[i];
            const uint32_t p = e / N, o = e - p * N;
            const float2 d = draw[spl > 1 ? (j & ~((32u << lspl) - 1u)) + slotK(j) : j];
            nd = d.x;
            ud = d.y;
            const float4 a = __ldg(omm + 2 * o), b = __ldg(omm + 2 * o + 1);
            const v3 axis = mk(a.w, b.x, b.y);
            fpo = b.w;
            const float sd = b.z / FWHM_SD_RATIO;
            v3 perp = cross(mk(0.0f, 1.0f, 0.0f), axis);
            perp = (perp.x + perp.y + perp.z == 0.0f) ? mk(0.0f, 0.0f, 1.0f) : normalize(perp);
            const v3 relPos = mk(a.x, a.y, a.z) - normalize(axis) * fpo;
            const float4* pp = poses + 4 * p;
            const float4 P0 = __ldg(pp), X = __ldg(pp + 1), Y = __ldg(pp + 2), Z = __ldg(pp + 3);
            org = mk(P0.x, P0.y, P0.z) + mk(X.x, X.y, X.z) * relPos.x + mk(Y.x, Y.y, Y.z) * relPos.y +
                  mk(Z.x, Z.y, Z.z) * relPos.z;
            const v3 splayed = rotatePoint(axis, nd * sd, perp);
            const v3 rel = rotatePoint(splayed, ud * CR_PI_F, axis);
            dir = mk(X.x, X.y, X.z) * rel.x + mk(Y.x, Y.y, Y.z) * rel.y + mk(Z.x, Z.y, Z.z) * rel.z;
            ray = setupRay(org, dir, sc.extent);
            dlen = sqrtf(dot(dir, dir));
            if (kWidth == 2) {
              live = beginTrace(sc, ray, fpo, 1e16f, h, stack, sp, node, restart, guard,
                                cuts ? cuts + static_cast<size_t>(p) * kCutStride : nullptr);
            } else {
              h.t = 1e16f;
              h.id = 0xffffffffu;
              h.pos = 0;
              sp = 0;
              node = 0;
              live = sc.triCount > 0;
            }
          } else {  // past the bucket's last entry: contributes nothing
            colR[j] = colG[j] = colB[j] = 0.f;
          }
        }
      }
      next = min(nSlots, next + nIdle);
    }
    if (__ballot_sync(0xffffffffu, slot >= 0) == 0u) {
      if (next >= nSlots) break;
      continue;  // every refilled slot was past the bucket's end: refill again
    }
    if (slot >= 0 && live) {
      if (kWidth == 2) {
        live = !traverseBurst(sc, ray, fpo, h, stack, sp, node, restart, guard, dlen, errFlag, L.steps);
      } else {
        uint32_t nv = 0, tt = 0;
        live = !traverseWide<kWidth == 8 ? 8 : 4>(sc, ray, fpo, h, stack, sp, node, errFlag, nv, tt, false, L.steps);
      }
    }
  }
  __syncwarp();

  // 3. Fixed-order sums of every task of the pool.
  for (uint32_t q = 0; q < nTasks; ++q) {
    v3 col = mk(0.f, 0.f, 0.f);
    for (uint32_t r = 0; r < spl; ++r) {
      const uint32_t j = (q * spl + r) * 32u + lane;
      col.x = fmaf(colR[j], invSpp, col.x);
      col.y = fmaf(colG[j], invSpp, col.y);
      col.z = fmaf(colB[j], invSpp, col.z);
    }
    for (uint32_t m = segWidth >> 1; m >= 1u; m >>= 1) {
      col.x += __shfl_xor_sync(0xffffffffu, col.x, static_cast<int>(m));
      col.y += __shfl_xor_sync(0xffffffffu, col.y, static_cast<int>(m));
      col.z += __shfl_xor_sync(0xffffffffu, col.z, static_cast<int>(m));
    }
    const uint32_t j0 = (q << (5 + lspl)) + lane;
    const uint32_t i = slotEntry(j0);
    if ((lane & (segWidth - 1u)) == 0u && i < B.count) {
      const uint64_t t = task0 + q;
      const uint32_t chunk = static_cast<uint32_t>(t) & (chunks - 1u);
      float* dst = chunks == 1 ? sums + 3 * static_cast<size_t>(B.entries[i])
                               : B.partials + (static_cast<size_t>(i) * chunks + chunk) * 3;
      dst[0] = col.x;
      dst[1] = col.y;
      dst[2] = col.z;
    }
  }
}

// Chunk partials of one bucket summed in chunk order into the entries' sums.
__global__ void adaptiveCombineKernel(AdaptiveBucket B, float* __restrict__ sums) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= B.count) return;
  const uint32_t chunks = adaptiveChunks(B.spp);
  const float* src = B.partials + i * chunks * 3;
  float x = 0.f, y = 0.f, z = 0.f;
  for (uint32_t c = 0; c < chunks; ++c) {
    x += src[3 * c];
    y += src[3 * c + 1];
    z += src[3 * c + 2];
  }
  float* dst = sums + 3 * static_cast<size_t>(B.entries[i]);
  dst[0] = x;
  dst[1] = y;
  dst[2] = z;
}

// Minimum-sample labels: for entries still unlabelled, the sample standard
// deviation (n - 1) across the k renders of this sample count, per channel;
// when every channel is below thr the entry's label becomes `spp`.  The
// arithmetic is explicitly rounded (sums in render order, one division, one
// square root) so that a CPU restatement gives the same labels bit for bit.
__global__ void labelKernel(const float* __restrict__ outs, int k, uint64_t rows, uint32_t spp, float thr,
                            uint16_t* __restrict__ label) {
  const uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= rows || label[e] != 0) return;
  float worst = 0.f;
  for (int ch = 0; ch < 3; ++ch) {
    float m = 0.f;
    for (int j = 0; j < k; ++j) m = xadd(m, outs[(static_cast<size_t>(j) * rows + e) * 3 + ch]);
    m = xdiv(m, static_cast<float>(k));
    float v = 0.f;
    for (int j = 0; j < k; ++j) {
      const float d = xsub(outs[(static_cast<size_t>(j) * rows + e) * 3 + ch], m);
      v = xadd(v, xmul(d, d));
    }
    worst = fmaxf(worst, xsqrt(xdiv(v, static_cast<float>(k - 1))));
  }
  if (worst < thr) label[e] = static_cast<uint16_t>(spp);
}

// Bucket of every entry from the allocator's prediction l (mean of its three
// outputs; the predicted count is 2^(10 l)): level = bucket index 0..8 of
// 4 << index samples, 0x80 | 8 for a fallback entry (more than 1024 needed),
// or kNoRender (at most featureSpp samples needed: the feature render suffices).
// The count rendered is 2^(exponent * log2(predicted) - halvings), the
// predicted count capped at 2048: exponent 1 divides every predicted count by
// 2^halvings (halvings >= 0, possibly fractional: the per-entry error budget
// traded for rays; a halving of 1 or more leaves no fallback); exponent 1/2
// renders counts proportional to the square root of the predicted count,
// i.e. to the entry's standard deviation, which for a fixed number of rays
// minimises the summed squared error of all entries (Neyman allocation).
// costExponent > 0 further divides the count by (cost / kCostRef)^costExponent,
// cost the entry's mean BVH node visits plus triangle tests per ray in the
// feature render (at least 1), so that for a fixed render time rather than a
// fixed number of rays the error is smallest at exponent = costExponent = 1/2.
__global__ void allocateKernel(const float* __restrict__ pred, uint64_t rows, uint32_t featureSpp,
                               uint8_t* __restrict__ level, unsigned long long* __restrict__ counts, float halvings,
                               float exponent, const float* __restrict__ stats, float costExponent) {
  const uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  int bucket = -1;  // counted bucket of this row (-1: none)
  if (e < rows) {
    const float l = (pred[3 * e] + pred[3 * e + 1] + pred[3 * e + 2]) * (1.0f / 3.0f);
    const float l10 = l * 10.0f;
    // Cost term: entries whose rays cost more get fewer of them (for a fixed
    // render time the summed squared error is smallest with counts in
    // proportion to sigma / sqrt(cost): exponent 1/2, costExponent 1/2).
    const float shift =
        costExponent != 0.0f ? costExponent * log2f(fmaxf(stats[e * kFeatureStats + kCostStat], 1.0f) / kCostRef)
                             : 0.0f;
    float kf = l10 == l10 ? ceilf(fminf(l10, 11.0f) * exponent - halvings - shift - 1e-3f) : 2.0f;  // NaN: least
    if (!(kf >= 2.0f)) kf = 2.0f;
    if (kf > 11.0f) kf = 11.0f;
    const int k = static_cast<int>(kf);
    uint8_t lv;
    if ((1u << k) <= featureSpp) {
      lv = kNoRender;
    } else if (k == 11) {
      lv = 0x80 | 8;
    } else {
      lv = static_cast<uint8_t>(k - 2);
    }
    level[e] = lv;
    if (lv != kNoRender) bucket = lv & 0x7f;
  }
  // One atomic per bucket and warp (blockDim is a multiple of 32).
  const unsigned peers = __match_any_sync(0xffffffffu, bucket);
  if (bucket >= 0 && (threadIdx.x & 31u) == static_cast<unsigned>(__ffs(peers) - 1))
    atomicAdd(counts + bucket, static_cast<unsigned long long>(__popc(peers)));
}

// Ordered bucket lists in three steps, so that every bucket lists its
// entries pose by pose and, within a pose, in the eye's direction order
// (consecutive warps then trace neighbouring ommatidia of one pose):
// per-block bucket counts over tiles of kScatterTile positions, an exclusive
// scan over the tiles per bucket, and the placement with warp ballots.
constexpr int kScatterTile = 1024;

__device__ __forceinline__ int bucketOf(uint8_t lv) { return lv == kNoRender ? -1 : (lv & 0x7f); }

// Entry at ordered position x (pose x / N, the (x % N)-th ommatidium of the order).
__device__ __forceinline__ uint64_t entryAt(uint64_t x, uint32_t N, const uint32_t* __restrict__ order) {
  const uint64_t p = x / N;
  const uint32_t j = static_cast<uint32_t>(x % N);
  return p * N + (order ? __ldg(order + j) : j);
}

__global__ void __launch_bounds__(kScatterTile) bucketCountKernel(const uint8_t* __restrict__ level, uint64_t rows,
                                                                   uint32_t N, const uint32_t* __restrict__ order,
                                                                   unsigned long long* __restrict__ tileCounts) {
  __shared__ unsigned int cnt[kAdaptiveBuckets];
  if (threadIdx.x < kAdaptiveBuckets) cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t x = static_cast<uint64_t>(blockIdx.x) * kScatterTile + threadIdx.x;
  const int k = x < rows ? bucketOf(level[entryAt(x, N, order)]) : -1;
  if (k >= 0) atomicAdd(&cnt[k], 1u);
  __syncthreads();
  if (threadIdx.x < kAdaptiveBuckets)
    tileCounts[static_cast<size_t>(blockIdx.x) * kAdaptiveBuckets + threadIdx.x] = cnt[threadIdx.x];
}

// One warp per bucket: tileCounts[t][k] becomes the first slot of tile t's
// bucket-k entries (bucket k starting at bucketBase[k]); the warp scans 32
// tiles per step with shuffles.
__global__ void bucketScanKernel(unsigned long long* __restrict__ tileCounts, uint64_t tiles,
                                 const unsigned long long* __restrict__ bucketBase) {
  const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (k >= static_cast<int>(kAdaptiveBuckets)) return;  // whole warps
  unsigned long long run = bucketBase[k];
  for (uint64_t t0 = 0; t0 < tiles; t0 += 32) {
    const uint64_t t = t0 + lane;
    const unsigned long long c = t < tiles ? tileCounts[t * kAdaptiveBuckets + k] : 0ull;
    unsigned long long inc = c;  // inclusive prefix over the warp's 32 tiles
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long o = __shfl_up_sync(0xffffffffu, inc, d);
      if (lane >= d) inc += o;
    }
    if (t < tiles) tileCounts[t * kAdaptiveBuckets + k] = run + inc - c;
    run += __shfl_sync(0xffffffffu, inc, 31);
  }
}

__global__ void __launch_bounds__(kScatterTile) bucketPlaceKernel(const uint8_t* __restrict__ level, uint64_t rows,
                                                                   uint32_t N, const uint32_t* __restrict__ order,
                                                                   const unsigned long long* __restrict__ tileFirst,
                                                                   uint32_t* __restrict__ entries) {
  __shared__ unsigned int warpCnt[kScatterTile / 32][kAdaptiveBuckets];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t x = static_cast<uint64_t>(blockIdx.x) * kScatterTile + threadIdx.x;
  const uint64_t e = x < rows ? entryAt(x, N, order) : 0;
  const int k = x < rows ? bucketOf(level[e]) : -1;
  unsigned int rank = 0;
  for (int b = 0; b < static_cast<int>(kAdaptiveBuckets); ++b) {
    const unsigned int m = __ballot_sync(0xffffffffu, k == b);
    if (k == b) rank = __popc(m & ((1u << lane) - 1u));
    if (lane == 0) warpCnt[warp][b] = __popc(m);
  }
  __syncthreads();
  if (k < 0) return;
  unsigned long long at = tileFirst[static_cast<size_t>(blockIdx.x) * kAdaptiveBuckets + k];
  for (int w = 0; w < warp; ++w) at += warpCnt[w][k];
  entries[at + rank] = static_cast<uint32_t>(e);
}

// Final colour of every entry: the denoised feature-render estimate where no
// extra samples were needed; the sample-weighted mean of the feature render
// and the adaptive render otherwise; the adaptive 1024-sample render alone
// for fallback entries.
__global__ void adaptiveFinishKernel(const uint8_t* __restrict__ level, uint64_t rows, uint32_t featureSpp,
                                     const float* __restrict__ stats, const float* __restrict__ learned,
                                     const float* __restrict__ sums, float* __restrict__ out) {
  const uint64_t e = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= rows) return;
  const uint8_t lv = level[e];
  for (int ch = 0; ch < 3; ++ch) {
    float v;
    if (lv == kNoRender) {
      v = learned ? learned[3 * e + ch] : stats[e * kFeatureStats + ch];
    } else if (lv & 0x80) {
      v = sums[3 * e + ch];
    } else {
      const float c = static_cast<float>(4u << lv), f = static_cast<float>(featureSpp);
      v = (f * stats[e * kFeatureStats + ch] + c * sums[3 * e + ch]) / (f + c);
    }
    out[3 * e + ch] = v;
  }
}

}  // namespace

static uint32_t g_refillIdle = 16;
static int g_refillSteps = 16;
static int g_adaptiveBlocks = 5;

void setAdaptiveSchedule(uint32_t refillIdle, int steps) {
  g_refillIdle = refillIdle < 1 ? 1u : (refillIdle > 32 ? 32u : refillIdle);
  g_refillSteps = steps < 1 ? 1 : (steps > 4096 ? 4096 : steps);
}
void adaptiveSchedule(uint32_t* refillIdle, int* steps) {
  *refillIdle = g_refillIdle;
  *steps = g_refillSteps;
}
void setAdaptiveBlocksPerSM(int blocks) { g_adaptiveBlocks = (blocks == 6 || blocks == 8) ? blocks : 5; }
int adaptiveBlocksPerSM() { return g_adaptiveBlocks; }

AdaptiveLaunch planAdaptive(const uint32_t* const* entries, const uint64_t* counts, const uint32_t* spp,
                            float* const* partials, uint32_t nBuckets) {
  AdaptiveLaunch L{};
  uint64_t tasks = 0, pools = 0;
  for (uint32_t k = 0; k < nBuckets && L.nBuckets < kAdaptiveBuckets; ++k) {
    if (counts[k] == 0) continue;
    AdaptiveBucket& B = L.b[L.nBuckets++];
    B.entries = entries[k];
    B.count = counts[k];
    B.spp = spp[k];
    B.partials = partials[k];
    B.taskBase = tasks;
    B.poolBase = pools;
    const uint64_t segWidth = spp[k] < 32 ? spp[k] : 32;
    const uint64_t perWarp = 32 / segWidth, chunks = adaptiveChunks(spp[k]);
    B.tasks = (counts[k] + perWarp - 1) / perWarp * chunks;
    const uint64_t tpp = kPoolRounds / adaptiveSamplesPerLane(spp[k]);
    tasks += B.tasks;
    pools += (B.tasks + tpp - 1) / tpp;
  }
  L.totalTasks = tasks;
  L.totalPools = pools;
  L.refillIdle = g_refillIdle;
  L.steps = g_refillSteps;
  L.blocksPerSM = g_adaptiveBlocks;
  return L;
}

size_t adaptivePartialFloats(uint64_t count, uint32_t spp) {
  return adaptiveChunks(spp) > 1 ? count * adaptiveChunks(spp) * 3 : 0;
}

namespace {

// Parity ray cast of sutil/hitscanprocessing.cpp:20-83 for many points, as
// the host query (gltf.cpp pointInsideHitbox) runs it, bit for bit: the
// object-space point from the 3x3 part of the inverse transform (the
// reference's product has w = 0) in explicitly rounded double arithmetic,
// rounded once to float, then the reference's float cast in its
// operation order on explicitly rounded single-precision PTX (no FTZ, no
// contraction, so the --use_fast_math build of this file does not change it).
// With a (y, z) grid only the triangles of the point's cell are tested; the
// grid lists every triangle the full loop could count there.
__device__ __forceinline__ float fdot(float ax, float ay, float az, float bx, float by, float bz) {
  return xadd(xadd(xmul(ax, bx), xmul(ay, by)), xmul(az, bz));
}
__device__ __forceinline__ void fcross(float ax, float ay, float az, float bx, float by, float bz, float& cx, float& cy,
                                       float& cz) {
  cx = xsub(xmul(ay, bz), xmul(az, by));
  cy = xsub(xmul(az, bx), xmul(ax, bz));
  cz = xsub(xmul(ax, by), xmul(ay, bx));
}
__device__ __forceinline__ void fnormalize(float& x, float& y, float& z) {
  const float inv = xdiv(1.0f, xsqrt(fdot(x, y, z, x, y, z)));
  x = xmul(x, inv);
  y = xmul(y, inv);
  z = xmul(z, inv);
}
// dot(n, cross(s1 - s0, hit - s0)) < 0: the hit lies outside edge s0 -> s1.
__device__ __forceinline__ bool outsideEdge(float nx, float ny, float nz, float3 s0, float3 s1, float hx, float hy,
                                            float hz) {
  float cx, cy, cz;
  fcross(xsub(s1.x, s0.x), xsub(s1.y, s0.y), xsub(s1.z, s0.z), xsub(hx, s0.x), xsub(hy, s0.y), xsub(hz, s0.z), cx, cy,
         cz);
  return fdot(nx, ny, nz, cx, cy, cz) < 0.0f;
}

__global__ void insideKernel(const float3* __restrict__ tris, uint32_t nTris, InsideQuery q,
                             const float* __restrict__ pts, size_t n, uint8_t* __restrict__ out) {
  const size_t k = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  // w = 0 in the reference's product: no translation (gltf.cpp hitboxObjectPoint)
  const double qx = static_cast<double>(pts[3 * k]);
  const double qy = static_cast<double>(pts[3 * k + 1]);
  const double qz = static_cast<double>(pts[3 * k + 2]);
  float o[3];
  for (int r = 0; r < 3; ++r)
    o[r] = __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(q.inv[3 * r], qx), __dmul_rn(q.inv[3 * r + 1], qy)),
                                       __dmul_rn(q.inv[3 * r + 2], qz)));
  const float sx = static_cast<float>(q.startX), sy = o[1], sz = o[2];
  float dx = xsub(o[0], sx), dy = xsub(o[1], sy), dz = xsub(o[2], sz);
  fnormalize(dx, dy, dz);
  unsigned crossings = 0;
  // The ray runs along x at the point's (y, z): only triangles listed in the
  // grid cell of (y, z), and those whose test does not depend on the point,
  // can be crossed.  A point at the ray start has a NaN direction, for which
  // every triangle's comparisons fail and every triangle counts: test them all.
  const bool grid = q.G > 0 && isfinite(dx) && isfinite(dy) && isfinite(dz);
  uint32_t first = 0, end = nTris;
  if (grid) {
    auto cellOf = [&](double v, double v0) {
      const double c = floor(__dmul_rn(__dsub_rn(v, v0), q.cellInv));
      return c < 0.0 ? 0 : (c >= static_cast<double>(q.G) ? q.G - 1 : static_cast<int>(c));
    };
    const uint32_t c = static_cast<uint32_t>(cellOf(sz, q.z0) * q.G + cellOf(sy, q.y0));
    first = q.cellStart[c];
    end = q.cellStart[c + 1];
  }
  const uint32_t nSpecial = grid ? q.nEverywhere : 0u;
  for (uint32_t j = first; j < end + nSpecial; ++j) {
    const uint32_t t = !grid ? j : (j < end ? q.cellItems[j] : q.everywhere[j - end]);
    const float3 p0 = tris[3 * t], p1 = tris[3 * t + 1], p2 = tris[3 * t + 2];
    float nx, ny, nz;
    fcross(xsub(p1.x, p0.x), xsub(p1.y, p0.y), xsub(p1.z, p0.z), xsub(p2.x, p0.x), xsub(p2.y, p0.y), xsub(p2.z, p0.z),
           nx, ny, nz);
    fnormalize(nx, ny, nz);
    const float den = fdot(nx, ny, nz, dx, dy, dz);
    if (den == 0.0f) continue;
    const float dist = xdiv(fdot(xsub(p0.x, sx), xsub(p0.y, sy), xsub(p0.z, sz), nx, ny, nz), den);
    if (dist == 0.0f) continue;
    const float hx = xadd(sx, xmul(dist, dx)), hy = xadd(sy, xmul(dist, dy)), hz = xadd(sz, xmul(dist, dz));
    if (dist < 0.0f || hx > o[0]) continue;
    if (outsideEdge(nx, ny, nz, p0, p1, hx, hy, hz) || outsideEdge(nx, ny, nz, p1, p2, hx, hy, hz) ||
        outsideEdge(nx, ny, nz, p2, p0, hx, hy, hz))
      continue;
    ++crossings;
  }
  out[k] = (crossings & 1u) ? 1 : 0;
}

}  // namespace

cudaError_t launchInside(const float3* tris, uint32_t nTris, const InsideQuery& q, const float* pts, size_t n,
                         uint8_t* out, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  insideKernel<<<static_cast<unsigned>((n + 127) / 128), 128, 0, stream>>>(tris, nTris, q, pts, n, out);
  return cudaGetLastError();
}

cudaError_t launchCuts(const DevScene& scene, const float4* poses, uint32_t P, float radius, float maxRel,
                       float4* cuts, cudaStream_t stream) {
  if (P == 0) return cudaSuccess;
  if (!(radius > 0.f) || !cuts) return cudaErrorInvalidValue;
  cutKernel<<<(P + 63) / 64, 64, 0, stream>>>(scene, poses, P, radius, maxRel, cuts);
  return cudaGetLastError();
}

cudaError_t launchAdaptive(const DevScene& scene, const float4* omm, uint32_t N, const float4* poses,
                           const AdaptiveLaunch& L, unsigned long long seed, float* sums, uint32_t* errFlag,
                           RayRecord* rec, cudaStream_t stream, const float4* cuts) {
  if (L.totalPools == 0) return cudaSuccess;
  if (rec && L.nBuckets != 1) return cudaErrorInvalidValue;
  for (uint32_t k = 0; k < L.nBuckets; ++k) {
    const uint32_t c = L.b[k].spp;
    if (c == 0 || c > 1024 || (c & (c - 1)) || L.b[k].count > 0xffffffffull || (adaptiveChunks(c) > 1 && !L.b[k].partials))
      return cudaErrorInvalidValue;
  }
  if (L.totalPools >= (1ull << 26)) return cudaErrorInvalidConfiguration;  // 32-bit thread ids
  if (L.refillIdle < 1 || L.refillIdle > 32 || L.steps < 1) return cudaErrorInvalidValue;
  const uint64_t blocks = (L.totalPools * 32 + 127) / 128;
  switch (scene.width) {
    case 4:
      adaptiveKernel<4><<<static_cast<unsigned>(blocks), 128, 0, stream>>>(scene, omm, N, poses, L, seed, sums, errFlag,
                                                                           rec, nullptr);
      break;
    case 8:
      adaptiveKernel<8><<<static_cast<unsigned>(blocks), 128, 0, stream>>>(scene, omm, N, poses, L, seed, sums, errFlag,
                                                                           rec, nullptr);
      break;
    default:  // the two-wide BVH: the register budget follows L.blocksPerSM (6: 80, 8: 64, else 96 registers)
      if (L.blocksPerSM == 8)
        adaptiveKernel<2, 8><<<static_cast<unsigned>(blocks), 128, 0, stream>>>(scene, omm, N, poses, L, seed, sums,
                                                                                errFlag, rec, cuts);
      else if (L.blocksPerSM == 6)
        adaptiveKernel<2, 6><<<static_cast<unsigned>(blocks), 128, 0, stream>>>(scene, omm, N, poses, L, seed, sums,
                                                                                errFlag, rec, cuts);
      else
        adaptiveKernel<2, 5><<<static_cast<unsigned>(blocks), 128, 0, stream>>>(scene, omm, N, poses, L, seed, sums,
                                                                                errFlag, rec, cuts);
      break;
  }
  cudaError_t e = cudaGetLastError();
  for (uint32_t k = 0; k < L.nBuckets && e == cudaSuccess; ++k) {
    if (adaptiveChunks(L.b[k].spp) == 1) continue;
    adaptiveCombineKernel<<<static_cast<unsigned>((L.b[k].count + 255) / 256), 256, 0, stream>>>(L.b[k], sums);
    e = cudaGetLastError();
  }
  return e;
}

cudaError_t launchLabels(const float* outs, int k, uint64_t rows, uint32_t spp, float thr, uint16_t* label,
                         cudaStream_t stream) {
  if (rows == 0) return cudaSuccess;
  labelKernel<<<static_cast<unsigned>((rows + 255) / 256), 256, 0, stream>>>(outs, k, rows, spp, thr, label);
  return cudaGetLastError();
}

cudaError_t launchAllocate(const float* pred, uint64_t rows, uint32_t featureSpp, uint8_t* level,
                           unsigned long long* counts, cudaStream_t stream, float halvings, float exponent,
                           const float* stats, float costExponent) {
  if (rows == 0) return cudaSuccess;
  if (costExponent != 0.0f && !stats) return cudaErrorInvalidValue;
  allocateKernel<<<static_cast<unsigned>((rows + 255) / 256), 256, 0, stream>>>(
      pred, rows, featureSpp, level, counts, halvings, exponent, stats, costExponent);
  return cudaGetLastError();
}

size_t scatterScratchWords(uint64_t rows) {
  return ((rows + kScatterTile - 1) / kScatterTile) * kAdaptiveBuckets;
}

cudaError_t launchScatterBuckets(const uint8_t* level, uint64_t rows, uint32_t N, const uint32_t* order,
                                 const unsigned long long* bucketBase, unsigned long long* scratch, uint32_t* entries,
                                 cudaStream_t stream) {
  if (rows == 0) return cudaSuccess;
  if (N == 0 || rows % N) return cudaErrorInvalidValue;
  const uint64_t tiles = (rows + kScatterTile - 1) / kScatterTile;
  if (tiles > 0x7fffffffULL) return cudaErrorInvalidConfiguration;
  bucketCountKernel<<<static_cast<unsigned>(tiles), kScatterTile, 0, stream>>>(level, rows, N, order, scratch);
  bucketScanKernel<<<1, 32 * kAdaptiveBuckets, 0, stream>>>(scratch, tiles, bucketBase);
  bucketPlaceKernel<<<static_cast<unsigned>(tiles), kScatterTile, 0, stream>>>(level, rows, N, order, scratch,
                                                                                entries);
  return cudaGetLastError();
}

cudaError_t launchAdaptiveFinish(const uint8_t* level, uint64_t rows, uint32_t featureSpp, const float* stats,
                                 const float* learned, const float* sums, float* out, cudaStream_t stream) {
  if (rows == 0) return cudaSuccess;
  adaptiveFinishKernel<<<static_cast<unsigned>((rows + 255) / 256), 256, 0, stream>>>(level, rows, featureSpp, stats,
                                                                                        learned, sums, out);
  return cudaGetLastError();
}

}  // namespace cr

// ---------------------------------------------------------------------------
// Scratch for the allocation-free entry point.
//
// The chunk partials of a render with more than 32 samples per ommatidium
// normally live in a buffer the library allocates.  For callers that must
// not allocate device memory at call time, the same partials can live in
// this fixed array instead.  It is part of the module image, so every GPU
// that loads the library holds its 16 MiB until the process exits.  Every
// call of the allocation-free entry point uses the same array; calls that
// overlap on the GPU (different streams, or several host threads) race on
// it.  Nothing in it needs clearing: each partial is written before it is
// read within the same call.
// ---------------------------------------------------------------------------
namespace cr {

constexpr size_t kNoAllocScratchFloats = size_t(4) << 20;  // 16 MiB of float
static __device__ __align__(256) float g_noAllocScratch[kNoAllocScratchFloats];

namespace {
constexpr int kNoAllocMaxDevices = 64;
// Per-device address cache.  It is filled without a lock: the library's
// entry points are not thread-safe (one host thread at a time, as the
// reference's global singletons), and this cache relies on that contract.
float* s_noAllocScratch[kNoAllocMaxDevices] = {};
}  // namespace

size_t noAllocScratchFloats() { return kNoAllocScratchFloats; }

// Device address of the array on the current device.  In host code the
// array's name only stands for it, so the address is looked up once per
// device, with that device current, and cached.
cudaError_t noAllocScratch(float** ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  if (!s_noAllocScratch[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noAllocScratch);
    if (e != cudaSuccess) return e;
    s_noAllocScratch[dev] = static_cast<float*>(p);
  }
  *ptr = s_noAllocScratch[dev];
  return cudaSuccess;
}

}  // namespace cr
