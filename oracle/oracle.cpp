// CPU oracle of the compound-eye render path.  TEST INFRASTRUCTURE ONLY:
// used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
// the checker; nothing in the product links or calls it.
//
// Parity status: UNPINNED against the reference's own outputs.  The
// reference renders through closed OptiX/RT-core code behind a GLFW window
// and cannot be built or run here (no OptiX SDK, no graphics stack), and it
// ships no tests or golden renders.  This file restates the reference's
// shader arithmetic from its source:
//   ray generation ........ libEyeRenderer3/shaders.cu:648-709
//   closest hit (no light)  libEyeRenderer3/shaders.cu:779-811,
//                           cuda/LocalGeometry.h:55-156
//   base colour textures .. libEyeRenderer3/MulticamScene.cpp:753-833 (a
//                           uchar4 array read as value/255 through a wrap /
//                           linear / normalised-coordinate sampler), filtered
//                           by the texture unit's documented bilinear rule
//                           with weights in 1/256 steps
//   lighting-on hit ....... libEyeRenderer3/shaders.cu:60-90, 812-880 (GGX /
//                           Smith, four point lights of
//                           libEyeRenderer.cpp:100-118, shadow rays as the
//                           closest-hit search limited to [0.001, d - 0.001])
//   miss programs ......... libEyeRenderer3/shaders.cu:740-756
//   sample scaling/sum .... libEyeRenderer3/shaders.cu:730, 341-347
//   make_color ............ libEyeRenderer3/shaders.cu:180-189
// with libm transcendentals in place of the fast-math GPU intrinsics.  The
// closest-hit search (OptiX in the reference) is restated as: the closest
// triangle in the (t, triangle id) order among those the watertight
// ray/triangle test of Woop, Benthin and Wald (JCGT 2013) accepts within
// [tmin, tmax], computed with explicitly rounded float operations, over a
// median-split BVH of this file's own; plus an independent double-precision
// Moller-Trumbore search to settle rays that pass within 1e-6 of an edge.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct V3 {
  float x, y, z;
};
inline V3 mk(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 scl(float s, V3 a) { return mk(s * a.x, s * a.y, s * a.z); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline V3 normalize(V3 v) {
  const float inv = 1.0f / std::sqrt(dot(v, v));
  return scl(inv, v);
}

constexpr float kPi = 3.14159265358979323846f;
constexpr float kFwhmSdRatio = 2.35482004503094938202313865291f;

// rotatePoint (shaders.cu:648-651).
V3 rotatePoint(V3 p, float angle, V3 axis) {
  const float c = std::cos(angle), s = std::sin(angle);
  return add(add(scl(c, p), scl(s, cross(axis, p))), scl((1 - c) * dot(axis, p), axis));
}

struct Scene {
  uint32_t T = 0;
  std::vector<float> v;   // 9 per triangle
  std::vector<float> c;   // 12 per triangle
  std::vector<uint8_t> f; // shading kind: 0 base colour, 1 vertex colours, 2 texture
  std::vector<uint32_t> texels;  // RGBA8, red in the low byte
  std::vector<int32_t> texTable; // per texture: first texel, width, height
  // lighting-on data: 20 floats per triangle (normals, uvs, metallic,
  // roughness, mr texture, normal texture, flags) and four lights
  std::vector<float> light;
  int lighting = 0;
  float lightPos[4][4] = {}, lightCol[4][3] = {};
  // BVH: nodes with a box and either two children or a triangle range.
  struct Node {
    double lo[3], hi[3];
    int32_t left = -1, right = -1;
    uint32_t first = 0, count = 0;
  };
  std::vector<Node> nodes;
  std::vector<uint32_t> idx;
};

void boxOf(const Scene& s, uint32_t t, double* lo, double* hi) {
  for (int k = 0; k < 3; ++k) {
    lo[k] = std::min({(double)s.v[9 * t + k], (double)s.v[9 * t + 3 + k], (double)s.v[9 * t + 6 + k]});
    hi[k] = std::max({(double)s.v[9 * t + k], (double)s.v[9 * t + 3 + k], (double)s.v[9 * t + 6 + k]});
  }
}

int32_t buildNode(Scene& s, uint32_t first, uint32_t count, std::vector<double>& cen) {
  Scene::Node n;
  for (int k = 0; k < 3; ++k) {
    n.lo[k] = INFINITY;
    n.hi[k] = -INFINITY;
  }
  double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t i = first; i < first + count; ++i) {
    double lo[3], hi[3];
    boxOf(s, s.idx[i], lo, hi);
    for (int k = 0; k < 3; ++k) {
      n.lo[k] = std::min(n.lo[k], lo[k]);
      n.hi[k] = std::max(n.hi[k], hi[k]);
      clo[k] = std::min(clo[k], cen[3 * s.idx[i] + k]);
      chi[k] = std::max(chi[k], cen[3 * s.idx[i] + k]);
    }
  }
  const int32_t me = static_cast<int32_t>(s.nodes.size());
  s.nodes.push_back(n);
  if (count <= 4) {
    s.nodes[me].first = first;
    s.nodes[me].count = count;
    return me;
  }
  int axis = 0;
  for (int k = 1; k < 3; ++k)
    if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
  const uint32_t mid = first + count / 2;
  std::nth_element(s.idx.begin() + first, s.idx.begin() + mid, s.idx.begin() + first + count,
                   [&](uint32_t a, uint32_t b) {
                     const double ca = cen[3 * a + axis], cb = cen[3 * b + axis];
                     return ca < cb || (ca == cb && a < b);
                   });
  const int32_t l = buildNode(s, first, mid - first, cen);
  const int32_t r = buildNode(s, mid, first + count - mid, cen);
  s.nodes[me].left = l;
  s.nodes[me].right = r;
  return me;
}

// Slab test in double with a relative widening; conservative for the float
// triangle test below.
bool boxHit(const Scene::Node& n, const double* o, const double* inv, double tmin, double tmax, double& tnear) {
  double t0 = tmin, t1 = tmax;
  for (int k = 0; k < 3; ++k) {
    double a = (n.lo[k] - o[k]) * inv[k];
    double b = (n.hi[k] - o[k]) * inv[k];
    if (std::isnan(a) || std::isnan(b)) {  // zero direction and origin on a face plane
      if (o[k] < n.lo[k] || o[k] > n.hi[k]) return false;
      continue;
    }
    if (a > b) std::swap(a, b);
    t0 = std::max(t0, a);
    t1 = std::min(t1, b);
  }
  tnear = t0;
  return t0 - std::fabs(t0) * 1e-6 <= t1 + std::fabs(t1) * 1e-6;
}

// ---------------------------------------------------------------------------
// Float watertight test with explicit operation order (no contraction).
// ---------------------------------------------------------------------------
struct WRay {
  float o[3];
  int kx, ky, kz;
  float nSx, nSy, Sz;
};

WRay setupW(const float* o, const float* d) {
  WRay r;
  std::memcpy(r.o, o, sizeof(r.o));
  const float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
  int kz = 0;
  float m = ax;
  if (ay > m) {
    kz = 1;
    m = ay;
  }
  if (az > m) kz = 2;
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  if (d[kz] < 0.0f) std::swap(kx, ky);
  r.kx = kx;
  r.ky = ky;
  r.kz = kz;
  r.Sz = 1.0f / d[kz];
  r.nSx = -(d[kx] * r.Sz);
  r.nSy = -(d[ky] * r.Sz);
  return r;
}

struct Hit32 {
  float t;
  uint32_t id = 0xffffffffu;
  float U = 0, V = 0, W = 0, det = 1;
};

void testW(const WRay& r, const float* v, uint32_t id, float tmin, Hit32& h) {
  const float* A = v;
  const float* B = v + 3;
  const float* C = v + 6;
  const float Akx = A[r.kx] - r.o[r.kx], Aky = A[r.ky] - r.o[r.ky], Akz = A[r.kz] - r.o[r.kz];
  const float Bkx = B[r.kx] - r.o[r.kx], Bky = B[r.ky] - r.o[r.ky], Bkz = B[r.kz] - r.o[r.kz];
  const float Ckx = C[r.kx] - r.o[r.kx], Cky = C[r.ky] - r.o[r.ky], Ckz = C[r.kz] - r.o[r.kz];
  const float Ax = std::fma(r.nSx, Akz, Akx), Ay = std::fma(r.nSy, Akz, Aky);
  const float Bx = std::fma(r.nSx, Bkz, Bkx), By = std::fma(r.nSy, Bkz, Bky);
  const float Cx = std::fma(r.nSx, Ckz, Ckx), Cy = std::fma(r.nSy, Ckz, Cky);
  float U = std::fma(Cx, By, -(Cy * Bx));
  float V = std::fma(Ax, Cy, -(Ay * Cx));
  float W = std::fma(Bx, Ay, -(By * Ax));
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = static_cast<float>((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = static_cast<float>((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = static_cast<float>((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return;
  const float det = (U + V) + W;
  if (det == 0.0f) return;
  const float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
  const float T = std::fma(U, Az, std::fma(V, Bz, W * Cz));
  const float t = T / det;
  if (!(t >= tmin && t <= h.t)) return;
  if (t == h.t && id >= h.id) return;
  h.t = t;
  h.id = id;
  h.U = U;
  h.V = V;
  h.W = W;
  h.det = det;
}

Hit32 trace32(const Scene& s, const float* o, const float* d, float tmin, float tmax) {
  Hit32 h;
  h.t = tmax;
  if (s.T == 0) return h;
  const WRay r = setupW(o, d);
  double od[3] = {o[0], o[1], o[2]}, inv[3];
  for (int k = 0; k < 3; ++k) inv[k] = 1.0 / (double)d[k];
  int32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const Scene::Node& n = s.nodes[stack[--sp]];
    double tn;
    if (!boxHit(n, od, inv, tmin, h.t, tn)) continue;
    if (n.left < 0) {
      for (uint32_t i = n.first; i < n.first + n.count; ++i) {
        const uint32_t t = s.idx[i];
        testW(r, &s.v[9 * t], t, tmin, h);
      }
      continue;
    }
    double tl = 0, tr = 0;
    const bool hl = boxHit(s.nodes[n.left], od, inv, tmin, h.t, tl);
    const bool hr = boxHit(s.nodes[n.right], od, inv, tmin, h.t, tr);
    if (hl && hr) {
      if (tl <= tr) {
        stack[sp++] = n.right;
        stack[sp++] = n.left;
      } else {
        stack[sp++] = n.left;
        stack[sp++] = n.right;
      }
    } else if (hl) {
      stack[sp++] = n.left;
    } else if (hr) {
      stack[sp++] = n.right;
    }
  }
  return h;
}

// ---------------------------------------------------------------------------
// Double-precision Moller-Trumbore closest hit (settles near-edge rays).
// ---------------------------------------------------------------------------
struct Hit64 {
  double t;
  int64_t id = -1;
  double b0 = 0, b1 = 0, b2 = 0;
};

void testMT(const Scene& s, uint32_t t, const double* o, const double* d, double tmin, Hit64& h) {
  const float* v = &s.v[9 * t];
  const double e1[3] = {(double)v[3] - v[0], (double)v[4] - v[1], (double)v[5] - v[2]};
  const double e2[3] = {(double)v[6] - v[0], (double)v[7] - v[1], (double)v[8] - v[2]};
  const double p[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
  const double det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
  if (det == 0.0) return;
  const double inv = 1.0 / det;
  const double tv[3] = {o[0] - v[0], o[1] - v[1], o[2] - v[2]};
  const double u = (tv[0] * p[0] + tv[1] * p[1] + tv[2] * p[2]) * inv;
  const double q[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
  const double w = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) * inv;
  if (u < 0.0 || w < 0.0 || u + w > 1.0) return;
  const double tt = (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * inv;
  if (!(tt >= tmin && tt <= h.t)) return;
  if (tt == h.t && static_cast<int64_t>(t) >= h.id) return;
  h.t = tt;
  h.id = t;
  h.b0 = 1.0 - u - w;
  h.b1 = u;
  h.b2 = w;
}

Hit64 trace64(const Scene& s, const float* of, const float* df, double tmin, double tmax) {
  Hit64 h;
  h.t = tmax;
  if (s.T == 0) return h;
  const double o[3] = {of[0], of[1], of[2]}, d[3] = {df[0], df[1], df[2]};
  double inv[3];
  for (int k = 0; k < 3; ++k) inv[k] = 1.0 / d[k];
  int32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const Scene::Node& n = s.nodes[stack[--sp]];
    double tn;
    if (!boxHit(n, o, inv, tmin, h.t * (1.0 + 1e-6), tn)) continue;
    if (n.left < 0) {
      for (uint32_t i = n.first; i < n.first + n.count; ++i) testMT(s, s.idx[i], o, d, tmin, h);
      continue;
    }
    stack[sp++] = n.left;
    stack[sp++] = n.right;
  }
  return h;
}

// Barycentric distance of ray (o, d) to the edges of triangle t, in double.
double edgeDistance(const Scene& s, uint32_t t, const float* of, const float* df) {
  const float* v = &s.v[9 * t];
  const double o[3] = {of[0], of[1], of[2]}, d[3] = {df[0], df[1], df[2]};
  const double e1[3] = {(double)v[3] - v[0], (double)v[4] - v[1], (double)v[5] - v[2]};
  const double e2[3] = {(double)v[6] - v[0], (double)v[7] - v[1], (double)v[8] - v[2]};
  const double p[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
  const double det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
  if (det == 0.0) return 0.0;
  const double inv = 1.0 / det;
  const double tv[3] = {o[0] - v[0], o[1] - v[1], o[2] - v[2]};
  const double u = (tv[0] * p[0] + tv[1] * p[1] + tv[2] * p[2]) * inv;
  const double q[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
  const double w = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) * inv;
  return std::min({std::fabs(u), std::fabs(w), std::fabs(1.0 - u - w)});
}

// ---------------------------------------------------------------------------
// Shading (lighting off).
// ---------------------------------------------------------------------------
// Bilinear texture lookup: wrap u to [0, 1] (frac), x = u * width - 0.5,
// first texel floor(x), weight A of the second = frac(x) in 1/256 steps
// rounded half up, both texel indices wrapped; the corner weights are the
// products of the axis weights rounded to 1/256 (ties to even) and the value
// sum(w * texel) / (256 * 255).  This restates the texture unit's documented
// bilinear rule with 8-bit fractional weights; on one-axis filtering it
// matches the unit's output to 2^-16, on two axes to a mean of about 2e-5.
void texAxis(float u, int n, int& i, int& A) {
  float f = u - std::floor(u);
  if (!(f >= 0.0f && f <= 1.0f)) f = 0.0f;
  const float xb = f * static_cast<float>(n) - 0.5f;
  const float fl = std::floor(xb);
  i = static_cast<int>(fl);
  A = static_cast<int>(std::floor((xb - fl) * 256.0f + 0.5f));
}

int wrapIndex(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

uint32_t div256Even(uint32_t x) {
  const uint32_t q = x >> 8, r = x & 255u;
  return q + ((r > 128u || (r == 128u && (q & 1u))) ? 1u : 0u);
}

void sampleTexture(const uint32_t* tx, int width, int height, float u, float v, float* rgba) {
  int i, j, A, B;
  texAxis(u, width, i, A);
  texAxis(v, height, j, B);
  const int i0 = wrapIndex(i, width), i1 = wrapIndex(i + 1, width);
  const int j0 = wrapIndex(j, height), j1 = wrapIndex(j + 1, height);
  const uint32_t T[4] = {tx[static_cast<size_t>(j0) * width + i0], tx[static_cast<size_t>(j0) * width + i1],
                         tx[static_cast<size_t>(j1) * width + i0], tx[static_cast<size_t>(j1) * width + i1]};
  const uint32_t a = static_cast<uint32_t>(A), b = static_cast<uint32_t>(B);
  const uint32_t w[4] = {div256Even((256u - a) * (256u - b)), div256Even(a * (256u - b)), div256Even((256u - a) * b),
                         div256Even(a * b)};
  for (int k = 0; k < 4; ++k) {
    uint32_t acc = 0;
    for (int q = 0; q < 4; ++q) acc += w[q] * ((T[q] >> (8 * k)) & 255u);
    rgba[k] = static_cast<float>(acc) / 65280.0f;
  }
}

V3 baseColour(const Scene& s, uint32_t t, float b1, float b2) {
  const float* c = &s.c[12 * t];
  if (!s.f[t]) return mk(c[0], c[1], c[2]);
  const float w0 = 1.0f - b1 - b2;
  if (s.f[t] == 2) {
    // UV = (1-b1-b2) UV0 + b1 UV1 + b2 UV2 (cuda/LocalGeometry.h:88-103).
    const float u = w0 * c[0] + b1 * c[4] + b2 * c[8];
    const float v = w0 * c[1] + b1 * c[5] + b2 * c[9];
    const int tex = static_cast<int>(c[2]);
    const int32_t* e = &s.texTable[3 * static_cast<size_t>(tex)];
    float rgba[4];
    sampleTexture(&s.texels[static_cast<size_t>(e[0])], e[1], e[2], u, v, rgba);
    return mk(std::pow(rgba[0], 2.2f), std::pow(rgba[1], 2.2f), std::pow(rgba[2], 2.2f));
  }
  const V3 C = mk(w0 * c[0] + b1 * c[4] + b2 * c[8], w0 * c[1] + b1 * c[5] + b2 * c[9], w0 * c[2] + b1 * c[6] + b2 * c[10]);
  return mk(std::pow(C.x, 2.2f), std::pow(C.y, 2.2f), std::pow(C.z, 2.2f));
}

Hit32 trace32(const Scene& s, const float* o, const float* d, float tmin, float tmax);

V3 vmul(V3 a, V3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }

// shaders.cu:67-90
V3 schlick(V3 spec, float VdH) {
  const float f = std::pow(1.0f - VdH, 5.0f);
  return add(spec, vmul(sub(mk(1, 1, 1), spec), mk(f, f, f)));
}
float smithVis(float NdL, float NdV, float alpha) {
  const float a2 = alpha * alpha;
  const float ggx0 = NdL * std::sqrt(NdV * NdV * (1.0f - a2) + a2);
  const float ggx1 = NdV * std::sqrt(NdL * NdL * (1.0f - a2) + a2);
  return 2.0f * NdL * NdV / (ggx0 + ggx1);
}
float ggxNormal(float NdH, float alpha) {
  const float a2 = alpha * alpha;
  const float x = NdH * NdH * (a2 - 1.0f) + 1.0f;
  return a2 / (kPi * x * x);
}

// Lighting-on shading of a hit with base colour `base` (shaders.cu:812-880).
V3 shadeLit(const Scene& s, uint32_t t, float b1, float b2, V3 dir, V3 base) {
  const float* L = &s.light[20 * static_cast<size_t>(t)];
  const float* v = &s.v[9 * static_cast<size_t>(t)];
  const V3 P0 = mk(v[0], v[1], v[2]), P1 = mk(v[3], v[4], v[5]), P2 = mk(v[6], v[7], v[8]);
  const float w0 = 1.0f - b1 - b2;
  const V3 P = add(add(scl(w0, P0), scl(b1, P1)), scl(b2, P2));
  const int flags = static_cast<int>(L[19]);
  V3 N = normalize(cross(sub(P1, P0), sub(P2, P0)));
  if (flags & 1)
    N = normalize(add(add(scl(w0, mk(L[0], L[1], L[2])), scl(b1, mk(L[3], L[4], L[5]))), scl(b2, mk(L[6], L[7], L[8]))));
  const float u0 = L[9], v0 = L[10], u1 = L[11], v1 = L[12], u2 = L[13], v2 = L[14];
  float U = b1, Vt = b2;
  if (flags & 2) {
    U = w0 * u0 + b1 * u1 + b2 * u2;
    Vt = w0 * v0 + b1 * v1 + b2 * v2;
  }
  float metallic = L[15], roughness = L[16];
  const int mrTex = static_cast<int>(L[17]), nTex = static_cast<int>(L[18]);
  auto sample = [&](int tex, float* rgba) {
    const int32_t* e = &s.texTable[3 * static_cast<size_t>(tex)];
    sampleTexture(&s.texels[static_cast<size_t>(e[0])], e[1], e[2], U, Vt, rgba);
  };
  if (mrTex >= 0) {
    float mr[4];
    sample(mrTex, mr);
    roughness *= mr[1];
    metallic *= mr[2];
  }
  const float F0 = 0.04f;
  const V3 diff = scl((1.0f - F0) * (1.0f - metallic), base);
  const V3 spec = add(mk(F0, F0, F0), scl(metallic, sub(base, mk(F0, F0, F0))));
  const float alpha = roughness * roughness;
  if (nTex >= 0) {
    float T[4];
    sample(nTex, T);
    const float du1 = u0 - u2, du2 = u1 - u2, dv1 = v0 - v2, dv2 = v1 - v2;
    const V3 dp1 = sub(P0, P2), dp2 = sub(P1, P2);
    const float invdet = 1.f / (du1 * dv2 - dv1 * du2);
    const V3 dpdu = scl(invdet, sub(scl(dv2, dp1), scl(dv1, dp2)));
    const V3 dpdv = scl(invdet, add(scl(-du2, dp1), scl(du1, dp2)));
    N = normalize(add(add(scl(2.0f * T[0] - 1.0f, normalize(dpdu)), scl(2.0f * T[1] - 1.0f, normalize(dpdv))),
                      scl(2.0f * T[2] - 1.0f, N)));
  }
  const V3 V = scl(-1.0f, normalize(dir));
  V3 result = mk(0, 0, 0);
  for (int i = 0; i < 4; ++i) {
    const V3 Lv = sub(mk(s.lightPos[i][0], s.lightPos[i][1], s.lightPos[i][2]), P);
    const float Ldist = std::sqrt(dot(Lv, Lv));
    const V3 Ld = scl(1.0f / Ldist, Lv);
    const V3 H = normalize(add(Ld, V));
    const float NdL = dot(N, Ld), NdV = dot(N, V), NdH = dot(N, H), VdH = dot(V, H);
    if (NdL > 0.0f && NdV > 0.0f) {
      const float o[3] = {P.x, P.y, P.z}, d[3] = {Ld.x, Ld.y, Ld.z};
      if (trace32(s, o, d, 0.001f, Ldist - 0.001f).id != 0xffffffffu) continue;
      const V3 F = schlick(spec, VdH);
      const float G = smithVis(NdL, NdV, alpha), D = ggxNormal(NdH, alpha);
      const V3 dterm = scl(1.0f / kPi, vmul(sub(mk(1, 1, 1), F), diff));
      const V3 sterm = scl(G * D, F);
      result = add(result, vmul(scl(s.lightPos[i][3] * NdL, mk(s.lightCol[i][0], s.lightCol[i][1], s.lightCol[i][2])),
                                add(dterm, sterm)));
    }
  }
  return result;
}

V3 shadeHit(const Scene& s, uint32_t t, float b1, float b2, V3 dir) {
  const V3 base = baseColour(s, t, b1, b2);
  return s.lighting ? shadeLit(s, t, b1, b2, dir, base) : base;
}

V3 shadeMiss(int miss, V3 dirIn) {
  const V3 dir = normalize(dirIn);
  if (miss == 1) {
    const float mix = std::min(std::max(0.0f, (std::asin(dir.y) * 2.0f) / kPi), 1.0f);
    const V3 upper = mk(1.0f / 255.0f, 31.0f / 255.0f, 117.0f / 255.0f);
    const V3 lower = mk(143.0f / 255.0f * 0.8f, 179.0f / 255.0f * 0.8f, 203.0f / 255.0f * 0.8f);
    return add(scl(1.0f - mix, lower), scl(mix, upper));
  }
  V3 c = mk((std::atan2(dir.z, dir.x) + kPi) / (kPi * 2.0f), (std::asin(dir.y) + kPi / 2.0f) / kPi, 0.0f);
  const float border = 0.01f;
  if (std::fabs(dir.x) < border || std::fabs(dir.y) < border || std::fabs(dir.z) < border) c = mk(0, 0, 0);
  return c;
}

// Ray of one sample (shaders.cu:652-709) from its two draws.
void genRay(const float* om, const float* pose, float nd, float ud, float* org, float* dir) {
  const V3 pos = mk(om[0], om[1], om[2]);
  const V3 axis = mk(om[3], om[4], om[5]);
  const float sd = om[6] / kFwhmSdRatio;
  const float splay = nd * sd;
  const float phi = ud * kPi;
  V3 perp = cross(mk(0.0f, 1.0f, 0.0f), axis);
  perp = (perp.x + perp.y + perp.z == 0.0f) ? mk(0.0f, 0.0f, 1.0f) : normalize(perp);
  const V3 splayed = rotatePoint(axis, splay, perp);
  const V3 rel = rotatePoint(splayed, phi, axis);
  const V3 relPos = sub(pos, scl(om[7], normalize(axis)));
  const V3 P = mk(pose[0], pose[1], pose[2]);
  const V3 X = mk(pose[3], pose[4], pose[5]), Y = mk(pose[6], pose[7], pose[8]), Z = mk(pose[9], pose[10], pose[11]);
  const V3 o = add(add(add(P, scl(relPos.x, X)), scl(relPos.y, Y)), scl(relPos.z, Z));
  const V3 d = add(add(scl(rel.x, X), scl(rel.y, Y)), scl(rel.z, Z));
  org[0] = o.x;
  org[1] = o.y;
  org[2] = o.z;
  dir[0] = d.x;
  dir[1] = d.y;
  dir[2] = d.z;
}

void setThreads(int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
}

}  // namespace

extern "C" {

// Base colour textures of a scene: the texels of all textures and per
// texture (first texel, width, height).
// Lighting-on data: 20 floats per triangle (original order), four lights
// as position xyz + intensity (16 floats) and colour (12 floats); on != 0
// switches the lit shading on.
void orc_scene_set_lighting(void* h, const float* light, const float* lightPos, const float* lightCol, int on) {
  Scene* s = static_cast<Scene*>(h);
  s->light.assign(light, light + 20 * static_cast<size_t>(s->T));
  for (int i = 0; i < 4; ++i) {
    for (int k = 0; k < 4; ++k) s->lightPos[i][k] = lightPos[4 * i + k];
    for (int k = 0; k < 3; ++k) s->lightCol[i][k] = lightCol[3 * i + k];
  }
  s->lighting = on;
}

void orc_scene_set_textures(void* h, const uint32_t* texels, size_t nTexels, const int32_t* table, uint32_t nTex) {
  Scene* s = static_cast<Scene*>(h);
  s->texels.assign(texels, texels + nTexels);
  s->texTable.assign(table, table + 3 * static_cast<size_t>(nTex));
}

// n lookups of one texture at (u, v) pairs: n x 4 floats.
void orc_sample_texture(const uint32_t* texels, int width, int height, const float* uv, size_t n, float* rgba) {
  for (size_t i = 0; i < n; ++i) sampleTexture(texels, width, height, uv[2 * i], uv[2 * i + 1], rgba + 4 * i);
}

void* orc_scene_create(const float* verts, const float* colours, const uint8_t* flags, uint32_t T) {
  Scene* s = new Scene;
  s->T = T;
  s->v.assign(verts, verts + 9 * static_cast<size_t>(T));
  s->c.assign(colours, colours + 12 * static_cast<size_t>(T));
  s->f.assign(flags, flags + T);
  if (T) {
    s->idx.resize(T);
    std::vector<double> cen(3 * static_cast<size_t>(T));
    for (uint32_t t = 0; t < T; ++t) {
      s->idx[t] = t;
      double lo[3], hi[3];
      boxOf(*s, t, lo, hi);
      for (int k = 0; k < 3; ++k) cen[3 * t + k] = 0.5 * (lo[k] + hi[k]);
    }
    s->nodes.reserve(2 * static_cast<size_t>(T) / 2 + 8);
    buildNode(*s, 0, T, cen);
  }
  return s;
}

void orc_scene_destroy(void* sc) { delete static_cast<Scene*>(sc); }

// Float watertight closest hit of n rays: hit id (-1 = miss), t, and the
// barycentrics b1 = V/det, b2 = W/det of the hit.
void orc_trace(void* sc, const float* org, const float* dir, const float* tmin, float tmax, size_t n, int32_t* hitId,
               float* t, float* b1, float* b2, int threads) {
  const Scene& s = *static_cast<Scene*>(sc);
  setThreads(threads);
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < static_cast<long long>(n); ++i) {
    const Hit32 h = trace32(s, org + 3 * i, dir + 3 * i, tmin[i], tmax);
    if (h.id == 0xffffffffu) {
      hitId[i] = -1;
      t[i] = -1.0f;
      b1[i] = b2[i] = 0.0f;
    } else {
      hitId[i] = static_cast<int32_t>(h.id);
      t[i] = h.t;
      b1[i] = h.V / h.det;
      b2[i] = h.W / h.det;
    }
  }
}

// Double-precision closest hit of n rays, and for each ray the smallest
// barycentric distance to an edge of the float hit (when given) and of the
// double hit.
void orc_trace_f64(void* sc, const float* org, const float* dir, const float* tmin, double tmax, size_t n,
                   const int32_t* hit32, int32_t* hitId, double* t, double* edge32, double* edge64, int threads) {
  const Scene& s = *static_cast<Scene*>(sc);
  setThreads(threads);
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < static_cast<long long>(n); ++i) {
    const Hit64 h = trace64(s, org + 3 * i, dir + 3 * i, tmin[i], tmax);
    hitId[i] = h.id < 0 ? -1 : static_cast<int32_t>(h.id);
    t[i] = h.id < 0 ? -1.0 : h.t;
    edge64[i] = h.id < 0 ? INFINITY : edgeDistance(s, static_cast<uint32_t>(h.id), org + 3 * i, dir + 3 * i);
    edge32[i] = (hit32 && hit32[i] >= 0) ? edgeDistance(s, static_cast<uint32_t>(hit32[i]), org + 3 * i, dir + 3 * i)
                                         : INFINITY;
  }
}

// Shaded colour of n rays given their hits (id -1 = miss, shaded by `miss`).
void orc_shade(void* sc, int miss, const float* dir, const int32_t* hitId, const float* b1, const float* b2, size_t n,
               float* rgb) {
  const Scene& s = *static_cast<Scene*>(sc);
  for (size_t i = 0; i < n; ++i) {
    const V3 d = mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    const V3 c = hitId[i] >= 0 ? shadeHit(s, static_cast<uint32_t>(hitId[i]), b1[i], b2[i], d) : shadeMiss(miss, d);
    rgb[3 * i] = c.x;
    rgb[3 * i + 1] = c.y;
    rgb[3 * i + 2] = c.z;
  }
}

// Rays of N*spp samples (ommatidium-major) at one pose from their draws
// (2 floats per sample: normal, uniform).  omm: N x 8 floats.
void orc_gen_rays(const float* omm, uint32_t N, uint32_t spp, const float* pose12, const float* draws, float* org,
                  float* dir) {
  for (size_t o = 0; o < N; ++o)
    for (size_t k = 0; k < spp; ++k) {
      const size_t i = o * spp + k;
      genRay(omm + 8 * o, pose12, draws[2 * i], draws[2 * i + 1], org + 3 * i, dir + 3 * i);
    }
}

// Per-ommatidium sums of given rays (P poses x N x spp, ommatidium-major per
// pose): trace, shade, scale by 1/spp and add in sample order.
void orc_render_rays(void* sc, int miss, const float* omm, uint32_t N, uint32_t spp, uint32_t P, const float* org,
                     const float* dir, float* out, int threads) {
  const Scene& s = *static_cast<Scene*>(sc);
  setThreads(threads);
  const float scale = 1.0f / static_cast<float>(spp);
#pragma omp parallel for schedule(dynamic, 1)
  for (long long po = 0; po < static_cast<long long>(P) * N; ++po) {
    const uint32_t o = static_cast<uint32_t>(po % N);
    const float tmin = omm[8 * o + 7];
    V3 sum = mk(0, 0, 0);
    for (uint32_t k = 0; k < spp; ++k) {
      const size_t i = static_cast<size_t>(po) * spp + k;
      const Hit32 h = trace32(s, org + 3 * i, dir + 3 * i, tmin, 1e16f);
      const V3 d = mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
      const V3 c = h.id != 0xffffffffu ? shadeHit(s, h.id, h.V / h.det, h.W / h.det, d) : shadeMiss(miss, d);
      sum = add(sum, scl(scale, c));
    }
    out[3 * po] = sum.x;
    out[3 * po + 1] = sum.y;
    out[3 * po + 2] = sum.z;
  }
}

// The whole path on the CPU from draws: P poses (12 floats each), draws of
// P x N x spp samples (2 floats each).  out: P x N x 3 sums.  Returns the
// number of rays traced.
size_t orc_render_draws(void* sc, int miss, const float* omm, uint32_t N, uint32_t spp, uint32_t P,
                        const float* poses12, const float* draws, float* out, int threads) {
  const Scene& s = *static_cast<Scene*>(sc);
  setThreads(threads);
  const float scale = 1.0f / static_cast<float>(spp);
#pragma omp parallel for schedule(dynamic, 1)
  for (long long po = 0; po < static_cast<long long>(P) * N; ++po) {
    const uint32_t p = static_cast<uint32_t>(po / N), o = static_cast<uint32_t>(po % N);
    const float tmin = omm[8 * o + 7];
    V3 sum = mk(0, 0, 0);
    for (uint32_t k = 0; k < spp; ++k) {
      const size_t i = static_cast<size_t>(po) * spp + k;
      float org[3], dir[3];
      genRay(omm + 8 * o, poses12 + 12 * p, draws[2 * i], draws[2 * i + 1], org, dir);
      const Hit32 h = trace32(s, org, dir, tmin, 1e16f);
      const V3 d = mk(dir[0], dir[1], dir[2]);
      const V3 c = h.id != 0xffffffffu ? shadeHit(s, h.id, h.V / h.det, h.W / h.det, d) : shadeMiss(miss, d);
      sum = add(sum, scl(scale, c));
    }
    out[3 * po] = sum.x;
    out[3 * po + 1] = sum.y;
    out[3 * po + 2] = sum.z;
  }
  return static_cast<size_t>(P) * N * spp;
}

// make_color (shaders.cu:180-189) of n RGB sums into n RGBA bytes.
void orc_make_color(const float* sums, size_t n, uint8_t* out) {
  const float invGamma = static_cast<float>(1.0 / static_cast<double>(2.2f));
  for (size_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) {
      const float c = std::min(std::max(sums[3 * i + k], 0.0f), 1.0f);
      out[4 * i + k] = static_cast<uint8_t>(std::pow(c, invGamma) * 255.0f);
    }
    out[4 * i + 3] = 255;
  }
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
