// GPU BVH construction for the compound-eye renderer (linear BVH).
//
// Builds, on the device, the same BVH2 layout the render kernel traverses
// (bvh.hpp) from world-space triangles, replacing the reference's OptiX
// acceleration-structure builds (libEyeRenderer3/MulticamScene.cpp:1052-1428):
//   1. 63-bit Morton codes (21 bits per axis) of the triangle centroids in
//      the centroid bounds' cube;
//   2. an LSD radix sort of (code, triangle) pairs, 8-bit digits, stable;
//   3. the binary radix tree of Karras ("Maximizing Parallelism in the
//      Construction of BVHs, Octrees, and k-d Trees", HPG 2012): internal
//      node i covers a contiguous range of sorted triangles, equal codes are
//      split by position;
//   4. bottom-up boxes and surface-area costs, one thread per leaf, the
//      second thread to reach a node builds its box and cost; a node of at
//      most kLbvhLeaf triangles becomes a leaf when that is cheaper under
//      the host builder's cost model (bvh.cpp: 1.2 per node, 1 per triangle);
//   5. the node array and the leaf-ordered triangle and shading arrays are
//      written out (a leaf's triangles are contiguous in sorted order).
// Internal node 0 is the root; node slots inside leaves stay unused.
#include <cuda_runtime.h>

#include <cstdint>

#include "device_api.hpp"

namespace cr {
namespace {

constexpr uint32_t kLbvhLeaf = 8;  // largest leaf (the render layout's 3-bit count)
constexpr float kLbvhCostNode = 1.2f, kLbvhCostTri = 1.0f;
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kRadix = 256;

// Spreads the low 21 bits of v to every third bit.
__device__ __forceinline__ uint64_t expandBits(uint64_t v) {
  v &= 0x1FFFFFull;
  v = (v | (v << 32)) & 0x001F00000000FFFFull;
  v = (v | (v << 16)) & 0x001F0000FF0000FFull;
  v = (v | (v << 8)) & 0x100F00F00F00F00Full;
  v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

__global__ void mortonKernel(const float* __restrict__ verts, uint32_t T, float3 lo, float3 scale,
                             uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const float* v = verts + 9 * static_cast<size_t>(t);
  float c[3];
  for (int k = 0; k < 3; ++k) {
    const float a = fminf(fminf(v[k], v[3 + k]), v[6 + k]);
    const float b = fmaxf(fmaxf(v[k], v[3 + k]), v[6 + k]);
    c[k] = 0.5f * a + 0.5f * b;
  }
  const float q[3] = {(c[0] - lo.x) * scale.x, (c[1] - lo.y) * scale.y, (c[2] - lo.z) * scale.z};
  uint64_t m[3];
  for (int k = 0; k < 3; ++k) m[k] = static_cast<uint64_t>(fminf(fmaxf(q[k], 0.0f), 2097151.0f));
  keys[t] = (expandBits(m[0]) << 2) | (expandBits(m[1]) << 1) | expandBits(m[2]);
  vals[t] = t;
}

// Radix sort pass 1: per-tile digit counts, stored digit-major
// (hist[d * tiles + tile]) so one exclusive scan gives global offsets.
__global__ void radixCountKernel(const uint64_t* __restrict__ keys, uint32_t n, int shift, uint32_t tiles,
                                 uint32_t* __restrict__ hist) {
  __shared__ uint32_t cnt[kRadix];
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) cnt[d] = 0;
  __syncthreads();
  const size_t base = static_cast<size_t>(blockIdx.x) * kSortTile;
  for (int r = 0; r < kSortItems; ++r) {
    const size_t i = base + static_cast<size_t>(r) * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[static_cast<uint32_t>(keys[i] >> shift) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x) hist[static_cast<size_t>(d) * tiles + blockIdx.x] = cnt[d];
}

// Exclusive scan of `count` words in place by one block (tiled).
__global__ void scanKernel(uint32_t* data, uint32_t count) {
  __shared__ uint32_t part[1024];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < count; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < count ? data[i] : 0u;
    part[threadIdx.x] = v;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {
      const uint32_t add = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
      __syncthreads();
      part[threadIdx.x] += add;
      __syncthreads();
    }
    if (i < count) data[i] = carry + part[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += part[1023];
    __syncthreads();
  }
}

// Radix sort pass 2: stable scatter.  The tile is processed in kSortItems
// rounds of one key per thread, in order; within a round a key's rank is the
// number of equal digits before it (earlier warps, then earlier lanes).
__global__ void radixScatterKernel(const uint64_t* __restrict__ keysIn, const uint32_t* __restrict__ valsIn,
                                   uint32_t n, int shift, uint32_t tiles, const uint32_t* __restrict__ offsets,
                                   uint64_t* __restrict__ keysOut, uint32_t* __restrict__ valsOut) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ uint32_t run[kRadix];            // keys of this digit already placed by this tile
  __shared__ uint32_t warpCnt[kWarps][kRadix];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int d = threadIdx.x; d < kRadix; d += blockDim.x)
    run[d] = offsets[static_cast<size_t>(d) * tiles + blockIdx.x];
  const size_t base = static_cast<size_t>(blockIdx.x) * kSortTile;
  for (int r = 0; r < kSortItems; ++r) {
    for (int k = threadIdx.x; k < kWarps * kRadix; k += blockDim.x) (&warpCnt[0][0])[k] = 0;
    __syncthreads();
    const size_t i = base + static_cast<size_t>(r) * kSortThreads + threadIdx.x;
    const bool ok = i < n;
    const uint64_t key = ok ? keysIn[i] : 0ull;
    const uint32_t d = ok ? static_cast<uint32_t>((key >> shift) & (kRadix - 1)) : kRadix;  // kRadix = no digit
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t before = __popc(peers & ((1u << lane) - 1u));
    if (ok && before == 0) warpCnt[warp][d] = __popc(peers);
    __syncthreads();
    // Exclusive prefix over warps, per digit, and advance the running base.
    for (int dd = threadIdx.x; dd < kRadix; dd += blockDim.x) {
      uint32_t acc = run[dd];
      for (int w = 0; w < kWarps; ++w) {
        const uint32_t c = warpCnt[w][dd];
        warpCnt[w][dd] = acc;
        acc += c;
      }
      run[dd] = acc;
    }
    __syncthreads();
    if (ok) {
      const uint32_t dst = warpCnt[warp][d] + before;
      keysOut[dst] = key;
      valsOut[dst] = valsIn[i];
    }
    __syncthreads();
  }
}

__device__ __forceinline__ int delta(const uint64_t* __restrict__ k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint64_t a = k[i], b = k[j];
  if (a != b) return __clzll(static_cast<long long>(a ^ b));
  return 64 + __clz(static_cast<uint32_t>(i) ^ static_cast<uint32_t>(j));
}

// Karras hierarchy.  Node ids: internal 0..n-2, leaf g -> n-1+g.
__global__ void hierarchyKernel(const uint64_t* __restrict__ keys, int n, int* __restrict__ left,
                                int* __restrict__ right, int* __restrict__ parent, int* __restrict__ first,
                                int* __restrict__ last) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = delta(keys, n, i, j);
  int s = 0;
  int step = l;
  do {
    step = (step + 1) >> 1;
    if (delta(keys, n, i, i + (s + step) * d) > dnode) s += step;
  } while (step > 1);
  const int g = i + s * d + (d < 0 ? -1 : 0);
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  const int lc = (lo == g) ? (n - 1 + g) : g;
  const int rc = (hi == g + 1) ? (n - 1 + g + 1) : (g + 1);
  left[i] = lc;
  right[i] = rc;
  parent[lc] = i;
  parent[rc] = i;
  first[i] = lo;
  last[i] = hi;
}

__device__ __forceinline__ float halfArea(const volatile float* b) {
  const float dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
  return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ int count(int node, int n, const int* first, const int* last) {
  return node >= n - 1 ? 1 : last[node] - first[node] + 1;
}

// Bottom-up boxes and costs.  boxes: 6 floats per node id (lo xyz, hi xyz);
// cost: surface-area cost of the node's subtree (half area times the
// expected work); leafy[i] = 1 when inner node i is cheaper as a leaf.  Each
// leaf thread climbs; the first thread to reach a node stops there, the
// second (which sees both children finished) builds the box and cost and
// continues.
__global__ void boxesKernel(const float* __restrict__ verts, const uint32_t* __restrict__ order, int n,
                            const int* __restrict__ left, const int* __restrict__ right,
                            const int* __restrict__ parent, const int* __restrict__ first,
                            const int* __restrict__ last, float* boxes, float* cost, uint8_t* leafy,
                            unsigned* visits) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const float* v = verts + 9 * static_cast<size_t>(order[g]);
  float* b = boxes + 6 * static_cast<size_t>(n - 1 + g);
  for (int k = 0; k < 3; ++k) {
    b[k] = fminf(fminf(v[k], v[3 + k]), v[6 + k]);
    b[3 + k] = fmaxf(fmaxf(v[k], v[3 + k]), v[6 + k]);
  }
  cost[n - 1 + g] = kLbvhCostTri * halfArea(b);
  int node = parent[n - 1 + g];
  while (node >= 0) {
    __threadfence();
    if (atomicAdd(&visits[node], 1u) == 0u) return;
    __threadfence();
    const int l = left[node], r = right[node];
    const volatile float* a = boxes + 6 * static_cast<size_t>(l);
    const volatile float* c = boxes + 6 * static_cast<size_t>(r);
    float* o = boxes + 6 * static_cast<size_t>(node);
    for (int k = 0; k < 3; ++k) {
      o[k] = fminf(a[k], c[k]);
      o[3 + k] = fmaxf(a[3 + k], c[3 + k]);
    }
    const float area = halfArea(o);
    const volatile float* cv = cost;
    const float split = kLbvhCostNode * area + cv[l] + cv[r];
    const int cnt = count(node, n, first, last);
    const float asLeaf = kLbvhCostTri * static_cast<float>(cnt) * area;
    const bool leaf = node != 0 && cnt <= static_cast<int>(kLbvhLeaf) && asLeaf <= split;
    leafy[node] = leaf ? 1 : 0;
    cost[node] = leaf ? asLeaf : split;
    if (node == 0) return;
    node = parent[node];
  }
}

// True when inner node i lies inside a leaf: it or an ancestor of at most
// kLbvhLeaf triangles was made a leaf.
__device__ __forceinline__ bool insideLeaf(int i, int n, const int* parent, const int* first, const int* last,
                                          const uint8_t* leafy) {
  for (int a = i; a > 0 && count(a, n, first, last) <= static_cast<int>(kLbvhLeaf); a = parent[a])
    if (leafy[a]) return true;
  return false;
}

__device__ __forceinline__ void centreExtent(const float* b, float* c, float* e) {
  for (int k = 0; k < 3; ++k) {
    c[k] = 0.5f * b[k] + 0.5f * b[3 + k];
    const double need = fmax(static_cast<double>(b[3 + k]) - c[k], static_cast<double>(c[k]) - b[k]);
    e[k] = __double2float_ru(need);
  }
}

// Child reference in the render layout: inner node index, or leaf code.
// Called for the children of emitted nodes only, so a child made a leaf is
// the top of its leaf.
__device__ __forceinline__ int childRef(int c, int n, const int* first, const int* last, const uint8_t* leafy) {
  if (c >= n - 1) return ~static_cast<int>((static_cast<uint32_t>(c - (n - 1)) << 3) | 0u);
  const int cnt = last[c] - first[c] + 1;
  if (leafy[c]) return ~static_cast<int>((static_cast<uint32_t>(first[c]) << 3) | static_cast<uint32_t>(cnt - 1));
  return c;
}

__global__ void emitNodesKernel(int n, const int* __restrict__ left, const int* __restrict__ right,
                                const int* __restrict__ parent, const int* __restrict__ first,
                                const int* __restrict__ last, const uint8_t* __restrict__ leafy,
                                const float* __restrict__ boxes, float4* __restrict__ nodes, unsigned* stats) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  if (insideLeaf(i, n, parent, first, last, leafy)) return;
  const int l = left[i], r = right[i];
  float ca[3], ea[3], cb[3], eb[3];
  centreExtent(boxes + 6 * static_cast<size_t>(l), ca, ea);
  centreExtent(boxes + 6 * static_cast<size_t>(r), cb, eb);
  const int rl = childRef(l, n, first, last, leafy), rr = childRef(r, n, first, last, leafy);
  float4* o = nodes + 4 * static_cast<size_t>(i);
  o[0] = make_float4(ca[0], ca[1], ca[2], ea[0]);
  o[1] = make_float4(ea[1], ea[2], cb[0], cb[1]);
  o[2] = make_float4(cb[2], eb[0], eb[1], eb[2]);
  o[3] = make_float4(__int_as_float(rl), __int_as_float(rr), 0.f, 0.f);
  atomicAdd(&stats[0], 1u);
  atomicAdd(&stats[1], (rl < 0 ? 1u : 0u) + (rr < 0 ? 1u : 0u));
}

// Depth (in inner nodes above it) of every emitted leaf reference: from
// Karras leaf g, skip the nodes inside the leaf that holds it (below its
// topmost ancestor made a leaf), then count the emitted ancestors.
__global__ void depthKernel(int n, const int* __restrict__ parent, const int* __restrict__ first,
                            const int* __restrict__ last, const uint8_t* __restrict__ leafy, unsigned* stats) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  int top = -1;
  for (int a = parent[n - 1 + g]; a > 0 && count(a, n, first, last) <= static_cast<int>(kLbvhLeaf); a = parent[a])
    if (leafy[a]) top = a;
  int node = top >= 0 ? parent[top] : parent[n - 1 + g];
  unsigned depth = 0;
  while (node >= 0) {
    ++depth;
    node = node == 0 ? -1 : parent[node];
  }
  atomicMax(&stats[2], depth);
}

__global__ void gatherKernel(const float* __restrict__ verts, const float* __restrict__ colours,
                             const uint8_t* __restrict__ flags, const uint32_t* __restrict__ order, uint32_t T,
                             float4* __restrict__ tris, float4* __restrict__ shade) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= T) return;
  const uint32_t t = order[p];
  const float* v = verts + 9 * static_cast<size_t>(t);
  const float* c = colours + 12 * static_cast<size_t>(t);
  tris[3 * static_cast<size_t>(p)] = make_float4(v[0], v[1], v[2], __uint_as_float(t));
  tris[3 * static_cast<size_t>(p) + 1] = make_float4(v[3], v[4], v[5], 0.f);
  tris[3 * static_cast<size_t>(p) + 2] = make_float4(v[6], v[7], v[8], 0.f);
  shade[3 * static_cast<size_t>(p)] = make_float4(c[0], c[1], c[2], static_cast<float>(flags[t]));
  shade[3 * static_cast<size_t>(p) + 1] = make_float4(c[4], c[5], c[6], c[7]);
  shade[3 * static_cast<size_t>(p) + 2] = make_float4(c[8], c[9], c[10], c[11]);
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

size_t lbvhTempBytes(uint32_t T) {
  const size_t n = T;
  const size_t tiles = (n + kSortTile - 1) / kSortTile;
  size_t b = 0;
  b += 2 * align256(n * 8);                    // keys, keysAlt
  b += 2 * align256(n * 4);                    // vals, valsAlt
  b += align256(tiles * kRadix * 4);           // histogram
  b += 5 * align256(2 * n * 4);                // left, right, parent, first, last (over-sized)
  b += align256(2 * n * 6 * 4);                // boxes of all node ids
  b += align256(2 * n * 4);                    // costs of all node ids
  b += align256(n);                            // leaf flags of the inner nodes
  b += align256(n * 4);                        // visit counters
  b += align256(16);                           // stats
  return b;
}

cudaError_t buildLbvh(const float* d_verts, const float* d_colours, const uint8_t* d_flags, uint32_t T,
                      const float* centroidLo, const float* centroidHi, float4* d_nodes, float4* d_tris,
                      float4* d_shade, void* d_temp, uint32_t* statsOut, cudaStream_t stream) {
  if (T < 9) return cudaErrorInvalidValue;  // tiny scenes use the host builder
  const size_t n = T;
  const uint32_t tiles = static_cast<uint32_t>((n + kSortTile - 1) / kSortTile);
  char* p = static_cast<char*>(d_temp);
  auto take = [&](size_t bytes) {
    char* q = p;
    p += align256(bytes);
    return q;
  };
  uint64_t* keys = reinterpret_cast<uint64_t*>(take(n * 8));
  uint32_t* vals = reinterpret_cast<uint32_t*>(take(n * 4));
  uint64_t* keys2 = reinterpret_cast<uint64_t*>(take(n * 8));
  uint32_t* vals2 = reinterpret_cast<uint32_t*>(take(n * 4));
  uint32_t* hist = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(tiles) * kRadix * 4));
  int* left = reinterpret_cast<int*>(take(2 * n * 4));
  int* right = reinterpret_cast<int*>(take(2 * n * 4));
  int* parent = reinterpret_cast<int*>(take(2 * n * 4));
  int* first = reinterpret_cast<int*>(take(2 * n * 4));
  int* last = reinterpret_cast<int*>(take(2 * n * 4));
  float* boxes = reinterpret_cast<float*>(take(2 * n * 6 * 4));
  float* cost = reinterpret_cast<float*>(take(2 * n * 4));
  uint8_t* leafy = reinterpret_cast<uint8_t*>(take(n));
  unsigned* visits = reinterpret_cast<unsigned*>(take(n * 4));
  unsigned* stats = reinterpret_cast<unsigned*>(take(16));

  float3 lo = make_float3(centroidLo[0], centroidLo[1], centroidLo[2]);
  float3 sc;
  const float ext[3] = {centroidHi[0] - centroidLo[0], centroidHi[1] - centroidLo[1], centroidHi[2] - centroidLo[2]};
  // One scale for all axes (the bounding cube): a flat scene then spends its
  // top-level splits on its long axes instead of cutting its thin axis as
  // often as the others, which would make sibling boxes overlap.
  const float big = fmaxf(fmaxf(ext[0], ext[1]), ext[2]);
  const float s = big > 0.f ? 2097151.0f / big : 0.f;
  sc.x = sc.y = sc.z = s;
  const unsigned g = static_cast<unsigned>((n + 255) / 256);
  mortonKernel<<<g, 256, 0, stream>>>(d_verts, T, lo, sc, keys, vals);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  uint64_t *kin = keys, *kout = keys2;
  uint32_t *vin = vals, *vout = vals2;
  for (int shift = 0; shift < 63; shift += 8) {
    radixCountKernel<<<tiles, kSortThreads, 0, stream>>>(kin, T, shift, tiles, hist);
    scanKernel<<<1, 1024, 0, stream>>>(hist, tiles * kRadix);
    radixScatterKernel<<<tiles, kSortThreads, 0, stream>>>(kin, vin, T, shift, tiles, hist, kout, vout);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint64_t* tk = kin;
    kin = kout;
    kout = tk;
    uint32_t* tv = vin;
    vin = vout;
    vout = tv;
  }
  e = cudaMemsetAsync(parent, 0xff, 2 * n * 4, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(visits, 0, n * 4, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(stats, 0, 16, stream);
  if (e != cudaSuccess) return e;
  const unsigned gi = static_cast<unsigned>((n - 1 + 255) / 256);
  hierarchyKernel<<<gi, 256, 0, stream>>>(kin, static_cast<int>(n), left, right, parent, first, last);
  boxesKernel<<<g, 256, 0, stream>>>(d_verts, vin, static_cast<int>(n), left, right, parent, first, last, boxes, cost,
                                     leafy, visits);
  emitNodesKernel<<<gi, 256, 0, stream>>>(static_cast<int>(n), left, right, parent, first, last, leafy, boxes, d_nodes,
                                          stats);
  depthKernel<<<g, 256, 0, stream>>>(static_cast<int>(n), parent, first, last, leafy, stats);
  gatherKernel<<<g, 256, 0, stream>>>(d_verts, d_colours, d_flags, vin, T, d_tris, d_shade);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(statsOut, stats, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(stream);
}

}  // namespace cr
