// Two-wide bounding volume hierarchy built on the host with binned SAH.
//
// Device layout (all little-endian, 16-byte aligned):
//   node i = 4 x float4 (64 B), child boxes as centre c and half-extent e
//   with [c - e, c + e] containing the exact box:
//     [0] = (c0.cx, c0.cy, c0.cz, c0.ex)
//     [1] = (c0.ey, c0.ez, c1.cx, c1.cy)
//     [2] = (c1.cz, c1.ex, c1.ey, c1.ez)
//     [3] = (int child0, int child1, 0, 0)
//   child >= 0 is an inner node index; child < 0 is a leaf whose bitwise
//   complement packs (first triangle << 3) | (count - 1), count in 1..8.
//   triangle j (BVH order) = 3 x float4: (v0, id) (v1, 0) (v2, 0) where id is
//   the original global triangle id stored as integer bits.
//   shade j = the triangle's 3 x float4 colour record (material colour,
//   vertex colours, or (u, v, texture, 0) per vertex) with c0.w replaced by
//   the shading kind as a float: 0 base colour, 1 vertex colours, 2 texture.
// Node 0 is the root and is always an inner node.
#pragma once

#include <cstdint>
#include <vector>

namespace cr {

struct BvhBuildStats {
  uint32_t innerNodes = 0;
  uint32_t leaves = 0;
  uint32_t maxDepth = 0;
  double sahCost = 0.0;
};

struct HostBvh {
  std::vector<float> nodes;   // 16 floats per node
  std::vector<float> tris;    // 12 floats per triangle, BVH order
  std::vector<float> shade;   // 12 floats per triangle, BVH order
  std::vector<uint32_t> order;  // BVH position -> original triangle id
  BvhBuildStats stats;
};

// verts: 9 floats per triangle (world space); colours: 12 floats per triangle;
// shading: 1 byte per triangle (the scene's kShade* kind).
void buildBvh(const float* verts, const float* colours, const uint8_t* shading, uint32_t triCount,
              HostBvh& out);

constexpr int kMaxLeafSize = 8;

}  // namespace cr
