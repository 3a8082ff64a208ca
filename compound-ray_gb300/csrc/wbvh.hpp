// Wide bounding volume hierarchy: 4 or 8 children per node with 8-bit
// quantised child boxes, collapsed from the two-wide BVH (bvh.hpp layout).
//
// Device layout of wide node i (little-endian, 16-byte aligned float4s):
//   [0] = (px, py, pz, meta): the quantisation origin, and meta = ex | ey << 8
//         | ez << 16 | count << 24 with e* the biased (IEEE float) exponents of
//         the per-axis scales s* = 2^(e* - 127) and count the children (2..W)
//   W = 4 (4 float4, 64 B):
//     [1] = (lo.x, lo.y, lo.z, hi.x)   [2] = (hi.y, hi.z, 0, 0)   [3] = children 0-3
//   W = 8 (6 float4, 96 B):
//     [1] = (lo.x[0-3], lo.x[4-7], lo.y[0-3], lo.y[4-7])
//     [2] = (lo.z[0-3], lo.z[4-7], hi.x[0-3], hi.x[4-7])
//     [3] = (hi.y[0-3], hi.y[4-7], hi.z[0-3], hi.z[4-7])
//     [4] = children 0-3              [5] = children 4-7
//   where lo.x[0-3] is one 32-bit word holding the lower x plane of children
//   0..3 as bytes (child k in byte k).  Child k's box along axis a is
//   [p_a + lo_a[k] * s_a, p_a + hi_a[k] * s_a], which contains the child's
//   exact box (bytes rounded outward in exact arithmetic).  Child refs use
//   the two-wide BVH's encoding: >= 0 a wide node, < 0 the complement of
//   (first triangle << 3) | (count - 1) of a leaf in the shared triangle
//   arrays.  Node 0 is the root.
#pragma once

#include <cstdint>
#include <vector>

namespace cr {

struct WideBvhStats {
  uint32_t nodes = 0;
  uint32_t maxDepth = 0;
  double meanChildren = 0.0;
};

// Float4s per wide node of width W (4 or 8).
inline uint32_t wideNodeFloat4s(int W) { return W == 8 ? 6u : 4u; }

// Collapses the two-wide BVH (nodes: 16 floats per inner node; tris: 12
// floats per triangle in leaf order, vertices in floats 0-2, 4-6, 8-10)
// into a W-wide one (W = 4 or 8): every wide node takes its two-wide node's
// children and repeatedly opens the inner child of largest surface area
// until it has W children or only leaves are left.  out: wide nodes as
// floats, wideNodeFloat4s(W) * 4 per node.
void collapseWideBvh(const float* nodes, uint32_t innerNodes, const float* tris, uint32_t triCount, int W,
                     std::vector<float>& out, WideBvhStats& stats);

}  // namespace cr
