// Test infrastructure (checker only): a C entry point around the reference's
// own point-in-mesh test, sutil/hitscanprocessing.cpp:20-83
// (sutil::hitscan::isPointWithinMesh), compiled unchanged from the reference
// checkout by oracle/build_ref.py into oracle/_ref/libref_hitscan.so.
//
// The reference keeps one TriangleMesh per glTF hitbox node with the node's
// float 4x4 transform and the object-space triangles
// (libEyeRenderer3/MulticamScene.cpp:329-344), computes the object box once
// (calculateObjectAabb, hitscanprocessing.cpp:87-101) and answers
// isInsideHitGeometry with isPointWithinMesh (MulticamScene.cpp:1755-1791).
// This driver builds that mesh from plain arrays and asks it about many
// points.  Nothing in the library links or loads it.
#include <cstddef>
#include <cstdint>

#include "sutil/hitscanprocessing.h"

extern "C" {

// tris: nTris x 9 floats (p0, p1, p2, object space); xform: row-major 4x4
// float node transform; pts: n x 3 world points; out: n bytes, 1 = inside.
// Returns 0, or -1 when the mesh has no triangle.
int ref_points_in_mesh(const float* tris, size_t nTris, const float* xform, const float* pts, size_t n,
                       uint8_t* out) {
  if (nTris == 0) return -1;
  sutil::hitscan::TriangleMesh tm;
  tm.name = "hitbox";
  tm.transform = sutil::Matrix4x4(xform);
  tm.triangles.reserve(nTris);
  for (size_t t = 0; t < nTris; ++t) {
    const float* v = tris + 9 * t;
    tm.triangles.push_back({make_float3(v[0], v[1], v[2]), make_float3(v[3], v[4], v[5]), make_float3(v[6], v[7], v[8])});
  }
  sutil::hitscan::calculateObjectAabb(tm);
  for (size_t k = 0; k < n; ++k)
    out[k] = sutil::hitscan::isPointWithinMesh(tm, make_float3(pts[3 * k], pts[3 * k + 1], pts[3 * k + 2])) ? 1 : 0;
  return 0;
}

}  // extern "C"
