// Host-side scene model of the compound-eye renderer.
//
// A loaded glTF scene is flattened into one world-space triangle list (the
// reference keeps one acceleration structure per glTF primitive under an
// instance transform, MulticamScene.cpp:1052-1428; here every primitive's
// vertices are pre-transformed so a single BVH covers the whole scene).
// The global triangle id is (primitive's offset in load order) + primitive
// index, i.e. the reference's (instanceId, primitiveIndex) pair flattened.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace cr {

struct f3 {
  float x = 0.f, y = 0.f, z = 0.f;
};

// Same 32-byte layout as the reference's Ommatidium
// (libEyeRenderer3/cameras/CompoundEyeDataTypes.h:22-28) and OmmatidiumPacket
// (libEyeRenderer3/libEyeRenderer.h:8-14).
struct Ommatidium {
  f3 pos;
  f3 dir;
  float acceptanceAngle;
  float focalPointOffset;
};
static_assert(sizeof(Ommatidium) == 32, "ommatidium record must stay 32 bytes");

// Camera local frame; defaults follow LocalSpace in
// libEyeRenderer3/cameras/GenericCameraDataTypes.h:16-29.
struct LocalSpace {
  f3 x{1.f, 0.f, 0.f};
  f3 y{0.f, 1.f, 0.f};
  f3 z{0.f, 0.f, 1.f};
};

enum class CameraKind { Perspective, Orthographic, Panoramic, Compound };

struct Camera {
  std::string name;
  CameraKind kind = CameraKind::Perspective;
  f3 position;
  LocalSpace ls;
  // Compound-eye fields (kind == Compound).
  std::string eyeDataPath;
  std::string projection;  // e.g. "single_dimension_fast" (no "__raygen__compound_projection_" prefix)
  std::vector<Ommatidium> omm;
  int spp = 1;
};

// One glTF mesh primitive (the reference's MeshGroup, MulticamScene.cpp:360-370).
struct MeshPrim {
  std::string name;
  double xform[16];  // row-major world transform of the owning node
  uint32_t triOffset = 0;
  uint32_t triCount = 0;
  int colourType = -1;  // 5121, 5123, 5126 or -1 (LocalGeometry.h:107-156)
  f3 worldMin, worldMax;
};

// Meshes flagged with the mesh extra "hitbox" are not rendered; they answer
// isInsideHitGeometry (MulticamScene.cpp:329-345, sutil/hitscanprocessing.cpp).
struct HitboxMesh {
  std::string name;
  double xform[16];
  std::vector<f3> tris;  // object space, 3 per triangle
  f3 objMin, objMax;
  f3 worldMin, worldMax;
};

enum class MissShader { DefaultBackground = 0, SimpleSky = 1 };

constexpr int kLightFloats = 20;

// How a triangle's hit colour is found (shaders.cu:788-811).
enum : uint8_t {
  kShadeBaseColour = 0,    // material base colour factor as is
  kShadeVertexColour = 1,  // pow(barycentric mix of the vertex colours, 2.2)
  kShadeTexture = 2,       // pow(bilinear sample of the base colour texture, 2.2)
};

// One base-colour texture: width x height RGBA8 texels starting at texel
// `offset` of SceneData::texels, row 0 first.
struct Texture {
  uint32_t offset = 0;
  int width = 0, height = 0;
};

struct SceneData {
  // World-space triangles, 9 floats each (v0, v1, v2).
  std::vector<float> triVerts;
  // Per triangle 12 floats, three float4 at v0, v1, v2, by shading kind:
  //   kShadeBaseColour:   the material base colour repeated,
  //   kShadeVertexColour: the vertex colours,
  //   kShadeTexture:      (u, v, texture index, 0) at each vertex.
  std::vector<float> triColours;
  std::vector<uint8_t> triShading;  // one kShade* per triangle
  // Lighting-on shading data (kLightFloats per triangle, original order):
  //   0-8   vertex normals n0, n1, n2 in world space (the object normals times
  //         the inverse transpose of the node transform, not normalised;
  //         zero without NORMAL)
  //   9-14  texture coordinates uv0, uv1, uv2 (TEXCOORD_0, else (0,0) (0,1)
  //         (1,0) as cuda/LocalGeometry.h:99-101)
  //   15    metallic factor, 16 roughness factor (default 1, 1)
  //   17    metallic-roughness texture (scene texture index, -1 none)
  //   18    normal texture (-1 none)
  //   19    flags: 1 = vertex normals, 2 = TEXCOORD_0 present
  std::vector<float> triLight;
  std::vector<uint32_t> texels;     // RGBA8 (r in the low byte) of every texture
  std::vector<Texture> textures;
  std::vector<MeshPrim> meshes;
  std::vector<HitboxMesh> hitboxes;
  std::vector<Camera> cameras;
  MissShader miss = MissShader::DefaultBackground;
  std::string missName = "default_background";
  f3 sceneMin, sceneMax;

  size_t triangleCount() const { return triShading.size(); }
};

// Loads a .gltf (ASCII glTF 2.0) file; throws std::runtime_error on failure.
void loadGltfScene(const std::string& path, SceneData& out, bool verbose);

// Parses a .eye file (8 space-separated floats per line:
// position xyz, direction xyz, acceptance angle in radians, focal offset;
// MulticamScene.cpp:289-299).  Throws on a malformed line.
std::vector<Ommatidium> parseEyeFile(const std::string& path);

// Parity ray cast of sutil/hitscanprocessing.cpp:20-83 for a hitbox mesh.
bool pointInsideHitbox(const HitboxMesh& m, f3 worldPoint);
// The two halves of pointInsideHitbox: the object-space point (double
// inverse, rounded once to float; false for a singular transform), and the
// float parity cast over the listed triangles (items, or all when null).
bool hitboxObjectPoint(const HitboxMesh& m, f3 worldPoint, f3& objectPoint);
bool pointInsideObject(const HitboxMesh& m, f3 objectPoint, const uint32_t* items, size_t nItems);
// Whether triangle t of a hitbox has a non-finite unit normal in that cast
// (zero area, or an overflowing cross product): such a triangle's test does
// not depend on the point's position, so a spatial grid must test it for
// every point.
bool hitboxTriangleCountsEverywhere(const HitboxMesh& m, size_t t);

// Rotates `point` by `angle` about `axis` (normalised first), the host pose
// arithmetic of libEyeRenderer3/cameras/DataRecordCamera.h:83-87.
f3 rotateAboutAxis(f3 point, float angle, f3 axis);

}  // namespace cr
