// glTF 2.0 (ASCII) scene loader for the compound-eye renderer.
//
// Follows the reference's scene rules (libEyeRenderer3/MulticamScene.cpp):
//  * root nodes = nodes that are nobody's child, in index order (:723-735);
//  * node transform = parent * matrix * T * R * S (:173-205);
//  * a node with a camera adds one camera and stops; a node with a mesh adds
//    its primitives (or a hitbox mesh when the mesh extra "hitbox" is true)
//    and stops; only other nodes recurse into their children (:207-525);
//  * camera frame: right = M*(1,0,0,0), up = M*(0,1,0,0),
//    forward = M*(0,0,-1,0), position = M*(0,0,0,1) (:215-219), stored as the
//    local space (x = right, y = up, z = forward) (:231, :311);
//  * compound eyes come from the camera extras "compound-eye",
//    "compound-structure" (.eye path, tried as given and then relative to
//    the glTF's folder) and "compound-projection" (:247-319);
//  * COLOR_0 is used only when it is VEC4 of float / unsigned short /
//    unsigned byte (:415-516), normalised by 1, 65535 or 255 at shading time
//    (cuda/LocalGeometry.h:105-156); otherwise the material baseColorFactor
//    (default white, cuda/MaterialData.h:42) is used;
//  * without vertex colours, a material "baseColorTexture" replaces the base
//    colour by the texture sampled at the TEXCOORD_0 coordinates (float
//    VEC2; without them the coordinates are the hit's barycentrics b1, b2)
//    (shaders.cu:801-805, cuda/LocalGeometry.h:88-103).  The texture's
//    sampler is not consulted: the reference translates the glTF wrap and
//    filter enums to CUDA modes and then compares those CUDA modes with the
//    GL enums again (:605-623, :800-828), which never match, so every
//    texture samples with wrap addressing and linear filtering on
//    normalised coordinates;
//  * every image is decoded up front to RGBA8 (forced four components,
//    tiny_gltf.h:2305-2389); 16-bit images are refused, as the reference's
//    upload into a uchar4 array with a 16-bit pitch fails (:753-795);
//  * the scene extra "background-shader" picks the miss shader (:555-565).
//
// Transforms are composed and applied in double precision and the world
// positions rounded once to float (the reference composes in float and lets
// OptiX apply the instance transform); both the loader here and the oracle
// use this same rule so their triangles agree bit for bit.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>

#include "json.hpp"
#include "png.hpp"
#include "scene.hpp"

namespace cr {
namespace {

using M4 = double[16];

void identity(double* m) {
  for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0 : 0.0;
}

// C = A * B, row-major, each entry summed in k order.
void mul(const double* a, const double* b, double* c) {
  double r[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = a[i * 4 + 0] * b[0 * 4 + j];
      s = s + a[i * 4 + 1] * b[1 * 4 + j];
      s = s + a[i * 4 + 2] * b[2 * 4 + j];
      s = s + a[i * 4 + 3] * b[3 * 4 + j];
      r[i * 4 + j] = s;
    }
  std::memcpy(c, r, sizeof(r));
}

// y = M * (x, y, z, w), each row summed left to right.
void apply(const double* m, double x, double y, double z, double w, double* out) {
  for (int i = 0; i < 3; ++i) {
    double s = m[i * 4 + 0] * x;
    s = s + m[i * 4 + 1] * y;
    s = s + m[i * 4 + 2] * z;
    s = s + m[i * 4 + 3] * w;
    out[i] = s;
  }
}

f3 applyF(const double* m, double x, double y, double z, double w) {
  double o[3];
  apply(m, x, y, z, w, o);
  return f3{static_cast<float>(o[0]), static_cast<float>(o[1]), static_cast<float>(o[2])};
}

// Rotation matrix of the unit quaternion (x, y, z, w) (glTF order).
void quatMatrix(double x, double y, double z, double w, double* m) {
  identity(m);
  const double xx = x * x, yy = y * y, zz = z * z;
  const double xy = x * y, xz = x * z, yz = y * z;
  const double wx = w * x, wy = w * y, wz = w * z;
  m[0] = 1.0 - 2.0 * (yy + zz);
  m[1] = 2.0 * (xy - wz);
  m[2] = 2.0 * (xz + wy);
  m[4] = 2.0 * (xy + wz);
  m[5] = 1.0 - 2.0 * (xx + zz);
  m[6] = 2.0 * (yz - wx);
  m[8] = 2.0 * (xz - wy);
  m[9] = 2.0 * (yz + wx);
  m[10] = 1.0 - 2.0 * (xx + yy);
}

bool extraIsTrue(const Json& extras, const char* key) {
  const Json& v = extras[key];
  if (v.isBool()) return v.asBool();
  if (v.isString()) {
    std::string s = v.asString();
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return static_cast<char>(std::tolower(c)); });
    return s == "true";
  }
  return false;
}

std::string readFile(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f.is_open()) throw std::runtime_error("cannot open '" + path + "'");
  std::ostringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

int b64val(unsigned char c) {
  if (c >= 'A' && c <= 'Z') return c - 'A';
  if (c >= 'a' && c <= 'z') return c - 'a' + 26;
  if (c >= '0' && c <= '9') return c - '0' + 52;
  if (c == '+' || c == '-') return 62;
  if (c == '/' || c == '_') return 63;
  return -1;
}

std::vector<uint8_t> base64Decode(const std::string& s, size_t begin) {
  std::vector<uint8_t> out;
  out.reserve((s.size() - begin) * 3 / 4);
  uint32_t acc = 0;
  int bits = 0;
  for (size_t i = begin; i < s.size(); ++i) {
    const int v = b64val(static_cast<unsigned char>(s[i]));
    if (v < 0) continue;  // padding, whitespace
    acc = (acc << 6) | static_cast<uint32_t>(v);
    bits += 6;
    if (bits >= 8) {
      bits -= 8;
      out.push_back(static_cast<uint8_t>((acc >> bits) & 0xFF));
    }
  }
  return out;
}

struct Model {
  Json doc;
  std::string dir;
  std::vector<std::vector<uint8_t>> buffers;
  std::vector<int> textureImage;  // glTF texture -> SceneData::textures index
};

// A read-only view of one accessor.
struct Accessor {
  const uint8_t* base = nullptr;
  size_t count = 0;
  size_t stride = 0;
  int compType = 0;
  int comps = 0;
  size_t avail = 0;  // bytes available from base

  static int compSize(int t) {
    switch (t) {
      case 5120: case 5121: return 1;
      case 5122: case 5123: return 2;
      case 5125: case 5126: return 4;
      default: return 0;
    }
  }
  // Raw component read as double (no normalisation).
  double get(size_t i, int c) const {
    const uint8_t* p = base + i * stride + static_cast<size_t>(c) * compSize(compType);
    switch (compType) {
      case 5120: return static_cast<double>(*reinterpret_cast<const int8_t*>(p));
      case 5121: return static_cast<double>(*p);
      case 5122: { int16_t v; std::memcpy(&v, p, 2); return v; }
      case 5123: { uint16_t v; std::memcpy(&v, p, 2); return v; }
      case 5125: { uint32_t v; std::memcpy(&v, p, 4); return v; }
      case 5126: { float v; std::memcpy(&v, p, 4); return v; }
      default: return 0.0;
    }
  }
  float getF(size_t i, int c) const {
    const uint8_t* p = base + i * stride + static_cast<size_t>(c) * 4;
    float v;
    std::memcpy(&v, p, 4);
    return v;
  }
  uint32_t getU(size_t i) const { return static_cast<uint32_t>(get(i, 0)); }
};

int typeComponents(const std::string& t) {
  if (t == "SCALAR") return 1;
  if (t == "VEC2") return 2;
  if (t == "VEC3") return 3;
  if (t == "VEC4") return 4;
  if (t == "MAT4") return 16;
  return 0;
}

Accessor accessor(const Model& m, int idx) {
  const Json& accs = m.doc["accessors"];
  if (idx < 0 || static_cast<size_t>(idx) >= accs.size()) throw std::runtime_error("accessor index out of range");
  const Json& a = accs[static_cast<size_t>(idx)];
  if (a.has("sparse")) throw std::runtime_error("sparse accessors are not supported");
  Accessor out;
  out.count = static_cast<size_t>(a.num("count", 0));
  out.compType = a.integer("componentType", 0);
  out.comps = typeComponents(a.str("type"));
  const int cs = Accessor::compSize(out.compType);
  if (cs == 0 || out.comps == 0) throw std::runtime_error("accessor has an unsupported component type");
  if (!a.has("bufferView")) throw std::runtime_error("accessor without bufferView is not supported");
  const Json& bv = m.doc["bufferViews"][static_cast<size_t>(a.integer("bufferView", 0))];
  const int bufIdx = bv.integer("buffer", -1);
  if (bufIdx < 0 || static_cast<size_t>(bufIdx) >= m.buffers.size()) throw std::runtime_error("bufferView buffer out of range");
  const std::vector<uint8_t>& buf = m.buffers[static_cast<size_t>(bufIdx)];
  const size_t off = static_cast<size_t>(bv.num("byteOffset", 0)) + static_cast<size_t>(a.num("byteOffset", 0));
  const size_t bvEnd = static_cast<size_t>(bv.num("byteOffset", 0)) + static_cast<size_t>(bv.num("byteLength", 0));
  out.stride = static_cast<size_t>(bv.num("byteStride", 0));
  if (out.stride == 0) out.stride = static_cast<size_t>(cs * out.comps);
  const size_t need = out.count == 0 ? 0 : (out.count - 1) * out.stride + static_cast<size_t>(cs * out.comps);
  if (off + need > buf.size() || off + need > bvEnd) throw std::runtime_error("accessor reads past the end of its buffer");
  out.base = buf.data() + off;
  out.avail = buf.size() - off;
  return out;
}

struct Loader {
  Model& m;
  SceneData& s;
  bool verbose;

  void log(const std::string& msg) const {
    if (verbose) std::cerr << msg << "\n";
  }

  void nodeMatrix(const Json& node, const double* parent, double* out) const {
    double t[16], r[16], sc[16], mx[16];
    identity(t);
    identity(r);
    identity(sc);
    identity(mx);
    const Json& tr = node["translation"];
    if (tr.isArray() && tr.size() == 3) {
      t[3] = tr[0].asNumber();
      t[7] = tr[1].asNumber();
      t[11] = tr[2].asNumber();
    }
    const Json& q = node["rotation"];
    if (q.isArray() && q.size() == 4) quatMatrix(q[0].asNumber(), q[1].asNumber(), q[2].asNumber(), q[3].asNumber(), r);
    const Json& scl = node["scale"];
    if (scl.isArray() && scl.size() == 3) {
      sc[0] = scl[0].asNumber();
      sc[5] = scl[1].asNumber();
      sc[10] = scl[2].asNumber();
    }
    const Json& mat = node["matrix"];
    if (mat.isArray() && mat.size() == 16) {
      // glTF stores column-major; keep row-major here.
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) mx[i * 4 + j] = mat[static_cast<size_t>(j * 4 + i)].asNumber();
    }
    double a[16];
    mul(parent, mx, a);
    mul(a, t, a);
    mul(a, r, a);
    mul(a, sc, out);
  }

  void addCamera(const Json& node, const double* xf) {
    const Json& cam = m.doc["cameras"][static_cast<size_t>(node.integer("camera", 0))];
    Camera c;
    c.name = cam.str("name");
    c.position = applyF(xf, 0, 0, 0, 1);
    c.ls.x = applyF(xf, 1, 0, 0, 0);
    c.ls.y = applyF(xf, 0, 1, 0, 0);
    c.ls.z = applyF(xf, 0, 0, -1, 0);
    const Json& extras = cam["extras"];
    if (cam.str("type") == "orthographic") {
      c.kind = CameraKind::Orthographic;
      s.cameras.push_back(c);
      return;
    }
    if (extraIsTrue(extras, "panoramic")) {
      c.kind = CameraKind::Panoramic;
      s.cameras.push_back(c);
      return;
    }
    if (extraIsTrue(extras, "compound-eye")) {
      const std::string eyePath = extras.str("compound-structure");
      const std::string proj = extras.str("compound-projection");
      if (eyePath.empty()) {
        std::cerr << "ERROR: Eye data path empty or non-existant." << std::endl;
        return;
      }
      if (proj.empty()) {
        std::cerr << "ERROR: Projection shader specifier empty or non-existant." << std::endl;
        return;
      }
      std::string used = eyePath;
      {
        std::ifstream f(eyePath);
        if (!f.is_open()) {
          used = m.dir + eyePath;
          std::ifstream g(used);
          if (!g.is_open()) {
            std::cerr << "ERROR: Unable to open \"" << used << "\", read cancelled." << std::endl;
            return;
          }
        }
      }
      std::vector<Ommatidium> omm = parseEyeFile(used);
      if (omm.empty()) {
        std::cerr << "  ERROR: Zero ommatidia loaded." << std::endl;
        return;
      }
      c.kind = CameraKind::Compound;
      c.eyeDataPath = used;
      c.projection = proj;
      c.omm = std::move(omm);
      s.cameras.push_back(std::move(c));
      return;
    }
    c.kind = CameraKind::Perspective;
    s.cameras.push_back(c);
  }

  void addHitbox(const Json& mesh, const double* xf) {
    HitboxMesh h;
    h.name = mesh.str("name");
    std::memcpy(h.xform, xf, sizeof(h.xform));
    for (const Json& prim : mesh["primitives"].items()) {
      if (prim.integer("mode", 4) != 4) continue;
      if (!prim.has("indices")) continue;
      const Accessor ia = accessor(m, prim.integer("indices", -1));
      const Accessor pa = accessor(m, prim["attributes"].integer("POSITION", -1));
      for (size_t i = 0; i + 3 <= ia.count; i += 3) {
        for (int k = 0; k < 3; ++k) {
          const uint32_t vi = ia.getU(i + static_cast<size_t>(k));
          if (vi >= pa.count) throw std::runtime_error("hitbox index out of range");
          h.tris.push_back(f3{static_cast<float>(pa.get(vi, 0)), static_cast<float>(pa.get(vi, 1)), static_cast<float>(pa.get(vi, 2))});
        }
      }
    }
    if (h.tris.empty()) {
      h.objMin = h.objMax = f3{};
    } else {
      h.objMin = h.objMax = h.tris[0];
      for (const f3& p : h.tris) {
        h.objMin = f3{std::min(h.objMin.x, p.x), std::min(h.objMin.y, p.y), std::min(h.objMin.z, p.z)};
        h.objMax = f3{std::max(h.objMax.x, p.x), std::max(h.objMax.y, p.y), std::max(h.objMax.z, p.z)};
      }
    }
    transformBox(xf, h.objMin, h.objMax, h.worldMin, h.worldMax);
    s.hitboxes.push_back(std::move(h));
  }

  static void transformBox(const double* xf, f3 lo, f3 hi, f3& wlo, f3& whi) {
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
      double o[3];
      apply(xf, (c & 1) ? hi.x : lo.x, (c & 2) ? hi.y : lo.y, (c & 4) ? hi.z : lo.z, 1.0, o);
      for (int k = 0; k < 3; ++k) {
        mn[k] = std::min(mn[k], o[k]);
        mx[k] = std::max(mx[k], o[k]);
      }
    }
    wlo = f3{static_cast<float>(mn[0]), static_cast<float>(mn[1]), static_cast<float>(mn[2])};
    whi = f3{static_cast<float>(mx[0]), static_cast<float>(mx[1]), static_cast<float>(mx[2])};
  }

  // Material base colour factor, and the scene texture index of its base
  // colour texture (-1 when it has none).
  int baseColour(int matIdx, float* rgba) const {
    rgba[0] = rgba[1] = rgba[2] = rgba[3] = 1.0f;
    if (matIdx < 0) return -1;
    if (static_cast<size_t>(matIdx) >= m.doc["materials"].size()) throw std::runtime_error("material index out of range");
    const Json& mat = m.doc["materials"][static_cast<size_t>(matIdx)];
    const Json& pbr = mat["pbrMetallicRoughness"];
    const Json& f = pbr["baseColorFactor"];
    if (f.isArray() && f.size() == 4)
      for (size_t k = 0; k < 4; ++k) rgba[k] = static_cast<float>(f[k].asNumber());
    if (!pbr.has("baseColorTexture")) return -1;
    const int t = pbr["baseColorTexture"].integer("index", -1);
    if (t < 0 || static_cast<size_t>(t) >= m.textureImage.size())
      throw std::runtime_error("material " + std::to_string(matIdx) + ": base colour texture index out of range");
    return m.textureImage[static_cast<size_t>(t)];
  }

  // Lighting parameters of a material (MulticamScene.cpp:626-715,
  // cuda/MaterialData.h:42-50): metallic and roughness factors (default 1),
  // metallic-roughness and normal textures as scene texture indices.
  void materialLighting(int matIdx, float& metallic, float& roughness, int& mrTex, int& nTex) const {
    metallic = roughness = 1.0f;
    mrTex = nTex = -1;
    if (matIdx < 0) return;
    const Json& mat = m.doc["materials"][static_cast<size_t>(matIdx)];
    const Json& pbr = mat["pbrMetallicRoughness"];
    if (pbr.has("metallicFactor")) metallic = static_cast<float>(pbr["metallicFactor"].asNumber());
    if (pbr.has("roughnessFactor")) roughness = static_cast<float>(pbr["roughnessFactor"].asNumber());
    auto texOf = [&](const Json& info) {
      const int t = info.integer("index", -1);
      if (t < 0 || static_cast<size_t>(t) >= m.textureImage.size())
        throw std::runtime_error("material " + std::to_string(matIdx) + ": texture index out of range");
      return m.textureImage[static_cast<size_t>(t)];
    };
    if (pbr.has("metallicRoughnessTexture")) mrTex = texOf(pbr["metallicRoughnessTexture"]);
    if (mat.has("normalTexture")) nTex = texOf(mat["normalTexture"]);
  }

  void addMesh(const Json& mesh, const double* xf) {
    for (const Json& prim : mesh["primitives"].items()) {
      if (prim.integer("mode", 4) != 4) {
        log("\tNon-triangle primitive: skipping");
        continue;
      }
      MeshPrim mp;
      mp.name = mesh.str("name");
      std::memcpy(mp.xform, xf, sizeof(mp.xform));
      mp.triOffset = static_cast<uint32_t>(s.triangleCount());
      const Json& attrs = prim["attributes"];
      if (!attrs.has("POSITION")) throw std::runtime_error("primitive without POSITION");
      const Accessor pa = accessor(m, attrs.integer("POSITION", -1));
      if (pa.compType != 5126 || pa.comps != 3) throw std::runtime_error("POSITION must be float VEC3");
      // Object-space bounds from the accessor's min/max (computed when absent).
      const Json& pacc = m.doc["accessors"][static_cast<size_t>(attrs.integer("POSITION", -1))];
      f3 lo{INFINITY, INFINITY, INFINITY}, hi{-INFINITY, -INFINITY, -INFINITY};
      if (pacc["min"].size() == 3 && pacc["max"].size() == 3) {
        lo = f3{static_cast<float>(pacc["min"][0].asNumber()), static_cast<float>(pacc["min"][1].asNumber()),
                static_cast<float>(pacc["min"][2].asNumber())};
        hi = f3{static_cast<float>(pacc["max"][0].asNumber()), static_cast<float>(pacc["max"][1].asNumber()),
                static_cast<float>(pacc["max"][2].asNumber())};
      } else {
        for (size_t i = 0; i < pa.count; ++i) {
          lo = f3{std::min(lo.x, pa.getF(i, 0)), std::min(lo.y, pa.getF(i, 1)), std::min(lo.z, pa.getF(i, 2))};
          hi = f3{std::max(hi.x, pa.getF(i, 0)), std::max(hi.y, pa.getF(i, 1)), std::max(hi.z, pa.getF(i, 2))};
        }
      }
      transformBox(xf, lo, hi, mp.worldMin, mp.worldMax);

      // Vertex colours: VEC4 float / u16 / u8 only.
      int ctype = -1;
      Accessor ca;
      if (attrs.has("COLOR_0")) {
        const Accessor c = accessor(m, attrs.integer("COLOR_0", -1));
        if (c.comps == 4 && (c.compType == 5126 || c.compType == 5123 || c.compType == 5121)) {
          ctype = c.compType;
          ca = c;
        } else if (c.comps != 4) {
          log("\t\t\tWarning: Vertex colours are not of type vec4. Ignoring vertex colours.");
        }
      }
      mp.colourType = ctype;
      float base[4];
      const int matTex = baseColour(prim.integer("material", -1), base);
      const int tex = ctype == -1 ? matTex : -1;  // vertex colours take precedence
      Accessor ta;
      bool hasUv = false;
      if (attrs.has("TEXCOORD_0")) {
        ta = accessor(m, attrs.integer("TEXCOORD_0", -1));
        if (ta.compType == 5121) throw std::runtime_error("gltf accessor component type not supported");
        if (tex >= 0 && (ta.compType != 5126 || ta.comps != 2)) throw std::runtime_error("TEXCOORD_0 must be float VEC2");
        hasUv = ta.compType == 5126 && ta.comps == 2;
      }
      // Lighting data: vertex normals (float VEC3) through the normal matrix.
      Accessor na;
      bool hasN = false;
      if (attrs.has("NORMAL")) {
        na = accessor(m, attrs.integer("NORMAL", -1));
        hasN = na.compType == 5126 && na.comps == 3;
      }
      double nm[9];  // inverse transpose of the upper 3x3 of xf
      {
        const double a = xf[0], b = xf[1], c = xf[2], d = xf[4], e = xf[5], f = xf[6], g = xf[8], h = xf[9],
                     i = xf[10];
        const double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
        const double id = det != 0.0 ? 1.0 / det : 0.0;
        // cofactor matrix / det = inverse transpose
        nm[0] = (e * i - f * h) * id;
        nm[1] = -(d * i - f * g) * id;
        nm[2] = (d * h - e * g) * id;
        nm[3] = -(b * i - c * h) * id;
        nm[4] = (a * i - c * g) * id;
        nm[5] = -(a * h - b * g) * id;
        nm[6] = (b * f - c * e) * id;
        nm[7] = -(a * f - c * d) * id;
        nm[8] = (a * e - b * d) * id;
      }
      float metallic, roughness;
      int mrTex, nTex;
      materialLighting(prim.integer("material", -1), metallic, roughness, mrTex, nTex);

      // Indices (u8 / u16 / u32); a primitive without indices has no triangles,
      // as a build input with zero index triplets in the reference.
      size_t triCount = 0;
      Accessor ia;
      if (prim.has("indices")) {
        ia = accessor(m, prim.integer("indices", -1));
        if (ia.comps != 1 || (ia.compType != 5121 && ia.compType != 5123 && ia.compType != 5125))
          throw std::runtime_error("gltf accessor component type not supported");
        triCount = ia.count / 3;
      }
      for (size_t t = 0; t < triCount; ++t) {
        float cols[12];
        for (int k = 0; k < 3; ++k) {
          const uint32_t vi = ia.getU(3 * t + static_cast<size_t>(k));
          if (vi >= pa.count) throw std::runtime_error("vertex index out of range in mesh '" + mp.name + "'");
          const f3 w = applyF(xf, pa.getF(vi, 0), pa.getF(vi, 1), pa.getF(vi, 2), 1.0);
          s.triVerts.push_back(w.x);
          s.triVerts.push_back(w.y);
          s.triVerts.push_back(w.z);
          if (tex >= 0) {
            // (u, v, texture, 0); the default coordinates (0,0) (1,0) (0,1)
            // interpolate to exactly (b1, b2).
            if (hasUv && vi >= ta.count) throw std::runtime_error("texture coordinate index out of range");
            cols[k * 4 + 0] = hasUv ? ta.getF(vi, 0) : (k == 1 ? 1.0f : 0.0f);
            cols[k * 4 + 1] = hasUv ? ta.getF(vi, 1) : (k == 2 ? 1.0f : 0.0f);
            cols[k * 4 + 2] = static_cast<float>(tex);
            cols[k * 4 + 3] = 0.0f;
            continue;
          }
          for (int q = 0; q < 4; ++q) {
            float v = base[q];
            if (ctype == 5126) v = ca.getF(vi, q);
            else if (ctype == 5123) v = static_cast<float>(ca.get(vi, q)) / 65535.0f;
            else if (ctype == 5121) v = static_cast<float>(ca.get(vi, q)) / 255.0f;
            cols[k * 4 + q] = v;
          }
        }
        s.triColours.insert(s.triColours.end(), cols, cols + 12);
        s.triShading.push_back(ctype != -1 ? kShadeVertexColour : tex >= 0 ? kShadeTexture : kShadeBaseColour);
        float lt[kLightFloats];
        static const float kDefaultUv[6] = {0.f, 0.f, 0.f, 1.f, 1.f, 0.f};
        for (int k = 0; k < 3; ++k) {
          const uint32_t vi = ia.getU(3 * t + static_cast<size_t>(k));
          for (int q = 0; q < 3; ++q) lt[3 * k + q] = 0.f;
          if (hasN && vi < na.count) {
            const double n0 = na.getF(vi, 0), n1 = na.getF(vi, 1), n2 = na.getF(vi, 2);
            for (int q = 0; q < 3; ++q) lt[3 * k + q] = static_cast<float>(nm[3 * q] * n0 + nm[3 * q + 1] * n1 + nm[3 * q + 2] * n2);
          }
          lt[9 + 2 * k] = hasUv && vi < ta.count ? ta.getF(vi, 0) : kDefaultUv[2 * k];
          lt[10 + 2 * k] = hasUv && vi < ta.count ? ta.getF(vi, 1) : kDefaultUv[2 * k + 1];
        }
        lt[15] = metallic;
        lt[16] = roughness;
        lt[17] = static_cast<float>(mrTex);
        lt[18] = static_cast<float>(nTex);
        lt[19] = static_cast<float>((hasN ? 1 : 0) | (hasUv ? 2 : 0));
        s.triLight.insert(s.triLight.end(), lt, lt + kLightFloats);
      }
      mp.triCount = static_cast<uint32_t>(triCount);
      s.meshes.push_back(mp);
    }
  }

  void node(size_t idx, const double* parent, int depth) {
    if (depth > 256) throw std::runtime_error("node hierarchy too deep (cycle?)");
    const Json& n = m.doc["nodes"][idx];
    double xf[16];
    nodeMatrix(n, parent, xf);
    if (n.has("camera") && n.integer("camera", -1) >= 0) {
      addCamera(n, xf);
    } else if (n.has("mesh") && n.integer("mesh", -1) >= 0 &&
               extraIsTrue(m.doc["meshes"][static_cast<size_t>(n.integer("mesh", 0))]["extras"], "hitbox")) {
      addHitbox(m.doc["meshes"][static_cast<size_t>(n.integer("mesh", 0))], xf);
    } else if (n.has("mesh") && n.integer("mesh", -1) >= 0) {
      addMesh(m.doc["meshes"][static_cast<size_t>(n.integer("mesh", 0))], xf);
    } else {
      for (const Json& c : n["children"].items()) node(static_cast<size_t>(c.asNumber()), xf, depth + 1);
    }
  }
};

}  // namespace

std::vector<Ommatidium> parseEyeFile(const std::string& path) {
  std::ifstream f(path);
  if (!f.is_open()) throw std::runtime_error("cannot open eye file '" + path + "'");
  std::vector<Ommatidium> out;
  std::string line;
  size_t lineNo = 0;
  while (std::getline(f, line)) {
    ++lineNo;
    // Tokens are separated by single spaces; runs of spaces give no empty
    // tokens except a trailing one (libEyeRenderer3/MulticamScene.cpp:147-163).
    std::vector<std::string> tok;
    size_t last = 0, at = line.find(' ');
    while (at != std::string::npos) {
      if (at != last) tok.push_back(line.substr(last, at - last));
      last = at + 1;
      at = line.find(' ', last);
    }
    tok.push_back(line.substr(last));
    if (tok.size() < 8) throw std::runtime_error("eye file '" + path + "' line " + std::to_string(lineNo) + ": expected 8 values");
    float v[8];
    for (int i = 0; i < 8; ++i) {
      const char* b = tok[static_cast<size_t>(i)].c_str();
      char* e = nullptr;
      v[i] = std::strtof(b, &e);
      if (e == b) throw std::runtime_error("eye file '" + path + "' line " + std::to_string(lineNo) + ": bad number");
    }
    out.push_back(Ommatidium{f3{v[0], v[1], v[2]}, f3{v[3], v[4], v[5]}, v[6], v[7]});
  }
  return out;
}

void loadGltfScene(const std::string& path, SceneData& out, bool verbose) {
  Model m;
  m.doc = Json::parse(readFile(path));
  const size_t slash = path.find_last_of("/\\");
  m.dir = slash == std::string::npos ? std::string() : path.substr(0, slash + 1);
  for (const Json& b : m.doc["buffers"].items()) {
    const std::string uri = b.str("uri");
    if (uri.rfind("data:", 0) == 0) {
      const size_t comma = uri.find(',');
      if (comma == std::string::npos || uri.find(";base64") == std::string::npos)
        throw std::runtime_error("unsupported data URI in buffer");
      m.buffers.push_back(base64Decode(uri, comma + 1));
    } else if (!uri.empty()) {
      const std::string raw = readFile(m.dir + uri);
      m.buffers.emplace_back(raw.begin(), raw.end());
    } else {
      throw std::runtime_error("buffer without uri (GLB) is not supported");
    }
  }
  SceneData s;
  // Images (all of them, used or not) then textures, which name an image.
  size_t imgIdx = 0;
  for (const Json& im : m.doc["images"].items()) {
    const std::string where = "image " + std::to_string(imgIdx++) + " '" + im.str("name") + "'";
    std::vector<uint8_t> bytes;
    const std::string uri = im.str("uri");
    if (uri.rfind("data:", 0) == 0) {
      const size_t comma = uri.find(',');
      if (comma == std::string::npos || uri.find(";base64") == std::string::npos)
        throw std::runtime_error(where + ": unsupported data URI");
      bytes = base64Decode(uri, comma + 1);
    } else if (!uri.empty()) {
      const std::string raw = readFile(m.dir + uri);
      bytes.assign(raw.begin(), raw.end());
    } else if (im.has("bufferView")) {
      const size_t bvi = static_cast<size_t>(im.integer("bufferView", -1));
      if (bvi >= m.doc["bufferViews"].size()) throw std::runtime_error(where + ": bufferView out of range");
      const Json& bv = m.doc["bufferViews"][bvi];
      const int bufIdx = bv.integer("buffer", -1);
      if (bufIdx < 0 || static_cast<size_t>(bufIdx) >= m.buffers.size())
        throw std::runtime_error(where + ": bufferView buffer out of range");
      const std::vector<uint8_t>& buf = m.buffers[static_cast<size_t>(bufIdx)];
      const size_t off = static_cast<size_t>(bv.num("byteOffset", 0)), len = static_cast<size_t>(bv.num("byteLength", 0));
      if (off + len > buf.size()) throw std::runtime_error(where + ": bufferView past the end of its buffer");
      bytes.assign(buf.begin() + static_cast<std::ptrdiff_t>(off), buf.begin() + static_cast<std::ptrdiff_t>(off + len));
    } else {
      throw std::runtime_error(where + ": no uri or bufferView");
    }
    if (!isPng(bytes.data(), bytes.size())) throw std::runtime_error(where + ": only PNG images are supported");
    Image img;
    try {
      img = decodePng(bytes.data(), bytes.size());
    } catch (const std::exception& e) {
      throw std::runtime_error(where + ": " + e.what());
    }
    if (img.bits == 16) throw std::runtime_error(where + ": 16-bit images are not supported");
    Texture t;
    t.offset = static_cast<uint32_t>(s.texels.size());
    t.width = img.width;
    t.height = img.height;
    const size_t n = static_cast<size_t>(img.width) * static_cast<size_t>(img.height);
    if (s.texels.size() + n > 0xFFFFFFFFull) throw std::runtime_error(where + ": texture memory exceeds 2^32 texels");
    for (size_t i = 0; i < n; ++i) {
      const uint8_t* p = &img.rgba[4 * i];
      s.texels.push_back(static_cast<uint32_t>(p[0]) | (static_cast<uint32_t>(p[1]) << 8) |
                         (static_cast<uint32_t>(p[2]) << 16) | (static_cast<uint32_t>(p[3]) << 24));
    }
    s.textures.push_back(t);
    if (verbose)
      std::cerr << "Processing " << where << "\n\t(" << img.width << "x" << img.height << ")x4\n\tbits: 8" << std::endl;
  }
  for (const Json& tx : m.doc["textures"].items()) {
    const int src = tx.integer("source", -1);
    if (src < 0 || static_cast<size_t>(src) >= s.textures.size())
      throw std::runtime_error("texture " + std::to_string(m.textureImage.size()) + ": source image out of range");
    m.textureImage.push_back(src);
  }
  for (const Json& sc : m.doc["scenes"].items()) {
    const std::string bg = sc["extras"].str("background-shader");
    if (!bg.empty()) s.missName = bg;
  }
  if (s.missName == "simple_sky") s.miss = MissShader::SimpleSky;
  else if (s.missName == "default_background") s.miss = MissShader::DefaultBackground;
  else throw std::runtime_error("unknown background shader '" + s.missName + "'");

  Loader L{m, s, verbose};
  const size_t nn = m.doc["nodes"].size();
  std::vector<int> isRoot(nn, 1);
  for (size_t i = 0; i < nn; ++i)
    for (const Json& c : m.doc["nodes"][i]["children"].items()) {
      const size_t ci = static_cast<size_t>(c.asNumber());
      if (ci < nn) isRoot[ci] = 0;
    }
  double id[16];
  identity(id);
  for (size_t i = 0; i < nn; ++i)
    if (isRoot[i]) L.node(i, id, 0);

  s.sceneMin = f3{INFINITY, INFINITY, INFINITY};
  s.sceneMax = f3{-INFINITY, -INFINITY, -INFINITY};
  for (const MeshPrim& mp : s.meshes) {
    s.sceneMin = f3{std::min(s.sceneMin.x, mp.worldMin.x), std::min(s.sceneMin.y, mp.worldMin.y), std::min(s.sceneMin.z, mp.worldMin.z)};
    s.sceneMax = f3{std::max(s.sceneMax.x, mp.worldMax.x), std::max(s.sceneMax.y, mp.worldMax.y), std::max(s.sceneMax.z, mp.worldMax.z)};
  }
  // A scene without cameras gets one default perspective camera, as the
  // reference's getCamera() does on finalize (MulticamScene.cpp:911-927).
  if (s.cameras.empty()) {
    Camera c;
    c.name = "Default Camera";
    s.cameras.push_back(c);
  }
  out = std::move(s);
}

f3 rotateAboutAxis(f3 p, float angle, f3 axis) {
  const float len = std::sqrt(axis.x * axis.x + axis.y * axis.y + axis.z * axis.z);
  const f3 a{axis.x / len, axis.y / len, axis.z / len};
  const float c = std::cos(angle), sn = std::sin(angle);
  const f3 cr{a.y * p.z - a.z * p.y, a.z * p.x - a.x * p.z, a.x * p.y - a.y * p.x};
  const float d = a.x * p.x + a.y * p.y + a.z * p.z;
  const float k = (1.0f - c) * d;
  return f3{c * p.x + sn * cr.x + k * a.x, c * p.y + sn * cr.y + k * a.y, c * p.z + sn * cr.z + k * a.z};
}

// The object-space point of a hitbox query, as the reference forms it
// (hitscanprocessing.cpp:22): the inverse node transform times
// make_float4(worldPoint), whose w is 0 (sutil/vec_math.h make_float4 of a
// float3), so only the 3x3 part of the inverse applies and the node's
// translation is ignored.  Here the 3x3 part is inverted by cofactors in
// double and the product rounded once to float.  false when the transform
// is singular.
bool hitboxObjectPoint(const HitboxMesh& m, f3 wp, f3& out) {
  const double* x = m.xform;
  const double a = x[0], b = x[1], c = x[2], d = x[4], e = x[5], f = x[6], g = x[8], h = x[9], i = x[10];
  const double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
  if (det == 0.0) return false;
  const double inv[9] = {(e * i - f * h) / det, (c * h - b * i) / det, (b * f - c * e) / det,
                         (f * g - d * i) / det, (a * i - c * g) / det, (c * d - a * f) / det,
                         (d * h - e * g) / det, (b * g - a * h) / det, (a * e - b * d) / det};
  const double q[3] = {wp.x, wp.y, wp.z};
  double o[3];
  for (int r = 0; r < 3; ++r) o[r] = inv[r * 3 + 0] * q[0] + inv[r * 3 + 1] * q[1] + inv[r * 3 + 2] * q[2];
  out = f3{static_cast<float>(o[0]), static_cast<float>(o[1]), static_cast<float>(o[2])};
  return true;
}

namespace {
// float3 algebra in the operation order of the reference's vector helpers
// (sutil/vec_math.h: dot left to right, cross by components, normalize as
// v * (1 / sqrt(dot(v, v)))); this file is built without contraction.
f3 sub(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
f3 cross(f3 a, f3 b) { return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
f3 normalize(f3 v) {
  const float inv = 1.0f / std::sqrt(dot(v, v));
  return f3{v.x * inv, v.y * inv, v.z * inv};
}
}  // namespace

bool hitboxTriangleCountsEverywhere(const HitboxMesh& m, size_t t) {
  // The cast's unit normal of triangle t, as pointInsideObject forms it: a
  // zero-area triangle gives 0 * inf = NaN components (an overflowing one
  // infinities), its plane and edge comparisons are all false, and it counts
  // as a crossing for every point, as in the reference.
  const f3 p0 = m.tris[3 * t], p1 = m.tris[3 * t + 1], p2 = m.tris[3 * t + 2];
  const f3 n = normalize(cross(sub(p1, p0), sub(p2, p0)));
  return !(std::isfinite(n.x) && std::isfinite(n.y) && std::isfinite(n.z));
}

bool pointInsideObject(const HitboxMesh& m, f3 obj, const uint32_t* items, size_t nItems) {
  // The reference's parity cast (sutil/hitscanprocessing.cpp:20-83), in float
  // in its operation order: a ray from x = object box min.x - 1 along +x to
  // the point, counting the triangle crossings before the point.  No special
  // case is added: a point at the ray start gives a NaN direction, as there.
  const f3 start{m.objMin.x - 1.0f, obj.y, obj.z};
  const f3 dir = normalize(sub(obj, start));
  unsigned crossings = 0;
  const size_t nt = items ? nItems : m.tris.size() / 3;
  for (size_t j = 0; j < nt; ++j) {
    const size_t t = 3 * (items ? items[j] : j);
    const f3 p0 = m.tris[t], p1 = m.tris[t + 1], p2 = m.tris[t + 2];
    const f3 n = normalize(cross(sub(p1, p0), sub(p2, p0)));
    const float den = dot(n, dir);
    if (den == 0) continue;
    const float dist = dot(sub(p0, start), n) / den;
    if (dist == 0) continue;
    const f3 hit{start.x + dist * dir.x, start.y + dist * dir.y, start.z + dist * dir.z};
    if (dist < 0 || hit.x > obj.x) continue;
    if (dot(n, cross(sub(p1, p0), sub(hit, p0))) < 0) continue;
    if (dot(n, cross(sub(p2, p1), sub(hit, p1))) < 0) continue;
    if (dot(n, cross(sub(p0, p2), sub(hit, p2))) < 0) continue;
    ++crossings;
  }
  return crossings % 2 == 1;
}

bool pointInsideHitbox(const HitboxMesh& m, f3 wp) {
  f3 obj;
  if (!hitboxObjectPoint(m, wp, obj)) return false;
  return pointInsideObject(m, obj, nullptr, 0);
}

}  // namespace cr
