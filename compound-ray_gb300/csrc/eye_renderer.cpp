// The C ABI of the headless compound-eye renderer (include/libEyeRenderer.h).
//
// Host state mirrors the reference's globals (libEyeRenderer3/libEyeRenderer.cpp:81-92):
// one scene, a list of cameras with a current index, a render size
// (default 400 x 400) and a verbosity flag.  Each compound camera owns its
// ommatidium records, generator states and a "configured" flag, which the
// first render of the eye sets (libEyeRenderer.cpp:178-179) and every sample
// count or ommatidium count change clears (cameras/CompoundEye.cpp:30-48,
// 98-115, 171-179).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/libEyeRenderer.h"
#include "bvh.hpp"
#include "wbvh.hpp"
#include "device_api.hpp"
#include "denoiser.hpp"
#include "scene.hpp"

namespace cr {
namespace {

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// Device bytes held by the library's buffers, and an optional cap on them
// (0: none) under which an allocation fails as an out-of-memory cudaMalloc
// would: the allocator's fault-injection knob (crSetDeviceMemoryCap).
size_t& devHeld() {
  static size_t held = 0;
  return held;
}
size_t& devCap() {
  static size_t cap = 0;
  return cap;
}

template <typename T>
struct DevBuf {
  T* ptr = nullptr;
  size_t count = 0;
  void release() {
    if (ptr) {
      cudaFree(ptr);
      devHeld() -= count * sizeof(T);
    }
    ptr = nullptr;
    count = 0;
  }
  void ensure(size_t n) {
    if (n <= count && ptr) return;
    release();
    if (n == 0) return;
    const size_t bytes = n * sizeof(T);
    if (devCap() && devHeld() + bytes > devCap())
      throw std::runtime_error("device memory cap reached: " + std::to_string(devHeld()) + " bytes held, " +
                               std::to_string(bytes) + " more requested, cap " + std::to_string(devCap()));
    check(cudaMalloc(reinterpret_cast<void**>(&ptr), bytes), "cudaMalloc");
    devHeld() += bytes;
    count = n;
  }
};

// One candidate grid of the spherical projections (SphereGridView).
struct SphereGrid {
  DevBuf<uint32_t> start, items;
  int G = 0;
};

struct EyeDev {
  DevBuf<float4> omm;
  DevBuf<uint32_t> order;  // warp-segment order of the ommatidia (directionOrder)
  DevBuf<uint32_t> rng;
  DevBuf<float> sums;  // N x 3 of the last frame
  SphereGrid grids[4];  // spherical-projection candidates, built on first use
  bool gridsBuilt = false;
  uint32_t N = 0, spp = 0;
  float maxRel = 0.f;  // largest |position - focal offset * unit axis| over the ommatidia
  bool configured = false;
  bool haveSums = false;
  void releaseGrids() {
    for (SphereGrid& g : grids) {
      g.start.release();
      g.items.release();
      g.G = 0;
    }
    gridsBuilt = false;
  }
  void release() {
    omm.release();
    order.release();
    rng.release();
    sums.release();
    releaseGrids();
    N = spp = 0;
    configured = false;
    haveSums = false;
  }
};

// Candidate grids of the spherical projections for an eye's ommatidia:
// set 0 positions, 1 directions, 2 / 3 directions of the ommatidia with
// position.x < 0 / > 0 (float comparisons, as the projection makes them).
// Index 0 is left out (it is every pixel's starting candidate), and so are
// vectors of zero or non-finite length (their angle is NaN and never wins).
// Unit vectors in double pick the cell; G ~ sqrt(n) / 3 puts about two
// candidates in a cell that the sphere crosses.
void buildSphereGrids(EyeDev& e, const std::vector<Ommatidium>& omm, cudaStream_t st) {
  const size_t N = omm.size();
  for (int which = 0; which < 4; ++which) {
    SphereGrid& g = e.grids[which];
    std::vector<uint32_t> idx;
    std::vector<std::array<double, 3>> unit;
    for (size_t i = 1; i < N; ++i) {
      const Ommatidium& o = omm[i];
      if (which == 2 && !(o.pos.x < 0.f)) continue;
      if (which == 3 && !(o.pos.x > 0.f)) continue;
      const f3 v = which == 0 ? o.pos : o.dir;
      const double x = v.x, y = v.y, z = v.z, l = std::sqrt(x * x + y * y + z * z);
      if (!(l > 0.0) || !std::isfinite(l)) continue;
      idx.push_back(static_cast<uint32_t>(i));
      unit.push_back({x / l, y / l, z / l});
    }
    g.start.release();
    g.items.release();
    g.G = 0;
    if (idx.empty()) continue;
    const int G = std::max(1, std::min(128, static_cast<int>(std::lround(0.33 * std::sqrt(double(idx.size()))))));
    const size_t cells = static_cast<size_t>(G) * G * G;
    std::vector<uint32_t> cellOf(idx.size()), start(cells + 1, 0), items(idx.size());
    for (size_t k = 0; k < idx.size(); ++k) {
      int c[3];
      for (int a = 0; a < 3; ++a)
        c[a] = std::min(G - 1, std::max(0, static_cast<int>(std::floor((unit[k][a] + 1.0) * 0.5 * G))));
      cellOf[k] = static_cast<uint32_t>((static_cast<size_t>(c[2]) * G + c[1]) * G + c[0]);
      ++start[cellOf[k] + 1];
    }
    for (size_t c = 0; c < cells; ++c) start[c + 1] += start[c];
    std::vector<uint32_t> fill(start.begin(), start.end() - 1);
    for (size_t k = 0; k < idx.size(); ++k) items[fill[cellOf[k]]++] = idx[k];
    g.start.ensure(cells + 1);
    g.items.ensure(items.size());
    check(cudaMemcpyAsync(g.start.ptr, start.data(), start.size() * 4, cudaMemcpyHostToDevice, st), "cudaMemcpy");
    check(cudaMemcpyAsync(g.items.ptr, items.data(), items.size() * 4, cudaMemcpyHostToDevice, st), "cudaMemcpy");
    check(cudaStreamSynchronize(st), "projection grid upload");
    g.G = G;
  }
  e.gridsBuilt = true;
}

constexpr uint32_t kMaxPosesPerLaunch = 256;
constexpr size_t kTuneSlots = 20;

// Order in which warp segments take an eye's ommatidia: by the 30-bit Morton
// code of the unit axis direction mapped into the cube [0, 1)^3 (ties by
// index), so a warp holding several ommatidia traces neighbouring directions.
std::vector<uint32_t> directionOrder(const std::vector<Ommatidium>& omm) {
  auto spread = [](uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
  };
  std::vector<std::pair<uint32_t, uint32_t>> keys(omm.size());
  for (size_t i = 0; i < omm.size(); ++i) {
    const f3 d = omm[i].dir;
    const double len = std::sqrt(double(d.x) * d.x + double(d.y) * d.y + double(d.z) * d.z);
    uint32_t q[3] = {0, 0, 0};
    const double c[3] = {d.x, d.y, d.z};
    for (int k = 0; k < 3; ++k) {
      const double u = len > 0 ? 0.5 + 0.5 * c[k] / len : 0.5;
      q[k] = static_cast<uint32_t>(std::min(1023.0, std::max(0.0, std::floor(u * 1024.0))));
    }
    keys[i] = {spread(q[0]) | (spread(q[1]) << 1) | (spread(q[2]) << 2), static_cast<uint32_t>(i)};
  }
  std::sort(keys.begin(), keys.end());
  std::vector<uint32_t> out(omm.size());
  for (size_t i = 0; i < omm.size(); ++i) out[i] = keys[i].second;
  return out;
}

// Bound on |position - focal offset * unit axis| over an eye's ommatidia
// (how far a ray origin can lie from the pose position, in eye units),
// widened by 0.1% + 1e-6 so the near-field cut's guaranteed radius stays
// conservative after float rounding.
float maxRelOf(const std::vector<Ommatidium>& omm) {
  float mr = 0.f;
  for (const Ommatidium& o : omm) {
    const double al = std::sqrt(double(o.dir.x) * o.dir.x + double(o.dir.y) * o.dir.y + double(o.dir.z) * o.dir.z);
    const double s = al > 0 ? o.focalPointOffset / al : 0.0;
    const double rx = o.pos.x - s * o.dir.x, ry = o.pos.y - s * o.dir.y, rz = o.pos.z - s * o.dir.z;
    mr = std::max(mr, static_cast<float>(std::sqrt(rx * rx + ry * ry + rz * rz) * 1.001 + 1e-6));
  }
  return mr;
}

void releaseBatches();

struct Renderer {
  SceneData scene;
  bool loaded = false;
  // The BVH is built on the host by loadGlTFscene and uploaded by the first
  // call that needs the GPU, so every host-side entry point works without one.
  std::unique_ptr<HostBvh> pendingBvh;
  bool pendingGpuBuild = false;
  int builder = 0;  // 0 = host binned SAH, 1 = GPU linear BVH (crSetBvhBuilder)
  BvhBuildStats bvhStats;
  DevBuf<float4> nodes, tris, shade;
  int bvhWidth = 2;   // crSetBvhWidth: 2 (the BVH2), 4 or 8 (wide BVH with quantised boxes)
  int wideBuilt = 0;  // width of the wide BVH in wnodes (0: none)
  uint32_t nodeSlots = 0;  // BVH2 nodes in the uploaded node array
  DevBuf<float4> wnodes;
  WideBvhStats wideStats;
  DevBuf<uint32_t> texels;
  DevBuf<int4> texTable;
  DevBuf<float4> light;  // lighting-on data, uploaded when lighting is first used
  bool lighting = false;  // crSetLighting; off as in the reference (libEyeRenderer.cpp:98)
  DevScene dev;
  std::vector<EyeDev> eyes;  // parallel to scene.cameras
  size_t current = 0;
  int width = 400, height = 400;
  DevBuf<uchar4> frame;
  std::vector<uchar4> hostFrame;
  DevBuf<float4> poses;
  DevBuf<float> scratch;
  DevBuf<float2> draws;  // pre-drawn random numbers of small-eye launches
  DevBuf<float4> cuts;   // per-pose near-field cuts
  float cutFactor = 0.f; // cut radius as a fraction of the scene extent (0: off)
  // Timings of the last crAutotune (ms): variants 0-2, block 128/256/512,
  // samples per warp 8/16/32, cut radius 0, 1/256 .. 1/16 of the extent.
  std::vector<float> tuneTimes;
  bool projectionGrid = true;  // spherical projections search candidate grids (false: every candidate)
  DevBuf<float> batchOut;
  DevBuf<uint32_t> err;
  cudaStream_t ownStream = nullptr;
  cudaStream_t userStream = nullptr;
  bool verbose = true;
  // Bumped whenever device buffers an existing batch points into may change.
  uint64_t generation = 0;

  cudaStream_t stream() {
    if (userStream) return userStream;
    if (!ownStream) check(cudaStreamCreateWithFlags(&ownStream, cudaStreamNonBlocking), "cudaStreamCreate");
    return ownStream;
  }

  void releaseAll() {
    ++generation;
    releaseBatches();
    for (EyeDev& e : eyes) e.release();
    eyes.clear();
    nodes.release();
    tris.release();
    shade.release();
    wnodes.release();
    wideBuilt = 0;
    nodeSlots = 0;
    texels.release();
    texTable.release();
    light.release();
    frame.release();
    poses.release();
    scratch.release();
    draws.release();
    batchOut.release();
    err.release();
    hostFrame.clear();
    dev = DevScene{};
    pendingBvh.reset();
    pendingGpuBuild = false;
    if (ownStream) cudaStreamDestroy(ownStream);
    ownStream = nullptr;
    loaded = false;
    scene = SceneData{};
    current = 0;
  }

  // GPU construction (lbvh.cu) from the flattened scene.
  void buildOnDevice() {
    const uint32_t T = static_cast<uint32_t>(scene.triangleCount());
    DevBuf<float> v, c;
    DevBuf<uint8_t> f;
    DevBuf<char> temp;
    v.ensure(scene.triVerts.size());
    c.ensure(scene.triColours.size());
    f.ensure(T);
    temp.ensure(lbvhTempBytes(T));
    nodes.ensure(4 * static_cast<size_t>(T - 1));
    nodeSlots = T - 1;
    tris.ensure(3 * static_cast<size_t>(T));
    shade.ensure(3 * static_cast<size_t>(T));
    cudaStream_t st = stream();
    check(cudaMemcpyAsync(v.ptr, scene.triVerts.data(), scene.triVerts.size() * 4, cudaMemcpyHostToDevice, st), "cudaMemcpy");
    check(cudaMemcpyAsync(c.ptr, scene.triColours.data(), scene.triColours.size() * 4, cudaMemcpyHostToDevice, st),
          "cudaMemcpy");
    check(cudaMemcpyAsync(f.ptr, scene.triShading.data(), T, cudaMemcpyHostToDevice, st), "cudaMemcpy");
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t t = 0; t < T; ++t)
      for (int k = 0; k < 3; ++k) {
        const float* p = &scene.triVerts[9 * static_cast<size_t>(t)];
        const float a = std::min({p[k], p[3 + k], p[6 + k]}), b = std::max({p[k], p[3 + k], p[6 + k]});
        const float cen = 0.5f * a + 0.5f * b;
        lo[k] = std::min(lo[k], cen);
        hi[k] = std::max(hi[k], cen);
      }
    uint32_t stats[3] = {0, 0, 0};
    const cudaError_t e = buildLbvh(v.ptr, c.ptr, f.ptr, T, lo, hi, nodes.ptr, tris.ptr, shade.ptr, temp.ptr, stats, st);
    v.release();
    c.release();
    f.release();
    temp.release();
    check(e, "GPU BVH build");
    bvhStats.innerNodes = stats[0];
    bvhStats.leaves = stats[1];
    bvhStats.maxDepth = stats[2];
    if (stats[2] + 2 > 64) throw std::runtime_error("GPU-built BVH deeper than the traversal stack");
  }

  void ensureUploaded() {
    ensureBase();
    ensureWide();
  }

  // The wide BVH of the selected width (crSetBvhWidth), collapsed on the host
  // from the two-wide BVH on the device when first needed.
  void ensureWide() {
    const uint32_t T = dev.triCount;
    if (bvhWidth == 2 || T == 0 || nodeSlots == 0) {
      dev.width = 2;
      dev.wnodes = nullptr;
      return;
    }
    if (wideBuilt != bvhWidth) {
      const uint32_t inner = nodeSlots;  // the node array (the GPU builder leaves unused slots in it)
      std::vector<float> hn(16 * static_cast<size_t>(inner)), ht(12 * static_cast<size_t>(T));
      cudaStream_t st = stream();
      check(cudaMemcpyAsync(hn.data(), nodes.ptr, hn.size() * 4, cudaMemcpyDeviceToHost, st), "cudaMemcpy");
      check(cudaMemcpyAsync(ht.data(), tris.ptr, ht.size() * 4, cudaMemcpyDeviceToHost, st), "cudaMemcpy");
      check(cudaStreamSynchronize(st), "BVH readback");
      std::vector<float> w;
      collapseWideBvh(hn.data(), inner, ht.data(), T, bvhWidth, w, wideStats);
      if (static_cast<int>(wideStats.maxDepth + 1) * (bvhWidth - 1) + 1 > kWideStackEntries)
        throw std::runtime_error("wide BVH deeper than its traversal stack");
      wnodes.release();
      wnodes.ensure(w.size() / 4);
      check(cudaMemcpyAsync(wnodes.ptr, w.data(), w.size() * 4, cudaMemcpyHostToDevice, st), "cudaMemcpy");
      check(cudaStreamSynchronize(st), "wide BVH upload");
      wideBuilt = bvhWidth;
    }
    dev.width = bvhWidth;
    dev.wnodes = wnodes.ptr;
  }

  void ensureBase() {
    if (pendingGpuBuild) {
      buildOnDevice();
      pendingGpuBuild = false;
      pendingBvh.reset();
      finishUpload();
      return;
    }
    if (!pendingBvh) return;
    const HostBvh& b = *pendingBvh;
    const size_t nn = b.nodes.size() / 4, nt = b.tris.size() / 4;
    nodeSlots = static_cast<uint32_t>(nn / 4);
    nodes.ensure(std::max<size_t>(1, nn));
    tris.ensure(std::max<size_t>(1, nt));
    shade.ensure(std::max<size_t>(1, nt));
    cudaStream_t st = stream();
    if (nn) check(cudaMemcpyAsync(nodes.ptr, b.nodes.data(), nn * sizeof(float4), cudaMemcpyHostToDevice, st), "cudaMemcpy");
    if (nt) {
      check(cudaMemcpyAsync(tris.ptr, b.tris.data(), nt * sizeof(float4), cudaMemcpyHostToDevice, st), "cudaMemcpy");
      check(cudaMemcpyAsync(shade.ptr, b.shade.data(), nt * sizeof(float4), cudaMemcpyHostToDevice, st), "cudaMemcpy");
    }
    check(cudaStreamSynchronize(st), "scene upload");
    pendingBvh.reset();
    finishUpload();
  }

  void finishUpload() {
    dev.nodes = nodes.ptr;
    dev.tris = tris.ptr;
    dev.shade = shade.ptr;
    dev.triCount = static_cast<uint32_t>(scene.triangleCount());
    dev.miss = static_cast<int>(scene.miss);
    if (!scene.textures.empty()) {
      std::vector<int4> table;
      for (const Texture& t : scene.textures) table.push_back(make_int4(static_cast<int>(t.offset), t.width, t.height, 0));
      texels.ensure(scene.texels.size());
      texTable.ensure(table.size());
      cudaStream_t st = stream();
      check(cudaMemcpyAsync(texels.ptr, scene.texels.data(), scene.texels.size() * 4, cudaMemcpyHostToDevice, st),
            "cudaMemcpy");
      check(cudaMemcpyAsync(texTable.ptr, table.data(), table.size() * sizeof(int4), cudaMemcpyHostToDevice, st),
            "cudaMemcpy");
      check(cudaStreamSynchronize(st), "texture upload");
    }
    dev.texels = texels.ptr;
    dev.texTable = texTable.ptr;
    applyLighting();
    float ext = 0.f;
    for (float v : scene.triVerts) ext = std::max(ext, std::fabs(v));
    dev.extent = ext;
  }

  // Lighting-on state of the device scene: the per-triangle data (uploaded on
  // first use) and the four point lights of libEyeRenderer.cpp:100-118, placed
  // around the scene's bounding box (centre c, largest extent e):
  //   c + (e, e, e), c + (-e, e/2, -e/2), c + (0, 4, -5), c + (1, -6, 0).
  void applyLighting() {
    dev.lighting = 0;
    dev.light = nullptr;
    if (!lighting || !loaded || scene.triangleCount() == 0) return;
    if (!light.ptr) {
      const size_t n = scene.triLight.size() / 4;
      light.ensure(n);
      check(cudaMemcpyAsync(light.ptr, scene.triLight.data(), n * sizeof(float4), cudaMemcpyHostToDevice, stream()),
            "cudaMemcpy");
      check(cudaStreamSynchronize(stream()), "lighting upload");
    }
    lightSetup(scene, dev.lightPos, dev.lightCol);
    dev.light = light.ptr;
    dev.lighting = 1;
  }

  static void lightSetup(const SceneData& sc, float4* pos, float4* col) {
    const f3 lo = sc.sceneMin, hi = sc.sceneMax;
    const float cx = (lo.x + hi.x) * 0.5f, cy = (lo.y + hi.y) * 0.5f, cz = (lo.z + hi.z) * 0.5f;
    const float e = std::max(hi.x - lo.x, std::max(hi.y - lo.y, hi.z - lo.z));
    pos[0] = make_float4(cx + e, cy + e, cz + e, 5.0f);
    pos[1] = make_float4(cx - e, cy + 0.5f * e, cz - 0.5f * e, 3.0f);
    pos[2] = make_float4(cx + 0.0f, cy + 4.0f, cz - 5.0f, 5.0f);
    pos[3] = make_float4(cx + 1.0f, cy - 6.0f, cz + 0.0f, 0.5f);
    col[0] = make_float4(1.0f, 1.0f, 0.8f, 0.f);
    col[1] = make_float4(0.8f, 0.8f, 1.0f, 0.f);
    col[2] = make_float4(1.0f, 1.0f, 0.8f, 0.f);
    col[3] = make_float4(1.0f, 1.0f, 0.8f, 0.f);
  }

  void requireUnlit(const char* what) const {
    if (lighting) throw std::runtime_error(std::string(what) + " renders with lighting off only (crSetLighting(0))");
  }

  Camera& cam() {
    if (!loaded || scene.cameras.empty()) throw std::runtime_error("no scene loaded");
    return scene.cameras[current];
  }
  bool compoundActive() const {
    return loaded && !scene.cameras.empty() && scene.cameras[current].kind == CameraKind::Compound;
  }

  void ensureFrame() {
    const size_t n = static_cast<size_t>(width) * static_cast<size_t>(height);
    if (frame.count != n) {
      frame.release();
      frame.ensure(n);
      if (n) check(cudaMemsetAsync(frame.ptr, 0, n * sizeof(uchar4), stream()), "cudaMemset");
    }
  }

  uint32_t* errWord() {
    if (!err.ptr) {
      err.ensure(1);
      check(cudaMemsetAsync(err.ptr, 0, sizeof(uint32_t), stream()), "cudaMemset");
    }
    return err.ptr;
  }

  void checkErrWord() {
    uint32_t h = 0;
    check(cudaMemcpyAsync(&h, errWord(), sizeof(uint32_t), cudaMemcpyDeviceToHost, stream()), "cudaMemcpy");
    check(cudaStreamSynchronize(stream()), "render");
    if (h != 0) {
      check(cudaMemsetAsync(errWord(), 0, sizeof(uint32_t), stream()), "cudaMemset");
      throw std::runtime_error("render kernel raised error flags " + std::to_string(h) +
                               ((h & kErrStackOverflow) ? " (BVH traversal stack overflow)" : "") +
                               ((h & kErrMmaTimeout) ? " (tensor-core wait timed out)" : ""));
    }
  }

  // Makes the device side of compound camera `i` match its host record.
  EyeDev& syncEye(size_t i) {
    ensureUploaded();
    Camera& c = scene.cameras[i];
    EyeDev& e = eyes[i];
    const uint32_t N = static_cast<uint32_t>(c.omm.size());
    const uint32_t spp = static_cast<uint32_t>(std::max(1, c.spp));
    if (e.N != N || e.spp != spp || !e.omm.ptr) {
      const bool countChanged = e.N != N || !e.omm.ptr;
      if (countChanged) {
        e.omm.release();
        e.omm.ensure(std::max<size_t>(1, 2 * static_cast<size_t>(N)));
        e.sums.release();
        e.sums.ensure(std::max<size_t>(1, 3 * static_cast<size_t>(N)));
      }
      ++generation;
      e.rng.release();
      e.rng.ensure(std::max<size_t>(1, static_cast<size_t>(kRngPlanes) * N * spp));
      e.N = N;
      e.spp = spp;
      e.configured = false;
      e.haveSums = false;
      e.releaseGrids();
      if (N) check(cudaMemcpyAsync(e.omm.ptr, c.omm.data(), sizeof(Ommatidium) * N, cudaMemcpyHostToDevice, stream()),
                   "cudaMemcpy");
      if (countChanged) {
        e.order.release();
        e.order.ensure(std::max<size_t>(1, N));
      }
      e.maxRel = maxRelOf(c.omm);
      if (N) {
        const std::vector<uint32_t> ord = directionOrder(c.omm);
        check(cudaMemcpyAsync(e.order.ptr, ord.data(), 4 * static_cast<size_t>(N), cudaMemcpyHostToDevice, stream()),
              "cudaMemcpy");
        check(cudaStreamSynchronize(stream()), "eye upload");
      }
    }
    return e;
  }

  DevEye devEye(EyeDev& e) {
    DevEye d;
    d.omm = e.omm.ptr;
    d.N = e.N;
    d.spp = e.spp;
    d.rng = e.rng.ptr;
    d.order = e.order.ptr;
    return d;
  }

  void ensureRng(EyeDev& e) {
    if (e.configured) return;
    check(launchRngInit(devEye(e), errWord(), stream()), "rng init launch");
    e.configured = true;
  }

  static void packPose(const Camera& c, float* p16) {
    const f3 v[4] = {c.position, c.ls.x, c.ls.y, c.ls.z};
    for (int k = 0; k < 4; ++k) {
      p16[4 * k + 0] = v[k].x;
      p16[4 * k + 1] = v[k].y;
      p16[4 * k + 2] = v[k].z;
      p16[4 * k + 3] = 0.f;
    }
  }

  // Renders `count` poses already on the device into d_out (count x N x 3).
  void renderDevicePoses(EyeDev& e, const float4* d_poses, size_t count, float* d_out, RayRecord* rec,
                         unsigned long long* stats = nullptr) {
    ensureRng(e);
    for (size_t first = 0; first < count; first += kMaxPosesPerLaunch) {
      const uint32_t P = static_cast<uint32_t>(std::min<size_t>(kMaxPosesPerLaunch, count - first));
      const size_t need = renderScratchFloats(dev, e.N, e.spp, P, rec != nullptr, stats != nullptr);
      if (need) scratch.ensure(need);
      DevEye de = devEye(e);
      withDraws(de, P, !rec && !stats);
      withCuts(de, P, e.maxRel);
      check(launchRender(dev, de, d_poses + 4 * first, P, d_out + 3 * first * e.N, need ? scratch.ptr : nullptr,
                         errWord(), rec, stream(), stats),
            "render launch");
    }
  }

  // Near-field cuts for a P-pose launch when a cut radius is set and the
  // traversal stack has room for the cut entries above the deepest leaf.
  void withCuts(DevEye& de, uint32_t P, float maxRel) {
    de.cuts = nullptr;
    if (!(cutFactor > 0.f) || !(dev.extent > 0.f)) return;
    if (bvhStats.maxDepth + kCutEntries + 2 > 64) return;
    cuts.ensure(static_cast<size_t>(P) * kCutStride);
    de.cuts = cuts.ptr;
    de.cutRadius = cutFactor * dev.extent;
    de.maxRel = maxRel;
  }

  // Gives a P-pose launch of a small eye a buffer for its pre-drawn random
  // numbers, so that its poses spread over more warps (renderDrawBytes).
  void withDraws(DevEye& de, uint32_t P, bool allowed) {
    de.draws = nullptr;
    if (!allowed) return;
    const size_t bytes = renderDrawBytes(de.N, de.spp, P);
    if (!bytes) return;
    draws.ensure(bytes / sizeof(float2));
    de.draws = draws.ptr;
  }

  // Compound projection shaders by name (the reference's
  // "__raygen__compound_projection_" programs without the prefix).
  static int projectionKind(const std::string& shader) {
    if (shader == "single_dimension_fast") return 0;
    if (shader == "single_dimension") return 1;
    if (shader == "spherical_positionwise") return 10;
    if (shader == "spherical_orientationwise") return 11;
    if (shader == "spherical_split_orientationwise") return 12;
    if (shader == "spherical_orientationwise_ids") return 13;
    if (shader == "spherical_positionwise_ids") return 14;
    if (shader == "raw_ommatidial_samples") return 20;
    throw std::runtime_error("unknown compound projection '" + shader + "'");
  }

  void project(EyeDev& e, const std::vector<Ommatidium>& omm, const std::string& shader, const RayRecord* rec) {
    ensureFrame();
    const int kind = projectionKind(shader);
    if (kind < 10) {
      check(launchProject(e.sums.ptr, e.N, frame.ptr, width, height, kind, stream()), "projection launch");
    } else if (kind < 20) {
      SphereGridSet set;
      if (projectionGrid) {
        if (!e.gridsBuilt) buildSphereGrids(e, omm, stream());
        for (int k = 0; k < 4; ++k) {
          set.g[k].start = e.grids[k].start.ptr;
          set.g[k].items = e.grids[k].items.ptr;
          set.g[k].G = e.grids[k].G;
        }
      }
      DevBuf<float> len;
      len.ensure(std::max<size_t>(1, 2 * static_cast<size_t>(e.N)));
      check(launchSpherical(e.omm.ptr, len.ptr, e.N, e.sums.ptr, frame.ptr, width, height, kind - 10,
                            projectionGrid ? &set : nullptr, stream()),
            "projection launch");
      check(cudaStreamSynchronize(stream()), "projection");
      len.release();
    } else {
      check(launchRawSamples(rec, e.N, e.spp, frame.ptr, width, height, stream()), "projection launch");
    }
  }
};

Renderer& R() {
  static Renderer r;
  return r;
}

// A batch of eyes recorded as one CUDA graph (see crBatchCreate).
struct Batch {
  std::vector<int> cams;
  size_t P = 0;
  std::vector<size_t> outOffset;  // floats, per camera
  DevBuf<BatchEye> table;
  DevBuf<unsigned long long> taskBase, cellBase, ctrl;
  DevBuf<float> scratch;
  DevBuf<float4> cuts;  // per eye P x kCutStride, when the near-field cut is on
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned long long totalTasks = 0, totalCells = 0;
  uint32_t cutPoses = 0;
  int variant = 0, grid = 0;
  uint64_t generation = 0;
  void release() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    table.release();
    taskBase.release();
    cellBase.release();
    ctrl.release();
    scratch.release();
    cuts.release();
  }
};

std::map<int, Batch>& batches() {
  static std::map<int, Batch> b;
  return b;
}

void releaseBatches() {
  for (auto& kv : batches()) kv.second.release();
  batches().clear();
}

thread_local std::string g_lastError;

void setError(const std::string& msg) {
  g_lastError = msg;
  std::cerr << "[libEyeRenderer3] ERROR: " << msg << std::endl;
}

template <typename F>
auto guarded(const char* fn, F&& f, decltype(f()) fallback) -> decltype(f()) {
  try {
    return f();
  } catch (const std::exception& ex) {
    setError(std::string(fn) + ": " + ex.what());
  } catch (...) {
    setError(std::string(fn) + ": unknown error");
  }
  return fallback;
}

template <typename F>
void guardedVoid(const char* fn, F&& f) {
  try {
    f();
  } catch (const std::exception& ex) {
    setError(std::string(fn) + ": " + ex.what());
  } catch (...) {
    setError(std::string(fn) + ": unknown error");
  }
}

}  // namespace
}  // namespace cr

using namespace cr;

extern "C" {

void setVerbosity(bool v) { R().verbose = v; }

void loadGlTFscene(const char* filepath) {
  guardedVoid("loadGlTFscene", [&] {
    if (!filepath) throw std::runtime_error("null path");
    Renderer& r = R();
    SceneData s;
    loadGltfScene(filepath, s, r.verbose);
    // GPU construction needs a handful of triangles at least; tiny scenes
    // always use the host builder.
    const bool gpuBuild = r.builder == 1 && s.triangleCount() >= 16;
    std::unique_ptr<HostBvh> bvh(new HostBvh);
    if (!gpuBuild) {
      buildBvh(s.triVerts.data(), s.triColours.data(), s.triShading.data(),
               static_cast<uint32_t>(s.triangleCount()), *bvh);
      if (bvh->stats.maxDepth + 2 > 64) throw std::runtime_error("BVH deeper than the traversal stack");
    }
    const bool keepVerbose = r.verbose;
    cudaStream_t user = r.userStream;
    r.releaseAll();
    r.verbose = keepVerbose;
    r.userStream = user;
    r.scene = std::move(s);
    r.bvhStats = bvh->stats;
    r.pendingBvh = std::move(bvh);
    r.pendingGpuBuild = gpuBuild;
    r.eyes.resize(r.scene.cameras.size());
    r.current = 0;
    r.loaded = true;
    if (r.verbose)
      std::cout << "[PyEye] Loaded scene '" << filepath << "': " << r.scene.triangleCount() << " triangles, "
                << r.scene.cameras.size() << " cameras, BVH " << r.bvhStats.innerNodes << " inner nodes / "
                << r.bvhStats.leaves << " leaves, depth " << r.bvhStats.maxDepth << "." << std::endl;
  });
}

void stop(void) {
  guardedVoid("stop", [&] {
    Renderer& r = R();
    if (r.verbose) std::cout << "[PyEye] Cleaning eye renderer resources." << std::endl;
    const bool v = r.verbose;
    r.releaseAll();
    r.userStream = nullptr;
    r.verbose = v;
  });
}

void setRenderSize(int w, int h) {
  guardedVoid("setRenderSize", [&] {
    Renderer& r = R();
    r.width = std::max(0, w);
    r.height = std::max(0, h);
    if (r.verbose) std::cout << "[PyEye] Resizing rendering buffer to (" << w << ", " << h << ")." << std::endl;
    r.hostFrame.clear();
  });
}

double renderFrame(void) {
  return guarded(
      "renderFrame",
      [&]() -> double {
        Renderer& r = R();
        Camera& c = r.cam();
        const auto t0 = std::chrono::steady_clock::now();
        r.ensureFrame();
        if (c.kind == CameraKind::Compound) {
          EyeDev& e = r.syncEye(r.current);
          float p16[16];
          Renderer::packPose(c, p16);
          r.poses.ensure(4);
          check(cudaMemcpyAsync(r.poses.ptr, p16, sizeof(p16), cudaMemcpyHostToDevice, r.stream()), "cudaMemcpy");
          // raw_ommatidial_samples shows individual samples: that projection
          // renders through the recording variant, which keeps them.
          const bool raw = Renderer::projectionKind(c.projection) == 20;
          DevBuf<RayRecord> rec;
          if (raw) rec.ensure(std::max<size_t>(1, static_cast<size_t>(e.N) * e.spp));
          r.renderDevicePoses(e, r.poses.ptr, 1, e.sums.ptr, raw ? rec.ptr : nullptr);
          e.haveSums = true;
          r.project(e, c.omm, c.projection, rec.ptr);
          if (raw) {
            check(cudaStreamSynchronize(r.stream()), "projection");
            rec.release();
          }
        } else {
          throw std::runtime_error("camera '" + c.name +
                                   "' is not a compound eye; only compound eyes are rendered by this library");
        }
        r.checkErrWord();
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        r.hostFrame.clear();
        if (r.verbose) std::cout << "[PyEye] Rendered frame in " << ms << "ms." << std::endl;
        return ms;
      },
      -1.0);
}

void displayFrame(void) {}

unsigned char* getFramePointer(void) {
  return guarded(
      "getFramePointer",
      [&]() -> unsigned char* {
        Renderer& r = R();
        if (r.verbose) std::cout << "[PyEye] Retrieving frame pointer..." << std::endl;
        const size_t n = static_cast<size_t>(r.width) * static_cast<size_t>(r.height);
        r.hostFrame.assign(std::max<size_t>(n, 1), make_uchar4(0, 0, 0, 0));
        if (n && r.loaded) {
          r.ensureFrame();
          check(cudaMemcpyAsync(r.hostFrame.data(), r.frame.ptr, n * sizeof(uchar4), cudaMemcpyDeviceToHost, r.stream()),
                "cudaMemcpy");
          check(cudaStreamSynchronize(r.stream()), "frame download");
        }
        return reinterpret_cast<unsigned char*>(r.hostFrame.data());
      },
      nullptr);
}

void saveFrameAs(char* ppmFilename) {
  guardedVoid("saveFrameAs", [&] {
    if (!ppmFilename) throw std::runtime_error("null file name");
    Renderer& r = R();
    const bool v = r.verbose;
    r.verbose = false;
    unsigned char* px = getFramePointer();
    r.verbose = v;
    if (!px) throw std::runtime_error("no frame");
    const int w = r.width, h = r.height;
    if (w < 1 || h < 1) throw std::invalid_argument("Image is ill-formed. Not saving");
    std::ofstream f(ppmFilename, std::ios::out | std::ios::binary);
    if (!f.is_open()) throw std::runtime_error("Could not open file for SavePPM");
    f << "P6\n" << w << " " << h << "\n255\n";
    std::vector<unsigned char> row(static_cast<size_t>(w) * 3);
    // The buffer is stored bottom row first (sutil/sutil.cpp:404-418).
    for (int j = h - 1; j >= 0; --j) {
      const unsigned char* src = px + static_cast<size_t>(4) * w * j;
      for (int i = 0; i < w; ++i) {
        row[3 * i + 0] = src[4 * i + 0];
        row[3 * i + 1] = src[4 * i + 1];
        row[3 * i + 2] = src[4 * i + 2];
      }
      f.write(reinterpret_cast<const char*>(row.data()), static_cast<std::streamsize>(row.size()));
    }
    if (r.verbose) std::cout << "[PyEye] Saved render as '" << ppmFilename << "'" << std::endl;
  });
}

size_t getCameraCount(void) {
  return guarded("getCameraCount", [&]() -> size_t { return R().loaded ? R().scene.cameras.size() : 0; }, size_t{0});
}

static void setCurrentCameraIndex(long idx) {
  Renderer& r = R();
  const long n = static_cast<long>(r.scene.cameras.size());
  if (n == 0) throw std::runtime_error("no scene loaded");
  r.current = static_cast<size_t>(((idx % n) + n) % n);
}

void nextCamera(void) {
  guardedVoid("nextCamera", [&] { setCurrentCameraIndex(static_cast<long>(R().current) + 1); });
}
void previousCamera(void) {
  guardedVoid("previousCamera", [&] { setCurrentCameraIndex(static_cast<long>(R().current) - 1); });
}
size_t getCurrentCameraIndex(void) { return R().current; }
const char* getCurrentCameraName(void) {
  return guarded("getCurrentCameraName", [&]() -> const char* { return R().cam().name.c_str(); }, "");
}
void gotoCamera(int index) {
  guardedVoid("gotoCamera", [&] { setCurrentCameraIndex(index); });
}
bool gotoCameraByName(char* name) {
  return guarded(
      "gotoCameraByName",
      [&]() -> bool {
        if (!name) return false;
        setCurrentCameraIndex(0);
        Renderer& r = R();
        for (size_t i = 0; i < r.scene.cameras.size(); ++i) {
          if (r.scene.cameras[r.current].name == name) return true;
          setCurrentCameraIndex(static_cast<long>(r.current) + 1);
        }
        return false;
      },
      false);
}

void setCameraPosition(float x, float y, float z) {
  guardedVoid("setCameraPosition", [&] { R().cam().position = f3{x, y, z}; });
}
void getCameraPosition(float& x, float& y, float& z) {
  guardedVoid("getCameraPosition", [&] {
    const f3 p = R().cam().position;
    x = p.x;
    y = p.y;
    z = p.z;
  });
}
void setCameraLocalSpace(float lxx, float lxy, float lxz, float lyx, float lyy, float lyz, float lzx, float lzy,
                         float lzz) {
  guardedVoid("setCameraLocalSpace", [&] {
    LocalSpace& ls = R().cam().ls;
    ls.x = f3{lxx, lxy, lxz};
    ls.y = f3{lyx, lyy, lyz};
    ls.z = f3{lzx, lzy, lzz};
  });
}

// DataRecordCamera.h:57-81.
static f3 toLocal(const LocalSpace& ls, f3 v) {
  return f3{v.x * ls.x.x + v.y * ls.y.x + v.z * ls.z.x, v.x * ls.x.y + v.y * ls.y.y + v.z * ls.z.y,
            v.x * ls.x.z + v.y * ls.y.z + v.z * ls.z.z};
}
static void rotateCam(Camera& c, float angle, f3 axis) {
  c.ls.x = rotateAboutAxis(c.ls.x, angle, axis);
  c.ls.y = rotateAboutAxis(c.ls.y, angle, axis);
  c.ls.z = rotateAboutAxis(c.ls.z, angle, axis);
}
static void moveCam(Camera& c, f3 s) { c.position = f3{c.position.x + s.x, c.position.y + s.y, c.position.z + s.z}; }

void rotateCameraAround(float angle, float x, float y, float z) {
  guardedVoid("rotateCameraAround", [&] { rotateCam(R().cam(), angle, f3{x, y, z}); });
}
void rotateCameraLocallyAround(float angle, float x, float y, float z) {
  guardedVoid("rotateCameraLocallyAround", [&] {
    Camera& c = R().cam();
    rotateCam(c, angle, toLocal(c.ls, f3{x, y, z}));
  });
}
void translateCamera(float x, float y, float z) {
  guardedVoid("translateCamera", [&] { moveCam(R().cam(), f3{x, y, z}); });
}
void translateCameraLocally(float x, float y, float z) {
  guardedVoid("translateCameraLocally", [&] {
    Camera& c = R().cam();
    moveCam(c, toLocal(c.ls, f3{x, y, z}));
  });
}
void resetCameraPose(void) {
  guardedVoid("resetCameraPose", [&] {
    Camera& c = R().cam();
    c.ls = LocalSpace{};
    c.position = f3{};
  });
}
void setCameraPose(float posX, float posY, float posZ, float rotX, float rotY, float rotZ) {
  // libEyeRenderer.cpp:380-388: reset, rotate about world X, Y, Z, translate.
  guardedVoid("setCameraPose", [&] {
    Camera& c = R().cam();
    c.ls = LocalSpace{};
    c.position = f3{};
    rotateCam(c, rotX, f3{1, 0, 0});
    rotateCam(c, rotY, f3{0, 1, 0});
    rotateCam(c, rotZ, f3{0, 0, 1});
    moveCam(c, f3{posX, posY, posZ});
  });
}

bool isCompoundEyeActive(void) { return R().compoundActive(); }

void setCurrentEyeSamplesPerOmmatidium(int s) {
  guardedVoid("setCurrentEyeSamplesPerOmmatidium", [&] {
    Renderer& r = R();
    if (!r.compoundActive()) return;
    r.scene.cameras[r.current].spp = std::max(1, s);
    // Reallocating the generator states resets them (CompoundEye.cpp:171-179).
    EyeDev& e = r.eyes[r.current];
    ++r.generation;
    e.rng.release();
    e.spp = 0;
    e.configured = false;
  });
}
int getCurrentEyeSamplesPerOmmatidium(void) {
  Renderer& r = R();
  if (!r.compoundActive()) return -1;
  return r.scene.cameras[r.current].spp;
}
void changeCurrentEyeSamplesPerOmmatidiumBy(int s) {
  Renderer& r = R();
  if (!r.compoundActive()) return;
  setCurrentEyeSamplesPerOmmatidium(r.scene.cameras[r.current].spp + s);
}
size_t getCurrentEyeOmmatidialCount(void) {
  Renderer& r = R();
  if (!r.compoundActive()) return 0;
  return r.scene.cameras[r.current].omm.size();
}
void setOmmatidia(OmmatidiumPacket* omms, size_t count) {
  guardedVoid("setOmmatidia", [&] {
    Renderer& r = R();
    if (!r.compoundActive()) return;
    if (count && !omms) throw std::runtime_error("null ommatidium array");
    Camera& c = r.scene.cameras[r.current];
    std::vector<Ommatidium> v(count);
    for (size_t i = 0; i < count; ++i) {
      const OmmatidiumPacket& p = omms[i];
      v[i] = Ommatidium{f3{p.posX, p.posY, p.posZ}, f3{p.dirX, p.dirY, p.dirZ}, p.acceptanceAngle, p.focalpointOffset};
    }
    EyeDev& e = r.eyes[r.current];
    if (count != c.omm.size()) {
      // A count change reallocates every eye buffer and resets the streams
      // (CompoundEye.cpp:35-48); the same count only copies the records in.
      ++r.generation;
      e.release();
    } else if (e.omm.ptr && count) {
      ++r.generation;  // tables built from the old ommatidia (neighbours, batches) are stale
      e.releaseGrids();
      check(cudaMemcpyAsync(e.omm.ptr, v.data(), sizeof(Ommatidium) * count, cudaMemcpyHostToDevice, r.stream()),
            "cudaMemcpy");
      const std::vector<uint32_t> ord = directionOrder(v);
      check(cudaMemcpyAsync(e.order.ptr, ord.data(), 4 * count, cudaMemcpyHostToDevice, r.stream()), "cudaMemcpy");
      check(cudaStreamSynchronize(r.stream()), "ommatidia upload");
      // The near-field cut's guaranteed radius depends on how far the ray
      // origins lie from the pose position: recompute it for the new records.
      e.maxRel = maxRelOf(v);
    }
    c.omm = std::move(v);
  });
}
const char* getCurrentEyeDataPath(void) {
  Renderer& r = R();
  if (!r.compoundActive()) return "";
  return r.scene.cameras[r.current].eyeDataPath.c_str();
}
void setCurrentEyeShaderName(char* name) {
  guardedVoid("setCurrentEyeShaderName", [&] {
    Renderer& r = R();
    if (!r.compoundActive() || !name) return;
    r.scene.cameras[r.current].projection = name;
  });
}

bool isInsideHitGeometry(float x, float y, float z, char* name) {
  return guarded(
      "isInsideHitGeometry",
      [&]() -> bool {
        if (!name) return false;
        for (const HitboxMesh& h : R().scene.hitboxes)
          if (h.name == name) return pointInsideHitbox(h, f3{x, y, z});
        std::cerr << "WARNING: No hitbox with the given name \"" << name << "\" is present in the scene." << std::endl;
        return false;
      },
      false);
}

// (y, z) grid of a hitbox mesh's object-space triangles for the batched
// inside query (InsideQuery).  A triangle is listed in every cell that its
// (y, z) box meets after widening by 1e-5 of (mesh extent + largest
// coordinate): the parity cast counts a triangle only where its point lies
// in the triangle's (y, z) projection up to double rounding, far inside that
// margin, so the cell of any point holds every triangle the full loop could
// count for it.  About two triangles per cell, at most 256 x 256 cells.
struct HitGrid {
  std::vector<uint32_t> start, items;
  std::vector<uint32_t> everywhere;  // triangles tested for every point (non-finite cast normal)
  double y0 = 0.0, z0 = 0.0, inv = 0.0;
  int G = 0;
};

HitGrid buildHitGrid(const HitboxMesh& m) {
  HitGrid g;
  const size_t nt = m.tris.size() / 3;
  if (nt == 0) return g;
  double ylo = INFINITY, yhi = -INFINITY, zlo = INFINITY, zhi = -INFINITY, big = 0.0;
  for (const f3& v : m.tris) {
    ylo = std::min(ylo, double(v.y));
    yhi = std::max(yhi, double(v.y));
    zlo = std::min(zlo, double(v.z));
    zhi = std::max(zhi, double(v.z));
    big = std::max({big, std::fabs(double(v.x)), std::fabs(double(v.y)), std::fabs(double(v.z))});
  }
  if (!std::isfinite(ylo + yhi + zlo + zhi + big)) return g;  // non-finite vertices: test every triangle
  const double ext = std::max(yhi - ylo, zhi - zlo);
  const double eps = 1e-5 * (ext + big) + 1e-30;
  g.G = std::max(1, std::min(256, static_cast<int>(std::sqrt(double(nt) / 2.0))));
  g.y0 = ylo - eps;
  g.z0 = zlo - eps;
  const double size = ext + 2.0 * eps;
  g.inv = double(g.G) / size;
  auto cellOf = [&](double v, double v0) {
    const double c = std::floor((v - v0) * g.inv);
    return c < 0.0 ? 0 : (c >= double(g.G) ? g.G - 1 : static_cast<int>(c));
  };
  std::vector<int> box(4 * nt);
  std::vector<uint8_t> special(nt, 0);
  for (size_t t = 0; t < nt; ++t)
    if (hitboxTriangleCountsEverywhere(m, t)) {
      special[t] = 1;
      g.everywhere.push_back(static_cast<uint32_t>(t));
    }
  g.start.assign(static_cast<size_t>(g.G) * g.G + 1, 0);
  for (size_t t = 0; t < nt; ++t) {
    int* bx = &box[4 * t];
    if (special[t]) {  // in no cell: listed apart
      bx[0] = bx[2] = 0;
      bx[1] = bx[3] = -1;
      continue;
    }
    const f3 &a = m.tris[3 * t], &b = m.tris[3 * t + 1], &c = m.tris[3 * t + 2];
    const double y0 = std::min({double(a.y), double(b.y), double(c.y)}) - eps;
    const double y1 = std::max({double(a.y), double(b.y), double(c.y)}) + eps;
    const double z0 = std::min({double(a.z), double(b.z), double(c.z)}) - eps;
    const double z1 = std::max({double(a.z), double(b.z), double(c.z)}) + eps;
    bx[0] = cellOf(y0, g.y0);
    bx[1] = cellOf(y1, g.y0);
    bx[2] = cellOf(z0, g.z0);
    bx[3] = cellOf(z1, g.z0);
    for (int cz = bx[2]; cz <= bx[3]; ++cz)
      for (int cy = bx[0]; cy <= bx[1]; ++cy) ++g.start[static_cast<size_t>(cz) * g.G + cy + 1];
  }
  for (size_t c = 0; c + 1 < g.start.size(); ++c) g.start[c + 1] += g.start[c];
  g.items.resize(g.start.back());
  std::vector<uint32_t> fill(g.start.begin(), g.start.end() - 1);
  for (size_t t = 0; t < nt; ++t) {
    const int* bx = &box[4 * t];
    for (int cz = bx[2]; cz <= bx[3]; ++cz)
      for (int cy = bx[0]; cy <= bx[1]; ++cy) g.items[fill[static_cast<size_t>(cz) * g.G + cy]++] = static_cast<uint32_t>(t);
  }
  return g;
}

int crInsideHitGeometryBatch(const float* points, size_t n, const char* name, unsigned char* inside) {
  return guarded(
      "crInsideHitGeometryBatch",
      [&]() -> int {
        if (!name || (n && (!points || !inside))) throw std::runtime_error("null pointer");
        const HitboxMesh* hm = nullptr;
        for (const HitboxMesh& h : R().scene.hitboxes)
          if (h.name == name) hm = &h;
        if (!hm) throw std::runtime_error(std::string("no hitbox named '") + name + "'");
        if (n == 0) return 0;
        // Inverse transform exactly as pointInsideHitbox forms it.
        const double* x = hm->xform;
        const double a = x[0], b = x[1], c = x[2], d = x[4], e = x[5], f = x[6], g = x[8], h = x[9], i = x[10];
        const double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
        if (det == 0.0) {
          std::memset(inside, 0, n);
          return 0;
        }
        InsideQuery q;
        const double inv[9] = {(e * i - f * h) / det, (c * h - b * i) / det, (b * f - c * e) / det,
                               (f * g - d * i) / det, (a * i - c * g) / det, (c * d - a * f) / det,
                               (d * h - e * g) / det, (b * g - a * h) / det, (a * e - b * d) / det};
        std::memcpy(q.inv, inv, sizeof(inv));
        q.startX = hm->objMin.x - 1.0f;  // in float, as the reference's ray start
        Renderer& r = R();
        cudaStream_t st = r.stream();
        const uint32_t nt = static_cast<uint32_t>(hm->tris.size() / 3);
        DevBuf<float3> tri;
        DevBuf<float> pts;
        DevBuf<uint8_t> res;
        tri.ensure(std::max<size_t>(1, hm->tris.size()));
        pts.ensure(3 * n);
        res.ensure(n);
        static_assert(sizeof(f3) == sizeof(float3), "f3 and float3 share a layout");
        if (nt) check(cudaMemcpyAsync(tri.ptr, hm->tris.data(), nt * 3 * sizeof(float3), cudaMemcpyHostToDevice, st),
                      "cudaMemcpy");
        const HitGrid grid = buildHitGrid(*hm);
        DevBuf<uint32_t> cellStart, cellItems, everywhere;
        if (grid.G > 0) {
          cellStart.ensure(grid.start.size());
          cellItems.ensure(std::max<size_t>(1, grid.items.size()));
          check(cudaMemcpyAsync(cellStart.ptr, grid.start.data(), grid.start.size() * 4, cudaMemcpyHostToDevice, st),
                "cudaMemcpy");
          if (!grid.items.empty())
            check(cudaMemcpyAsync(cellItems.ptr, grid.items.data(), grid.items.size() * 4, cudaMemcpyHostToDevice, st),
                  "cudaMemcpy");
          q.cellStart = cellStart.ptr;
          q.cellItems = cellItems.ptr;
          if (!grid.everywhere.empty()) {
            everywhere.ensure(grid.everywhere.size());
            check(cudaMemcpyAsync(everywhere.ptr, grid.everywhere.data(), grid.everywhere.size() * 4,
                                  cudaMemcpyHostToDevice, st),
                  "cudaMemcpy");
            q.everywhere = everywhere.ptr;
            q.nEverywhere = static_cast<uint32_t>(grid.everywhere.size());
          }
          q.y0 = grid.y0;
          q.z0 = grid.z0;
          q.cellInv = grid.inv;
          q.G = grid.G;
        }
        check(cudaMemcpyAsync(pts.ptr, points, 3 * n * sizeof(float), cudaMemcpyHostToDevice, st), "cudaMemcpy");
        check(launchInside(tri.ptr, nt, q, pts.ptr, n, res.ptr, st), "hitbox query");
        check(cudaMemcpyAsync(inside, res.ptr, n, cudaMemcpyDeviceToHost, st), "cudaMemcpy");
        check(cudaStreamSynchronize(st), "hitbox query");
        return 0;
      },
      -1);
}

static float3 boundsByName(const char* name, bool wantMax) {
  if (!name) return make_float3(0.f, 0.f, 0.f);
  const SceneData& s = R().scene;
  for (const HitboxMesh& h : s.hitboxes)
    if (h.name == name) {
      const f3 v = wantMax ? h.worldMax : h.worldMin;
      return make_float3(v.x, v.y, v.z);
    }
  for (const MeshPrim& m : s.meshes)
    if (m.name == name) {
      const f3 v = wantMax ? m.worldMax : m.worldMin;
      return make_float3(v.x, v.y, v.z);
    }
  return make_float3(0.f, 0.f, 0.f);
}
float3 getGeometryMaxBounds(char* name) { return boundsByName(name, true); }
float3 getGeometryMinBounds(char* name) { return boundsByName(name, false); }

int crGetLastError(char* buf, size_t len) {
  const int n = static_cast<int>(g_lastError.size());
  if (buf && len) {
    const size_t k = std::min(len - 1, g_lastError.size());
    std::memcpy(buf, g_lastError.data(), k);
    buf[k] = '\0';
  }
  g_lastError.clear();
  return n;
}

int getOmmatidialColoursF32(float* out) {
  return guarded(
      "getOmmatidialColoursF32",
      [&]() -> int {
        Renderer& r = R();
        if (!r.compoundActive()) throw std::runtime_error("current camera is not a compound eye");
        EyeDev& e = r.eyes[r.current];
        if (!e.haveSums) throw std::runtime_error("the current eye has not been rendered yet");
        if (!out) throw std::runtime_error("null output");
        if (e.N) {
          check(cudaMemcpyAsync(out, e.sums.ptr, sizeof(float) * 3 * e.N, cudaMemcpyDeviceToHost, r.stream()), "cudaMemcpy");
          check(cudaStreamSynchronize(r.stream()), "colour download");
        }
        return 0;
      },
      -1);
}

int crRenderPoses(const float* poses, size_t count, float* out) {
  return guarded(
      "crRenderPoses",
      [&]() -> int {
        Renderer& r = R();
        if (!r.compoundActive()) throw std::runtime_error("current camera is not a compound eye");
        if (count == 0) return 0;
        if (!poses || !out) throw std::runtime_error("null pose or output array");
        EyeDev& e = r.syncEye(r.current);
        std::vector<float> p16(16 * count);
        for (size_t i = 0; i < count; ++i)
          for (int k = 0; k < 4; ++k) {
            p16[16 * i + 4 * k + 0] = poses[12 * i + 3 * k + 0];
            p16[16 * i + 4 * k + 1] = poses[12 * i + 3 * k + 1];
            p16[16 * i + 4 * k + 2] = poses[12 * i + 3 * k + 2];
            p16[16 * i + 4 * k + 3] = 0.f;
          }
        r.poses.ensure(4 * count);
        const size_t outFloats = 3 * count * e.N;
        r.batchOut.ensure(std::max<size_t>(1, outFloats));
        check(cudaMemcpyAsync(r.poses.ptr, p16.data(), p16.size() * sizeof(float), cudaMemcpyHostToDevice, r.stream()),
              "cudaMemcpy");
        r.renderDevicePoses(e, r.poses.ptr, count, r.batchOut.ptr, nullptr);
        if (outFloats)
          check(cudaMemcpyAsync(out, r.batchOut.ptr, outFloats * sizeof(float), cudaMemcpyDeviceToHost, r.stream()),
                "cudaMemcpy");
        // The last pose's colours become the eye's current frame.
        if (e.N)
          check(cudaMemcpyAsync(e.sums.ptr, r.batchOut.ptr + 3 * (count - 1) * e.N, 3 * e.N * sizeof(float),
                                cudaMemcpyDeviceToDevice, r.stream()),
                "cudaMemcpy");
        e.haveSums = true;
        r.checkErrWord();
        return 0;
      },
      -1);
}

int crRenderPosesDevice(const float* d_poses, size_t count, float* d_out) {
  return guarded(
      "crRenderPosesDevice",
      [&]() -> int {
        Renderer& r = R();
        if (!r.compoundActive()) throw std::runtime_error("current camera is not a compound eye");
        if (count == 0) return 0;
        if (!d_poses || !d_out) throw std::runtime_error("null pose or output pointer");
        EyeDev& e = r.syncEye(r.current);
        r.renderDevicePoses(e, reinterpret_cast<const float4*>(d_poses), count, d_out, nullptr);
        return 0;
      },
      -1);
}

int crMeasureTraversal(const float* d_poses, size_t count, double* nodesPerRay, double* trisPerRay) {
  return guarded(
      "crMeasureTraversal",
      [&]() -> int {
        Renderer& r = R();
        if (!r.compoundActive()) throw std::runtime_error("current camera is not a compound eye");
        if (count == 0 || !d_poses) throw std::runtime_error("no poses");
        EyeDev& e = r.syncEye(r.current);
        DevBuf<unsigned long long> st;
        st.ensure(2);
        DevBuf<float> out;
        out.ensure(std::max<size_t>(1, 3 * count * e.N));
        check(cudaMemsetAsync(st.ptr, 0, 2 * sizeof(unsigned long long), r.stream()), "cudaMemset");
        r.renderDevicePoses(e, reinterpret_cast<const float4*>(d_poses), count, out.ptr, nullptr, st.ptr);
        unsigned long long h[2] = {0, 0};
        check(cudaMemcpyAsync(h, st.ptr, sizeof(h), cudaMemcpyDeviceToHost, r.stream()), "cudaMemcpy");
        r.checkErrWord();
        const double rays = static_cast<double>(count) * e.N * e.spp;
        if (nodesPerRay) *nodesPerRay = rays > 0 ? static_cast<double>(h[0]) / rays : 0.0;
        if (trisPerRay) *trisPerRay = rays > 0 ? static_cast<double>(h[1]) / rays : 0.0;
        st.release();
        out.release();
        return 0;
      },
      -1);
}

// Batched rendering of many eyes (the compound cameras of the scene) in one
// persistent launch, recorded once into a CUDA graph and replayed.
int crBatchCreate(const int* cams, size_t nCams, size_t posesPerCam, const float* d_poses, float* d_out) {
  return guarded(
      "crBatchCreate",
      [&]() -> int {
        R().requireUnlit("crBatchCreate");
        Renderer& r = R();
        if (!r.loaded) throw std::runtime_error("no scene loaded");
        if (!cams || nCams == 0 || posesPerCam == 0 || !d_poses || !d_out)
          throw std::runtime_error("empty batch or null pointer");
        Batch b;
        b.cams.assign(cams, cams + nCams);
        b.P = posesPerCam;
        std::vector<BatchEye> table(nCams);
        std::vector<unsigned long long> tb(nCams), cb(nCams);
        size_t outOff = 0, scratchFloats = 0;
        // The near-field cut radius in force now is recorded into the graph.
        r.ensureUploaded();
        const bool useCuts = r.cutFactor > 0.f && r.dev.extent > 0.f && r.dev.width == 2 &&
                             r.bvhStats.maxDepth + kCutEntries + 2 <= 64;
        if (useCuts) {
          b.cuts.ensure(nCams * posesPerCam * kCutStride);
          b.cutPoses = static_cast<uint32_t>(posesPerCam);
        }
        for (size_t i = 0; i < nCams; ++i) {
          const int ci = cams[i];
          if (ci < 0 || static_cast<size_t>(ci) >= r.scene.cameras.size() ||
              r.scene.cameras[static_cast<size_t>(ci)].kind != CameraKind::Compound)
            throw std::runtime_error("camera " + std::to_string(ci) + " is not a compound eye");
          for (size_t j = 0; j < i; ++j)
            if (cams[j] == ci) throw std::runtime_error("camera " + std::to_string(ci) + " appears twice");
          EyeDev& e = r.syncEye(static_cast<size_t>(ci));
          r.ensureRng(e);
          BatchEye& be = table[i];
          be.eye = r.devEye(e);
          be.poses = reinterpret_cast<const float4*>(d_poses) + 4 * posesPerCam * i;
          be.out = d_out + outOff;
          be.plan = planBatch(e.N, e.spp);
          be.P = static_cast<uint32_t>(posesPerCam);
          be.scratch = nullptr;
          if (useCuts) {
            be.eye.cuts = b.cuts.ptr + i * posesPerCam * kCutStride;
            be.eye.cutRadius = r.cutFactor * r.dev.extent;
            be.eye.maxRel = e.maxRel;
          }
          tb[i] = b.totalTasks;
          cb[i] = b.totalCells;
          b.outOffset.push_back(outOff);
          outOff += 3 * posesPerCam * e.N;
          b.totalTasks += e.N ? be.plan.tasks * 1ull : 0ull;
          if (be.plan.chunks > 1 && e.N) {
            scratchFloats += posesPerCam * e.N * be.plan.chunks * 3;
            b.totalCells += static_cast<unsigned long long>(posesPerCam) * e.N;
          }
        }
        if (scratchFloats) b.scratch.ensure(scratchFloats);
        size_t so = 0;
        for (size_t i = 0; i < nCams; ++i)
          if (table[i].plan.chunks > 1 && table[i].eye.N) {
            table[i].scratch = b.scratch.ptr + so;
            so += posesPerCam * table[i].eye.N * table[i].plan.chunks * 3;
          }
        b.table.ensure(nCams);
        b.taskBase.ensure(nCams);
        b.cellBase.ensure(nCams);
        b.ctrl.ensure(2 + nCams);
        cudaStream_t st = r.stream();
        check(cudaMemcpyAsync(b.table.ptr, table.data(), nCams * sizeof(BatchEye), cudaMemcpyHostToDevice, st), "cudaMemcpy");
        check(cudaMemcpyAsync(b.taskBase.ptr, tb.data(), nCams * sizeof(unsigned long long), cudaMemcpyHostToDevice, st),
              "cudaMemcpy");
        check(cudaMemcpyAsync(b.cellBase.ptr, cb.data(), nCams * sizeof(unsigned long long), cudaMemcpyHostToDevice, st),
              "cudaMemcpy");
        uint32_t* err = r.errWord();
        check(cudaStreamSynchronize(st), "batch set-up");
        int dev = 0, sms = 0;
        check(cudaGetDevice(&dev), "cudaGetDevice");
        check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
        b.variant = renderVariant();
        b.grid = sms * std::max(1, batchBlocksPerSM(b.variant));
        // Record: reset the counters, the persistent launch, the chunk sums.
        check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        cudaError_t ce = cudaMemsetAsync(b.ctrl.ptr, 0, (2 + nCams) * sizeof(unsigned long long), st);
        if (ce == cudaSuccess) ce = cudaMemsetAsync(b.ctrl.ptr + 1, 0xff, sizeof(unsigned long long), st);
        if (ce == cudaSuccess)
          ce = launchBatch(r.dev, b.table.ptr, b.taskBase.ptr, b.cellBase.ptr, static_cast<uint32_t>(nCams),
                           b.totalTasks, b.totalCells, b.ctrl.ptr, err, b.variant, b.grid, b.cutPoses, st);
        cudaGraph_t g = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(st, &g);
        check(ce, "batch capture");
        check(ee, "cudaStreamEndCapture");
        b.graph = g;
        check(cudaGraphInstantiate(&b.exec, b.graph, 0), "cudaGraphInstantiate");
        b.generation = r.generation;
        int id = 1;
        while (batches().count(id)) ++id;
        batches()[id] = std::move(b);
        return id;
      },
      -1);
}

int crBatchLaunch(int handle) {
  return guarded(
      "crBatchLaunch",
      [&]() -> int {
        R().requireUnlit("crBatchLaunch");
        auto it = batches().find(handle);
        if (it == batches().end()) throw std::runtime_error("unknown batch handle");
        if (it->second.generation != R().generation)
          throw std::runtime_error("batch invalidated by a change of scene or eye configuration; recreate it");
        check(cudaGraphLaunch(it->second.exec, R().stream()), "cudaGraphLaunch");
        return 0;
      },
      -1);
}

int crBatchLatencies(int handle, float* msPerCam, float* totalMs) {
  return guarded(
      "crBatchLatencies",
      [&]() -> int {
        auto it = batches().find(handle);
        if (it == batches().end()) throw std::runtime_error("unknown batch handle");
        Batch& b = it->second;
        Renderer& r = R();
        std::vector<unsigned long long> h(2 + b.cams.size());
        check(cudaMemcpyAsync(h.data(), b.ctrl.ptr, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                              r.stream()),
              "cudaMemcpy");
        r.checkErrWord();
        unsigned long long last = 0;
        for (size_t i = 0; i < b.cams.size(); ++i) {
          const unsigned long long done = h[2 + i];
          last = std::max(last, done);
          if (msPerCam) msPerCam[i] = done > h[1] ? static_cast<float>((done - h[1]) * 1e-6) : 0.f;
        }
        if (totalMs) *totalMs = last > h[1] ? static_cast<float>((last - h[1]) * 1e-6) : 0.f;
        return 0;
      },
      -1);
}

size_t crBatchOutputOffset(int handle, size_t camIndex) {
  auto it = batches().find(handle);
  if (it == batches().end() || camIndex >= it->second.outOffset.size()) return 0;
  return it->second.outOffset[camIndex];
}

int crBatchDestroy(int handle) {
  auto it = batches().find(handle);
  if (it == batches().end()) return -1;
  cudaStreamSynchronize(R().stream());
  it->second.release();
  batches().erase(it);
  return 0;
}

int renderBatch(const int* cams, size_t nCams, size_t posesPerCam, const float* d_poses, float* d_out) {
  const int h = crBatchCreate(cams, nCams, posesPerCam, d_poses, d_out);
  if (h < 0) return -1;
  int rc = crBatchLaunch(h);
  if (rc == 0) {
    rc = guarded(
        "renderBatch",
        [&]() -> int {
          check(cudaStreamSynchronize(R().stream()), "renderBatch");
          return 0;
        },
        -1);
  }
  crBatchDestroy(h);
  return rc;
}

// Same work as crRenderPosesDevice for callers that cannot allocate device
// memory when they render: the chunk partials go to the library's fixed
// device array instead of a library-allocated buffer, and the call makes no
// cudaMalloc/cudaFree.  The eye's device state (scene, ommatidia, random
// streams, error word) must already exist, i.e. the current eye must have been
// rendered once through an allocating entry point with its present ommatidium
// and sample counts; otherwise the call fails without doing anything.
int crRenderPosesDeviceNoAlloc(const float* d_poses, size_t count, float* d_out) {
  return guarded(
      "crRenderPosesDeviceNoAlloc",
      [&]() -> int {
        Renderer& r = R();
        if (!r.compoundActive()) throw std::runtime_error("current camera is not a compound eye");
        if (count == 0) return 0;
        if (!d_poses || !d_out) throw std::runtime_error("null pose or output pointer");
        const Camera& c = r.scene.cameras[r.current];
        const uint32_t N = static_cast<uint32_t>(c.omm.size());
        const uint32_t spp = static_cast<uint32_t>(std::max(1, c.spp));
        const size_t perPose = renderScratchFloats(r.dev, N, spp, 1, false, false, true);  // chunk partials in scratch
        const size_t cap = noAllocScratchFloats();
        if (perPose > cap)
          throw std::runtime_error("an eye of " + std::to_string(N) + " ommatidia x " + std::to_string(spp) +
                                   " samples needs " + std::to_string(perPose) +
                                   " floats of scratch per pose; the allocation-free path holds at most " +
                                   std::to_string(cap) + " floats (16 MiB)");
        EyeDev& e = r.eyes[r.current];
        if (r.pendingBvh || r.pendingGpuBuild || !e.omm.ptr || !e.rng.ptr || e.N != N || e.spp != spp || !r.err.ptr)
          throw std::runtime_error(
              "the eye's device state is not set up: render it once with renderFrame, crRenderPoses or "
              "crRenderPosesDevice before using the allocation-free entry point");
        float* scratch = nullptr;
        check(noAllocScratch(&scratch), "cudaGetSymbolAddress");
        r.ensureRng(e);
        const size_t batch = perPose ? std::min<size_t>(kMaxPosesPerLaunch, cap / perPose) : kMaxPosesPerLaunch;
        const float4* poses = reinterpret_cast<const float4*>(d_poses);
        for (size_t first = 0; first < count; first += batch) {
          const uint32_t P = static_cast<uint32_t>(std::min(batch, count - first));
          check(launchRender(r.dev, r.devEye(e), poses + 4 * first, P, d_out + 3 * first * N, perPose ? scratch : nullptr,
                             r.err.ptr, nullptr, r.stream(), nullptr, true),
                "render launch");
        }
        return 0;
      },
      -1);
}

int crAutotune(const float* d_poses, size_t count, int* bestVariant, float* msPerVariant) {
  return guarded(
      "crAutotune",
      [&]() -> int {
        Renderer& r = R();
        if (!r.compoundActive()) throw std::runtime_error("current camera is not a compound eye");
        if (count == 0 || !d_poses) throw std::runtime_error("no poses");
        EyeDev& e = r.syncEye(r.current);
        r.ensureRng(e);
        // Trial renders must not advance the eye's random streams: keep a
        // copy of the states and put it back after every trial.
        const size_t words = static_cast<size_t>(kRngPlanes) * e.N * e.spp;
        DevBuf<uint32_t> saved;
        saved.ensure(std::max<size_t>(1, words));
        DevBuf<float> out;
        out.ensure(std::max<size_t>(1, 3 * count * e.N));
        cudaStream_t st = r.stream();
        check(cudaMemcpyAsync(saved.ptr, e.rng.ptr, words * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st), "cudaMemcpy");
        cudaEvent_t a, b;
        check(cudaEventCreate(&a), "cudaEventCreate");
        check(cudaEventCreate(&b), "cudaEventCreate");
        const int prev = renderVariant();
        int best = 0;
        float bestMs = INFINITY;
        float variantMs[3] = {0.f, 0.f, 0.f};
        setRenderLayout(0, 0);  // variants timed with the automatic layout
        for (int v = 0; v < renderVariantCount(); ++v) {
          setRenderVariant(v);
          float ms = INFINITY;
          for (int rep = 0; rep < 2; ++rep) {  // first pass warms caches and code
            check(cudaEventRecord(a, st), "cudaEventRecord");
            r.renderDevicePoses(e, reinterpret_cast<const float4*>(d_poses), count, out.ptr, nullptr);
            check(cudaEventRecord(b, st), "cudaEventRecord");
            check(cudaEventSynchronize(b), "cudaEventSynchronize");
            check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
            check(cudaMemcpyAsync(e.rng.ptr, saved.ptr, words * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st),
                  "cudaMemcpy");
          }
          if (msPerVariant) msPerVariant[v] = ms;
          if (v < 3) variantMs[v] = ms;
          if (ms < bestMs) {
            bestMs = ms;
            best = v;
          }
        }
        auto trial = [&]() {
          float ms = INFINITY;
          for (int rep = 0; rep < 2; ++rep) {  // first pass warms caches and code
            check(cudaEventRecord(a, st), "cudaEventRecord");
            r.renderDevicePoses(e, reinterpret_cast<const float4*>(d_poses), count, out.ptr, nullptr);
            check(cudaEventRecord(b, st), "cudaEventRecord");
            check(cudaEventSynchronize(b), "cudaEventSynchronize");
            check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
            check(cudaMemcpyAsync(e.rng.ptr, saved.ptr, words * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st),
                  "cudaMemcpy");
          }
          return ms;
        };
        setRenderVariant(best);
        r.tuneTimes.assign(kTuneSlots, 0.f);
        for (int v = 0; v < 3; ++v) r.tuneTimes[v] = variantMs[v];
        // Block size (results identical), then samples per warp segment.
        const uint32_t blocks[] = {128, 256, 512};
        uint32_t bestBlock = 128, bestSeg = 0;
        float bestLayoutMs = INFINITY;
        for (int k = 0; k < 3; ++k) {
          setRenderLayout(blocks[k], 0);
          const float ms = trial();
          r.tuneTimes[3 + k] = ms;
          if (ms < bestLayoutMs) {
            bestLayoutMs = ms;
            bestBlock = blocks[k];
          }
        }
        const uint32_t segs[] = {8, 16};  // 32 (the default) was timed above
        r.tuneTimes[8] = bestLayoutMs;
        for (int k = 0; k < 2; ++k) {
          setRenderLayout(bestBlock, segs[k]);
          const float ms = trial();
          r.tuneTimes[6 + k] = ms;
          if (ms < bestLayoutMs) {
            bestLayoutMs = ms;
            bestSeg = segs[k];
          }
        }
        setRenderLayout(bestBlock, bestSeg);
        // Near-field cut radius (fraction of the scene extent), with the best variant and layout.
        const float factors[] = {0.f, 1.f / 256, 1.f / 128, 1.f / 64, 1.f / 32, 1.f / 16};
        float bestCut = 0.f, bestCutMs = INFINITY;
        for (int k = 0; k < 6; ++k) {
          r.cutFactor = factors[k];
          const float ms = trial();
          r.tuneTimes[9 + k] = ms;
          if (ms < bestCutMs) {
            bestCutMs = ms;
            bestCut = factors[k];
          }
        }
        r.cutFactor = bestCut;
        // Refinement: the geometric midpoints on either side of the best
        // non-zero radius (a factor of sqrt 2 each way).
        if (bestCut > 0.f) {
          const float around[] = {bestCut * 0.70710678f, bestCut * 1.41421356f};
          float refined = bestCut;
          for (int k = 0; k < 2; ++k) {
            if (!(around[k] <= 1.f)) continue;
            r.cutFactor = around[k];
            const float ms = trial();
            r.tuneTimes[18 + k] = ms;
            if (ms < bestCutMs) {
              bestCutMs = ms;
              refined = around[k];
            }
          }
          bestCut = refined;
          r.cutFactor = bestCut;
        }
        // BVH width: the two-wide BVH with its best cut against the wide ones.
        const int prevWidth = r.bvhWidth;
        int bestWidth = 2;
        float bestWidthMs = INFINITY;
        for (int k = 0; k < 3; ++k) {
          const int W = k == 0 ? 2 : (k == 1 ? 4 : 8);
          r.bvhWidth = W;
          r.ensureUploaded();
          const float ms = trial();
          r.tuneTimes[15 + k] = ms;
          if (ms < bestWidthMs) {
            bestWidthMs = ms;
            bestWidth = W;
          }
        }
        r.bvhWidth = bestWidth;
        r.ensureUploaded();
        if (bestWidth != prevWidth) ++r.generation;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        r.checkErrWord();
        (void)prev;
        if (bestVariant) *bestVariant = best;
        saved.release();
        out.release();
        return 0;
      },
      -1);
}

int crGetAutotuneTimes(float* ms, size_t n) {
  return guarded(
      "crGetAutotuneTimes",
      [&]() -> int {
        if (!ms) throw std::runtime_error("null pointer");
        const std::vector<float>& t = R().tuneTimes;
        if (t.empty()) throw std::runtime_error("crAutotune has not run");
        for (size_t k = 0; k < n; ++k) ms[k] = k < t.size() ? t[k] : 0.f;
        return 0;
      },
      -1);
}

int crSetRenderLayout(int blockThreads, int samplesPerWarp) {
  return guarded(
      "crSetRenderLayout",
      [&]() -> int {
        if (blockThreads != 0 && blockThreads != 128 && blockThreads != 256 && blockThreads != 512)
          throw std::runtime_error("blockThreads must be 0 (automatic), 128, 256 or 512");
        if (samplesPerWarp != 0 && samplesPerWarp != 8 && samplesPerWarp != 16 && samplesPerWarp != 32)
          throw std::runtime_error("samplesPerWarp must be 0 (32), 8, 16 or 32");
        setRenderLayout(static_cast<uint32_t>(blockThreads), samplesPerWarp == 32 ? 0u : static_cast<uint32_t>(samplesPerWarp));
        ++R().generation;  // recorded batches follow the layout they were made with
        return 0;
      },
      -1);
}

int crGetRenderLayout(int* blockThreads, int* samplesPerWarp) {
  return guarded(
      "crGetRenderLayout",
      [&]() -> int {
        if (!blockThreads || !samplesPerWarp) throw std::runtime_error("null pointer");
        uint32_t bt = 0, sw = 0;
        renderLayout(&bt, &sw);
        *blockThreads = static_cast<int>(bt);
        *samplesPerWarp = sw ? static_cast<int>(sw) : 32;
        return 0;
      },
      -1);
}

int crSetLighting(int on) {
  return guarded(
      "crSetLighting",
      [&]() -> int {
        Renderer& r = R();
        r.lighting = on != 0;
        if (r.loaded && !r.pendingBvh && !r.pendingGpuBuild) r.applyLighting();
        return 0;
      },
      -1);
}

int crGetLighting(void) { return R().lighting ? 1 : 0; }

int crGetSceneLighting(float* light, float* lightPos, float* lightCol) {
  Renderer& r = R();
  if (!r.loaded) {
    setError("crGetSceneLighting: no scene loaded");
    return -1;
  }
  if (light) std::memcpy(light, r.scene.triLight.data(), r.scene.triLight.size() * sizeof(float));
  float4 pos[4], col[4];
  Renderer::lightSetup(r.scene, pos, col);
  for (int i = 0; i < 4; ++i) {
    if (lightPos) {
      lightPos[4 * i] = pos[i].x;
      lightPos[4 * i + 1] = pos[i].y;
      lightPos[4 * i + 2] = pos[i].z;
      lightPos[4 * i + 3] = pos[i].w;
    }
    if (lightCol) {
      lightCol[3 * i] = col[i].x;
      lightCol[3 * i + 1] = col[i].y;
      lightCol[3 * i + 2] = col[i].z;
    }
  }
  return 0;
}

int crSetCutRadius(float fractionOfExtent) {
  if (!(fractionOfExtent >= 0.f) || fractionOfExtent > 1.f) {
    setError("crSetCutRadius: the fraction must lie in [0, 1]");
    return -1;
  }
  R().cutFactor = fractionOfExtent;
  return 0;
}

float crGetCutRadius(void) { return R().cutFactor; }

int crSetRenderVariant(int variant) {
  if (variant < 0 || variant >= renderVariantCount()) {
    setError("crSetRenderVariant: variant out of range");
    return -1;
  }
  setRenderVariant(variant);
  return 0;
}

int crGetRenderVariant(void) { return renderVariant(); }

int crGetRenderVariantCount(void) { return renderVariantCount(); }

int crSetDeviceMemoryCap(size_t bytes) {
  devCap() = bytes;
  return 0;
}

size_t crGetDeviceMemoryHeld(void) { return devHeld(); }

int crSelfTestBoundedWait(unsigned int polls) {
  return guarded(
      "crSelfTestBoundedWait",
      [&]() -> int {
        Renderer& r = R();
        uint32_t* err = r.errWord();
        cudaStream_t st = r.stream();
        check(cudaMemsetAsync(err, 0, sizeof(uint32_t), st), "cudaMemset");
        check(launchWaitProbe(polls, err, st), "wait probe");
        uint32_t word = 0;
        check(cudaMemcpyAsync(&word, err, sizeof(word), cudaMemcpyDeviceToHost, st), "cudaMemcpy");
        check(cudaStreamSynchronize(st), "wait probe");
        check(cudaMemsetAsync(err, 0, sizeof(uint32_t), st), "cudaMemset");
        check(cudaStreamSynchronize(st), "wait probe");
        return (word & kErrMmaTimeout) ? 1 : 0;
      },
      -1);
}

int crSetProjectionSearch(int mode) {
  if (mode != 0 && mode != 1) {
    setError("crSetProjectionSearch: mode must be 0 (grid) or 1 (every candidate)");
    return -1;
  }
  R().projectionGrid = mode == 0;
  return 0;
}

int crGetProjectionSearch(void) { return R().projectionGrid ? 0 : 1; }

// ---------------------------------------------------------------------------
// Learned denoiser (denoiser.hpp): the network is process-wide; its feature
// render uses its own random streams (spp of the feature render) so that the
// camera's own streams are untouched.
// ---------------------------------------------------------------------------
}  // extern "C"

namespace cr {
namespace {

struct DenoiseState {
  Denoiser net;
  int inferKernel = 1;  // 0: mma.sync fused kernel, 1: tcgen05 fused kernel (default)
  size_t cam = static_cast<size_t>(-1);
  uint64_t generation = ~0ull;
  DevBuf<int> nb;
  DevBuf<uint32_t> targetRng;  // XORWOW streams of the 1024-sample training targets
  uint32_t targetSpp = 0;
  bool targetReady = false;
  DevBuf<float> stats, base, out, scratch;
  DevBuf<float4> derived, axes;  // inputs of the tcgen05 inference (deriveFeatureStats)
  DevBuf<uint16_t> X;
  DevBuf<float4> poses;
  // Sample-count allocator: a second network of the same shape, trained on
  // minimum-sample labels; and the adaptive render's buffers.
  Denoiser alloc;
  uint64_t adaptiveFrame = 0;  // frames rendered adaptively since the eye was bound (draw seed offset)
  DevBuf<float> pred, learned, sums, partials, labelOuts;
  DevBuf<uint32_t> entries;
  DevBuf<uint8_t> level;
  DevBuf<uint16_t> labels;
  DevBuf<unsigned long long> counts, tileScratch;
  std::vector<uint16_t> lastLabels;
  double lastRays = 0;  // rays traced by the last adaptive render (feature + adaptive)
  uint64_t featFrame = 0;  // feature-render frames of the current eye so far (keys its draws)
  uint64_t lastPassRows = 0;  // rows of the last adaptive pass (its pred, stats and level stay in place)
  float allocHalvings = 0.f;  // predicted counts are divided by 2^allocHalvings (crSetAllocatorHalvings)
  float allocExponent = 1.f;  // counts follow the predicted count to this power (crSetAllocatorExponent)
  float allocCostExponent = 0.f;  // counts scale as traversal cost^-this (crSetAllocatorCostExponent)
};

DenoiseState& DS() {
  static DenoiseState d;
  return d;
}

// Ties the denoiser's per-eye state (neighbour table, streams) to the
// current eye, rebuilding it when the eye or its buffers changed.
EyeDev& denoiseEye(Renderer& r, DenoiseState& d) {
  if (!r.compoundActive()) throw std::runtime_error("current camera is not a compound eye");
  EyeDev& e = r.syncEye(r.current);
  if (d.cam != r.current || d.generation != r.generation) {
    d.cam = r.current;
    d.generation = r.generation;
    d.nb.release();
    d.nb.ensure(std::max<size_t>(1, static_cast<size_t>(kNeighbours) * e.N));
    check(nearestOmmatidia(e.omm.ptr, e.N, d.nb.ptr, r.stream()), "neighbour search");
    d.targetReady = false;
    d.targetSpp = 0;
    d.adaptiveFrame = 0;
    d.featFrame = 0;
  }
  return e;
}

DevEye streamsFor(Renderer& r, EyeDev& e, DevBuf<uint32_t>& rng, uint32_t& haveSpp, bool& ready, uint32_t spp) {
  DevEye d;
  d.omm = e.omm.ptr;
  d.order = e.order.ptr;
  d.N = e.N;
  d.spp = spp;
  if (haveSpp != spp || !ready) {
    rng.release();
    rng.ensure(std::max<size_t>(1, static_cast<size_t>(kRngPlanes) * e.N * spp));
    d.rng = rng.ptr;
    check(launchRngInit(d, r.errWord(), r.stream()), "rng init launch");
    haveSpp = spp;
    ready = true;
  }
  d.rng = rng.ptr;
  return d;
}

// Feature rows (and 8-sample means) of `count` device poses of the current eye.
// Feature render of `count` poses into d.stats; with `rows`, also the
// feature rows and residual bases (d.X, d.base) the training set and the
// layer-by-layer path use.
constexpr unsigned long long kFeatureSeed = 0xfea70000ull;  // draw seed of the feature renders

void denoiseFeatures(Renderer& r, DenoiseState& d, EyeDev& e, const float4* dposes, size_t count, uint32_t featSpp,
                     bool rows = true) {
  if (featSpp < 1 || featSpp > 32) throw std::runtime_error("feature renders use 1 to 32 samples per ommatidium");
  if (count > 0xffffffffull) throw std::runtime_error("too many poses in one feature render");
  // Stratified draws keyed by frame (featFrame + p) of the eye and the
  // ommatidium, so all poses render in one launch spread over any number of
  // warps; reloading the scene or switching eyes restarts the frame count.
  DevEye fe;
  fe.omm = e.omm.ptr;
  fe.order = e.order.ptr;
  fe.N = e.N;
  fe.spp = featSpp;
  fe.netDraws = true;
  fe.drawSeed = kFeatureSeed;
  fe.frame0 = d.featFrame;
  d.featFrame += count;
  d.lastPassRows = 0;  // the statistics of the last adaptive pass are overwritten
  d.stats.ensure(std::max<size_t>(1, count * e.N * kFeatureStats));
  r.withCuts(fe, static_cast<uint32_t>(count), e.maxRel);
  check(launchFeatures(r.dev, fe, dposes, static_cast<uint32_t>(count), d.stats.ptr, r.errWord(), r.stream(), false),
        "feature render");
  if (!rows) return;
  d.X.ensure(std::max<size_t>(1, count * e.N * kFeatureWidth));
  d.base.ensure(std::max<size_t>(1, count * e.N * 3));
  check(assembleFeatures(d.stats.ptr, e.omm.ptr, d.nb.ptr, e.N, static_cast<uint32_t>(count), d.X.ptr, d.base.ptr,
                         r.stream()),
        "feature rows");
}

void uploadPoses12(DevBuf<float4>& dst, const float* poses12, size_t count, cudaStream_t s) {
  std::vector<float> p16(16 * count, 0.f);
  for (size_t i = 0; i < count; ++i)
    for (int k = 0; k < 4; ++k)
      for (int c = 0; c < 3; ++c) p16[16 * i + 4 * k + c] = poses12[12 * i + 3 * k + c];
  dst.ensure(std::max<size_t>(1, 4 * count));
  check(cudaMemcpyAsync(dst.ptr, p16.data(), p16.size() * 4, cudaMemcpyHostToDevice, s), "cudaMemcpy");
}

}  // namespace
}  // namespace cr

extern "C" {

int crDenoiserInit(int seed) {
  return guarded(
      "crDenoiserInit",
      [&]() -> int {
        DS().net.init(static_cast<uint32_t>(seed), R().stream());
        return 0;
      },
      -1);
}

size_t crDenoiserParamCount(void) { return Denoiser::kParams; }

void crDenoiserRelease(void) { DS().net.release(); }

int crSetDenoiserKernel(int kind) {
  if (kind != 0 && kind != 1) {
    setError("crSetDenoiserKernel: kind must be 0 (mma.sync) or 1 (tcgen05)");
    return -1;
  }
  DS().inferKernel = kind;
  return 0;
}

int crGetDenoiserKernel(void) { return DS().inferKernel; }

int crDenoiserAddTrainingPoses(const float* poses12, size_t count, int featureSpp, int targetSpp) {
  return guarded(
      "crDenoiserAddTrainingPoses",
      [&]() -> int {
        R().requireUnlit("crDenoiserAddTrainingPoses");
        Renderer& r = R();
        DenoiseState& d = DS();
        if (!d.net.ready()) throw std::runtime_error("call crDenoiserInit first");
        if (!poses12 || count == 0) throw std::runtime_error("no poses");
        if (targetSpp < 1) throw std::runtime_error("target sample count must be positive");
        EyeDev& e = denoiseEye(r, d);
        uploadPoses12(d.poses, poses12, count, r.stream());
        denoiseFeatures(r, d, e, d.poses.ptr, count, static_cast<uint32_t>(featureSpp));
        const DevEye te = streamsFor(r, e, d.targetRng, d.targetSpp, d.targetReady, static_cast<uint32_t>(targetSpp));
        d.out.ensure(std::max<size_t>(1, count * e.N * 3));
        for (size_t first = 0; first < count; first += kMaxPosesPerLaunch) {
          const uint32_t P = static_cast<uint32_t>(std::min<size_t>(kMaxPosesPerLaunch, count - first));
          const size_t need = renderScratchFloats(r.dev, e.N, te.spp, P);
          if (need) d.scratch.ensure(need);
          check(launchRender(r.dev, te, d.poses.ptr + 4 * first, P, d.out.ptr + 3 * first * e.N,
                             need ? d.scratch.ptr : nullptr, r.errWord(), nullptr, r.stream()),
                "target render");
        }
        d.net.addRows(d.X.ptr, d.base.ptr, d.out.ptr, count * e.N, r.stream());
        r.checkErrWord();
        return 0;
      },
      -1);
}

int crDenoiserTrain(int steps, int batch, float lr, int seed, float* lossHistory) {
  return guarded(
      "crDenoiserTrain",
      [&]() -> int {
        DS().net.train(steps, batch, lr, static_cast<uint32_t>(seed), lossHistory, R().stream(),
                       DS().inferKernel == 1);
        return 0;
      },
      -1);
}

size_t crDenoiserTrainingRows(void) { return DS().net.rows(); }

int crDenoiserRenderPosesDevice(const float* d_poses, size_t count, int featureSpp, float* d_out) {
  return guarded(
      "crDenoiserRenderPosesDevice",
      [&]() -> int {
        R().requireUnlit("crDenoiserRenderPosesDevice");
        Renderer& r = R();
        DenoiseState& d = DS();
        if (!d.net.ready()) throw std::runtime_error("call crDenoiserInit or crDenoiserLoad first");
        if (count == 0) return 0;
        if (!d_poses || !d_out) throw std::runtime_error("null pointer");
        EyeDev& e = denoiseEye(r, d);
        denoiseFeatures(r, d, e, reinterpret_cast<const float4*>(d_poses), count, static_cast<uint32_t>(featureSpp),
                        false);
        for (size_t first = 0; first < count; first += kMaxPosesPerLaunch) {
          const uint32_t P = static_cast<uint32_t>(std::min<size_t>(kMaxPosesPerLaunch, count - first));
          const float* st = d.stats.ptr + first * e.N * kFeatureStats;
          if (d.inferKernel == 1) {
            d.derived.ensure(static_cast<size_t>(3) * P * e.N);
            d.axes.ensure(std::max<size_t>(1, e.N));
            check(deriveFeatureStats(st, e.omm.ptr, e.N, P, d.derived.ptr, d.axes.ptr, r.stream()), "feature statistics");
          }
          check(d.inferKernel == 1
                    ? inferDenoiserTc(d.derived.ptr, d.axes.ptr, d.nb.ptr, e.N, P, d.net.weights(),
                                      d_out + 3 * first * e.N, r.errWord(), r.stream(), true, e.order.ptr)
                    : inferDenoiser(st, e.omm.ptr, d.nb.ptr, e.N, P, d.net.weights(), d_out + 3 * first * e.N,
                                    r.stream()),
                "denoiser inference");
        }
        return 0;
      },
      -1);
}

int crDenoiserRenderPoses(const float* poses12, size_t count, int featureSpp, float* out) {
  return guarded(
      "crDenoiserRenderPoses",
      [&]() -> int {
        Renderer& r = R();
        DenoiseState& d = DS();
        if (!poses12 || !out) throw std::runtime_error("null pointer");
        if (count == 0) return 0;
        EyeDev& e = denoiseEye(r, d);
        uploadPoses12(d.poses, poses12, count, r.stream());
        DevBuf<float> o;
        o.ensure(std::max<size_t>(1, count * e.N * 3));
        if (crDenoiserRenderPosesDevice(reinterpret_cast<const float*>(d.poses.ptr), count, featureSpp, o.ptr) != 0)
          throw std::runtime_error(g_lastError);
        check(cudaMemcpyAsync(out, o.ptr, count * e.N * 12, cudaMemcpyDeviceToHost, r.stream()), "cudaMemcpy");
        r.checkErrWord();
        o.release();
        return 0;
      },
      -1);
}

int crDenoiserFeatureRows(const float* poses12, size_t count, int featureSpp, uint16_t* xBf16, float* base) {
  return guarded(
      "crDenoiserFeatureRows",
      [&]() -> int {
        Renderer& r = R();
        DenoiseState& d = DS();
        if (!poses12 || !xBf16 || !base) throw std::runtime_error("null pointer");
        if (count == 0) return 0;
        EyeDev& e = denoiseEye(r, d);
        uploadPoses12(d.poses, poses12, count, r.stream());
        denoiseFeatures(r, d, e, d.poses.ptr, count, static_cast<uint32_t>(featureSpp));
        const size_t rows = count * e.N;
        check(cudaMemcpyAsync(xBf16, d.X.ptr, rows * kFeatureWidth * 2, cudaMemcpyDeviceToHost, r.stream()),
              "cudaMemcpy");
        check(cudaMemcpyAsync(base, d.base.ptr, rows * 12, cudaMemcpyDeviceToHost, r.stream()), "cudaMemcpy");
        r.checkErrWord();
        return 0;
      },
      -1);
}

int crDenoiserPredictRows(const uint16_t* xBf16, const float* base, size_t rows, float* out) {
  return guarded(
      "crDenoiserPredictRows",
      [&]() -> int {
        Renderer& r = R();
        DenoiseState& d = DS();
        if (!d.net.ready()) throw std::runtime_error("call crDenoiserInit or crDenoiserLoad first");
        if (rows == 0) return 0;
        if (!xBf16 || !base || !out) throw std::runtime_error("null pointer");
        DevBuf<uint16_t> x;
        DevBuf<float> b, o;
        x.ensure(rows * kFeatureWidth);
        b.ensure(rows * 3);
        o.ensure(rows * 3);
        check(cudaMemcpyAsync(x.ptr, xBf16, rows * kFeatureWidth * 2, cudaMemcpyHostToDevice, r.stream()), "cudaMemcpy");
        check(cudaMemcpyAsync(b.ptr, base, rows * 12, cudaMemcpyHostToDevice, r.stream()), "cudaMemcpy");
        d.net.infer(x.ptr, b.ptr, rows, o.ptr, r.stream());
        check(cudaMemcpyAsync(out, o.ptr, rows * 12, cudaMemcpyDeviceToHost, r.stream()), "cudaMemcpy");
        check(cudaStreamSynchronize(r.stream()), "prediction");
        return 0;
      },
      -1);
}

float crDenoiserGradient(const uint16_t* xBf16, const float* base, const float* target, int rows, float* grads,
                         float* params) {
  return guarded(
      "crDenoiserGradient",
      [&]() -> float {
        Renderer& r = R();
        DenoiseState& d = DS();
        if (!d.net.ready()) throw std::runtime_error("call crDenoiserInit first");
        if (rows <= 0 || !xBf16 || !base || !target) throw std::runtime_error("empty input");
        DevBuf<uint16_t> X;
        DevBuf<float> b, t;
        X.ensure(static_cast<size_t>(rows) * kFeatureWidth);
        b.ensure(static_cast<size_t>(rows) * 3);
        t.ensure(static_cast<size_t>(rows) * 3);
        cudaStream_t s = r.stream();
        check(cudaMemcpyAsync(X.ptr, xBf16, static_cast<size_t>(rows) * kFeatureWidth * 2, cudaMemcpyHostToDevice, s),
              "cudaMemcpy");
        check(cudaMemcpyAsync(b.ptr, base, static_cast<size_t>(rows) * 12, cudaMemcpyHostToDevice, s), "cudaMemcpy");
        check(cudaMemcpyAsync(t.ptr, target, static_cast<size_t>(rows) * 12, cudaMemcpyHostToDevice, s), "cudaMemcpy");
        const float l = d.net.gradient(X.ptr, b.ptr, t.ptr, rows, grads, params, s, d.inferKernel == 1);
        X.release();
        b.release();
        t.release();
        return l;
      },
      -1.0f);
}

int crDenoiserAdamStep(float* w, const float* g, float* m, float* v, size_t n, float lr, float c1, float c2,
                       uint16_t* wbBits) {
  return guarded(
      "crDenoiserAdamStep",
      [&]() -> int {
        if (n == 0) return 0;
        if (!w || !g || !m || !v || !wbBits) throw std::runtime_error("null pointer");
        if (n > 0x7fffffffu) throw std::runtime_error("too many parameters");
        cudaStream_t s = R().stream();
        DevBuf<float> dw, dg, dm, dv, sched;
        DevBuf<uint16_t> wb;
        DevBuf<int> idx;
        dw.ensure(n);
        dg.ensure(n);
        dm.ensure(n);
        dv.ensure(n);
        wb.ensure(n);
        sched.ensure(3);
        idx.ensure(1);
        const float e[3] = {lr, c1, c2};
        check(cudaMemcpyAsync(dw.ptr, w, n * 4, cudaMemcpyHostToDevice, s), "cudaMemcpy");
        check(cudaMemcpyAsync(dg.ptr, g, n * 4, cudaMemcpyHostToDevice, s), "cudaMemcpy");
        check(cudaMemcpyAsync(dm.ptr, m, n * 4, cudaMemcpyHostToDevice, s), "cudaMemcpy");
        check(cudaMemcpyAsync(dv.ptr, v, n * 4, cudaMemcpyHostToDevice, s), "cudaMemcpy");
        check(cudaMemcpyAsync(sched.ptr, e, sizeof(e), cudaMemcpyHostToDevice, s), "cudaMemcpy");
        check(cudaMemsetAsync(idx.ptr, 0, sizeof(int), s), "cudaMemset");
        // The training loop's call: step size and bias corrections read from
        // the device schedule at the device step index.
        check(adamStep(dw.ptr, dg.ptr, dm.ptr, dv.ptr, static_cast<int>(n), 0.f, 0.9f, 0.999f, 1e-8f, 1, wb.ptr, s,
                       nullptr, nullptr, sched.ptr, idx.ptr),
              "adam");
        check(cudaMemcpyAsync(w, dw.ptr, n * 4, cudaMemcpyDeviceToHost, s), "cudaMemcpy");
        check(cudaMemcpyAsync(m, dm.ptr, n * 4, cudaMemcpyDeviceToHost, s), "cudaMemcpy");
        check(cudaMemcpyAsync(v, dv.ptr, n * 4, cudaMemcpyDeviceToHost, s), "cudaMemcpy");
        check(cudaMemcpyAsync(wbBits, wb.ptr, n * 2, cudaMemcpyDeviceToHost, s), "cudaMemcpy");
        check(cudaStreamSynchronize(s), "adam");
        return 0;
      },
      -1);
}

int crDenoiserScaleOutput(float alpha) {
  return guarded(
      "crDenoiserScaleOutput",
      [&]() -> int {
        if (!(alpha >= 0.f && alpha <= 1.f)) throw std::runtime_error("alpha must be in [0, 1]");
        DenoiseState& d = DS();
        if (!d.net.ready()) throw std::runtime_error("call crDenoiserInit first");
        d.net.scaleOutput(alpha, R().stream());
        return 0;
      },
      -1);
}

int crDenoiserSave(const char* path) {
  return guarded(
      "crDenoiserSave",
      [&]() -> int {
        if (!path) throw std::runtime_error("null path");
        DS().net.save(path, R().stream());
        return 0;
      },
      -1);
}

int crDenoiserLoad(const char* path) {
  return guarded(
      "crDenoiserLoad",
      [&]() -> int {
        if (!path) throw std::runtime_error("null path");
        DS().net.load(path, R().stream());
        return 0;
      },
      -1);
}

// ---- Learned sample allocator and adaptive rendering ----------------------

int crAllocatorInit(int seed) {
  return guarded(
      "crAllocatorInit",
      [&]() -> int {
        DS().alloc.init(static_cast<uint32_t>(seed), R().stream());
        return 0;
      },
      -1);
}

int crAllocatorAddTrainingPoses(const float* poses12, size_t count, int featureSpp, float threshold, int seeds,
                                uint16_t* labelsOut) {
  return guarded(
      "crAllocatorAddTrainingPoses",
      [&]() -> int {
        R().requireUnlit("crAllocatorAddTrainingPoses");
        Renderer& r = R();
        DenoiseState& d = DS();
        if (!d.alloc.ready()) throw std::runtime_error("call crAllocatorInit first");
        if (!poses12 || count == 0) throw std::runtime_error("no poses");
        if (seeds < 2 || seeds > 64) throw std::runtime_error("the label search needs 2 to 64 seeds");
        if (!(threshold > 0.f)) throw std::runtime_error("threshold must be positive");
        if (count > kMaxPosesPerLaunch) throw std::runtime_error("at most 256 poses per call");
        EyeDev& e = denoiseEye(r, d);
        cudaStream_t st = r.stream();
        uploadPoses12(d.poses, poses12, count, st);
        denoiseFeatures(r, d, e, d.poses.ptr, count, static_cast<uint32_t>(featureSpp));
        const uint64_t rows = static_cast<uint64_t>(count) * e.N;
        // Minimum-sample search: every entry rendered `seeds` times (independent
        // streams) at 4, 8, ..., 1024 samples; the label is the first count at
        // which the colour's standard deviation across the renders falls below
        // the threshold in every channel (0 = none up to 1024).  Entries are
        // listed pose by pose in the eye's direction order, for coherent warps.
        const std::vector<uint32_t> ord = directionOrder(r.scene.cameras[r.current].omm);
        std::vector<uint32_t> iota(rows);
        for (uint64_t i = 0; i < rows; ++i)
          iota[i] = static_cast<uint32_t>((i / e.N) * e.N + ord[static_cast<size_t>(i % e.N)]);
        d.entries.ensure(rows);
        check(cudaMemcpyAsync(d.entries.ptr, iota.data(), rows * 4, cudaMemcpyHostToDevice, st), "cudaMemcpy");
        d.labels.ensure(rows);
        check(cudaMemsetAsync(d.labels.ptr, 0, rows * 2, st), "cudaMemset");
        d.labelOuts.ensure(static_cast<size_t>(seeds) * rows * 3);
        d.partials.ensure(std::max<size_t>(1, adaptivePartialFloats(rows, 1024)));
        for (uint32_t c = 4; c <= 1024; c *= 2) {
          const uint32_t* ent = d.entries.ptr;
          float* part = d.partials.ptr;
          const AdaptiveLaunch L = planAdaptive(&ent, &rows, &c, &part, 1);
          DevEye ce;
          r.withCuts(ce, static_cast<uint32_t>(count), e.maxRel);
          if (ce.cuts)
            check(launchCuts(r.dev, d.poses.ptr, static_cast<uint32_t>(count), ce.cutRadius, ce.maxRel, ce.cuts, st),
                  "cuts");
          for (int k = 0; k < seeds; ++k)
            check(launchAdaptive(r.dev, e.omm.ptr, e.N, d.poses.ptr, L, 0x5eed0000ull + static_cast<uint64_t>(k),
                                 d.labelOuts.ptr + static_cast<size_t>(k) * rows * 3, r.errWord(), nullptr, st,
                                 ce.cuts),
                  "label render");
          check(launchLabels(d.labelOuts.ptr, seeds, rows, c, threshold, d.labels.ptr, st), "labels");
        }
        d.lastLabels.assign(rows, 0);
        check(cudaMemcpyAsync(d.lastLabels.data(), d.labels.ptr, rows * 2, cudaMemcpyDeviceToHost, st), "cudaMemcpy");
        r.checkErrWord();
        // Targets: log2(label) / 10 in all three outputs (label 0 -> 2048).
        std::vector<float> target(rows * 3);
        for (uint64_t i = 0; i < rows; ++i) {
          const uint32_t lab = d.lastLabels[i] ? d.lastLabels[i] : 2048u;
          const float l = std::log2(static_cast<float>(lab)) / 10.0f;
          target[3 * i] = target[3 * i + 1] = target[3 * i + 2] = l;
        }
        DevBuf<float> t, zero;
        t.ensure(rows * 3);
        zero.ensure(rows * 3);
        check(cudaMemcpyAsync(t.ptr, target.data(), rows * 12, cudaMemcpyHostToDevice, st), "cudaMemcpy");
        check(cudaMemsetAsync(zero.ptr, 0, rows * 12, st), "cudaMemset");
        d.alloc.addRows(d.X.ptr, zero.ptr, t.ptr, rows, st);
        check(cudaStreamSynchronize(st), "allocator rows");
        if (labelsOut) std::memcpy(labelsOut, d.lastLabels.data(), rows * 2);
        return 0;
      },
      -1);
}

int crAllocatorTrain(int steps, int batch, float lr, int seed, float* lossHistory) {
  return guarded(
      "crAllocatorTrain",
      [&]() -> int {
        DS().alloc.train(steps, batch, lr, static_cast<uint32_t>(seed), lossHistory, R().stream(),
                         DS().inferKernel == 1);
        return 0;
      },
      -1);
}

size_t crAllocatorTrainingRows(void) { return DS().alloc.rows(); }

int crAllocatorSave(const char* path) {
  return guarded(
      "crAllocatorSave",
      [&]() -> int {
        if (!path) throw std::runtime_error("null path");
        DS().alloc.save(path, R().stream());
        return 0;
      },
      -1);
}

int crSetAllocatorHalvings(float halvings) {
  if (!(halvings >= -4.f) || halvings > 6.f) {
    setError("crSetAllocatorHalvings: the value must lie in [-4, 6]");
    return -1;
  }
  DS().allocHalvings = halvings;
  return 0;
}

float crGetAllocatorHalvings(void) { return DS().allocHalvings; }

int crSetAllocatorExponent(float exponent) {
  if (!(exponent >= 0.25f) || exponent > 1.f) {
    setError("crSetAllocatorExponent: the value must lie in [0.25, 1]");
    return -1;
  }
  DS().allocExponent = exponent;
  return 0;
}

float crGetAllocatorExponent(void) { return DS().allocExponent; }

int crSetAllocatorCostExponent(float costExponent) {
  if (!(costExponent >= 0.f) || costExponent > 1.f) {
    setError("crSetAllocatorCostExponent: the value must lie in [0, 1]");
    return -1;
  }
  DS().allocCostExponent = costExponent;
  return 0;
}

float crGetAllocatorCostExponent(void) { return DS().allocCostExponent; }

int crAllocatorLoad(const char* path) {
  return guarded(
      "crAllocatorLoad",
      [&]() -> int {
        if (!path) throw std::runtime_error("null path");
        DS().alloc.load(path, R().stream());
        return 0;
      },
      -1);
}

int crAdaptiveRenderPosesDevice(const float* d_poses, size_t count, int featureSpp, float* d_out, uint8_t* d_level,
                                double* raysTraced) {
  return guarded(
      "crAdaptiveRenderPosesDevice",
      [&]() -> int {
        R().requireUnlit("crAdaptiveRenderPosesDevice");
        Renderer& r = R();
        DenoiseState& d = DS();
        if (!d.alloc.ready()) throw std::runtime_error("call crAllocatorInit (and train) or crAllocatorLoad first");
        if (count == 0) return 0;
        if (!d_poses || !d_out) throw std::runtime_error("null pointer");
        EyeDev& e = denoiseEye(r, d);
        cudaStream_t st = r.stream();
        const float4* poses = reinterpret_cast<const float4*>(d_poses);
        const uint32_t fs = static_cast<uint32_t>(featureSpp);
        double rays = 0;
        // Poses per pass: at least 256, and up to 2^21 entries, so that a small
        // eye's trajectory allocates once (one host wait for the bucket sizes)
        // while the adaptive launch stays below 2^26 warp tasks.
        const size_t perPass = std::max<size_t>(kMaxPosesPerLaunch, (size_t(1) << 21) / std::max<uint32_t>(1u, e.N));
        for (size_t first = 0; first < count; first += perPass) {
          const uint32_t P = static_cast<uint32_t>(std::min<size_t>(perPass, count - first));
          const uint64_t rows = static_cast<uint64_t>(P) * e.N;
          denoiseFeatures(r, d, e, poses + 4 * first, P, fs, false);
          rays += static_cast<double>(rows) * fs;
          d.pred.ensure(rows * 3);
          if (d.inferKernel == 1) {
            d.derived.ensure(3 * rows);
            d.axes.ensure(std::max<size_t>(1, e.N));
            check(deriveFeatureStats(d.stats.ptr, e.omm.ptr, e.N, P, d.derived.ptr, d.axes.ptr, st),
                  "feature statistics");
          }
          auto infer = [&](const MlpWeights& w, float* o, bool residual) {
            return d.inferKernel == 1
                       ? inferDenoiserTc(d.derived.ptr, d.axes.ptr, d.nb.ptr, e.N, P, w, o, r.errWord(), st, residual,
                                         e.order.ptr)
                       : inferDenoiser(d.stats.ptr, e.omm.ptr, d.nb.ptr, e.N, P, w, o, st, residual);
          };
          check(infer(d.alloc.weights(), d.pred.ptr, false), "allocator inference");
          const float* learned = nullptr;
          if (d.net.ready()) {
            d.learned.ensure(rows * 3);
            check(infer(d.net.weights(), d.learned.ptr, true), "denoiser inference");
            learned = d.learned.ptr;
          }
          d.level.ensure(rows);
          d.counts.ensure(kAdaptiveBuckets);
          check(cudaMemsetAsync(d.counts.ptr, 0, kAdaptiveBuckets * 8, st), "cudaMemset");
          check(launchAllocate(d.pred.ptr, rows, fs, d.level.ptr, d.counts.ptr, st, d.allocHalvings, d.allocExponent,
                               d.stats.ptr, d.allocCostExponent),
                "allocation");
          unsigned long long cnt[kAdaptiveBuckets];
          check(cudaMemcpyAsync(cnt, d.counts.ptr, sizeof(cnt), cudaMemcpyDeviceToHost, st), "cudaMemcpy");
          check(cudaStreamSynchronize(st), "allocation");
          unsigned long long off[kAdaptiveBuckets];
          uint64_t total = 0, partialFloats = 0;
          for (uint32_t k = 0; k < kAdaptiveBuckets; ++k) {
            off[k] = total;
            total += cnt[k];
            partialFloats += adaptivePartialFloats(cnt[k], 4u << k);
            rays += static_cast<double>(cnt[k]) * static_cast<double>(4u << k);
          }
          d.sums.ensure(rows * 3);
          if (total) {
            d.entries.ensure(total);
            d.partials.ensure(std::max<uint64_t>(1, partialFloats));
            check(cudaMemcpyAsync(d.counts.ptr, off, sizeof(off), cudaMemcpyHostToDevice, st), "cudaMemcpy");
            d.tileScratch.ensure(scatterScratchWords(rows));
            check(launchScatterBuckets(d.level.ptr, rows, e.N, e.order.ptr, d.counts.ptr, d.tileScratch.ptr,
                                       d.entries.ptr, st),
                  "bucket lists");
            const uint32_t* ent[kAdaptiveBuckets];
            uint64_t n[kAdaptiveBuckets];
            uint32_t spp[kAdaptiveBuckets];
            float* part[kAdaptiveBuckets];
            uint64_t pf = 0;
            for (uint32_t k = 0; k < kAdaptiveBuckets; ++k) {
              ent[k] = d.entries.ptr + off[k];
              n[k] = cnt[k];
              spp[k] = 4u << k;
              part[k] = d.partials.ptr + pf;
              pf += adaptivePartialFloats(cnt[k], spp[k]);
            }
            const AdaptiveLaunch L = planAdaptive(ent, n, spp, part, kAdaptiveBuckets);
            DevEye ce;
            r.withCuts(ce, P, e.maxRel);
            if (ce.cuts) check(launchCuts(r.dev, poses + 4 * first, P, ce.cutRadius, ce.maxRel, ce.cuts, st), "cuts");
            check(launchAdaptive(r.dev, e.omm.ptr, e.N, poses + 4 * first, L, 0xada90000ull + d.adaptiveFrame,
                                 d.sums.ptr, r.errWord(), nullptr, st, ce.cuts),
                  "adaptive render");
          }
          check(launchAdaptiveFinish(d.level.ptr, rows, fs, d.stats.ptr, learned, d.sums.ptr, d_out + 3 * first * e.N,
                                     st),
                "adaptive finish");
          if (d_level)
            check(cudaMemcpyAsync(d_level + first * e.N, d.level.ptr, rows, cudaMemcpyDeviceToDevice, st),
                  "cudaMemcpy");
          d.adaptiveFrame += P;
          d.lastPassRows = rows;
        }
        d.lastRays = rays;
        if (raysTraced) *raysTraced = rays;
        return 0;
      },
      -1);
}

int crAdaptiveLastPass(float* prediction, float* cost, uint8_t* level, size_t rows) {
  return guarded(
      "crAdaptiveLastPass",
      [&]() -> int {
        DenoiseState& d = DS();
        if (d.lastPassRows == 0)
          throw std::runtime_error("no adaptive pass to read (none yet, or a later feature render replaced it)");
        if (rows != d.lastPassRows)
          throw std::runtime_error("rows must equal the last pass's rows (" + std::to_string(d.lastPassRows) + ")");
        cudaStream_t st = R().stream();
        if (prediction)
          check(cudaMemcpyAsync(prediction, d.pred.ptr, rows * 3 * sizeof(float), cudaMemcpyDeviceToHost, st),
                "cudaMemcpy");
        if (cost)
          check(cudaMemcpy2DAsync(cost, sizeof(float), d.stats.ptr + kCostStat, kFeatureStats * sizeof(float),
                                  sizeof(float), rows, cudaMemcpyDeviceToHost, st),
                "cudaMemcpy2D");
        if (level) check(cudaMemcpyAsync(level, d.level.ptr, rows, cudaMemcpyDeviceToHost, st), "cudaMemcpy");
        check(cudaStreamSynchronize(st), "adaptive pass copy");
        return 0;
      },
      -1);
}

int crSetAdaptiveSchedule(int refillIdle, int steps) {
  return guarded(
      "crSetAdaptiveSchedule",
      [&]() -> int {
        if (refillIdle < 1 || refillIdle > 32) throw std::runtime_error("refillIdle must be in [1, 32]");
        if (steps < 1 || steps > 4096) throw std::runtime_error("steps must be in [1, 4096]");
        setAdaptiveSchedule(static_cast<uint32_t>(refillIdle), steps);
        return 0;
      },
      -1);
}

int crGetAdaptiveSchedule(int* refillIdle, int* steps) {
  return guarded(
      "crGetAdaptiveSchedule",
      [&]() -> int {
        if (!refillIdle || !steps) throw std::runtime_error("null pointer");
        uint32_t r = 0;
        adaptiveSchedule(&r, steps);
        *refillIdle = static_cast<int>(r);
        return 0;
      },
      -1);
}

int crSetAdaptiveOccupancy(int blocksPerSM) {
  return guarded(
      "crSetAdaptiveOccupancy",
      [&]() -> int {
        if (blocksPerSM != 5 && blocksPerSM != 6 && blocksPerSM != 8)
          throw std::runtime_error("blocksPerSM must be 5, 6 or 8");
        setAdaptiveBlocksPerSM(blocksPerSM);
        return 0;
      },
      -1);
}

int crGetAdaptiveOccupancy(void) { return adaptiveBlocksPerSM(); }

int crAdaptiveRecord(const float* poses12, size_t count, int spp, unsigned long long seed, void* records,
                     float* sums) {
  return guarded(
      "crAdaptiveRecord",
      [&]() -> int {
        R().requireUnlit("crAdaptiveRecord");
        Renderer& r = R();
        DenoiseState& d = DS();
        if (!poses12 || !records || !sums) throw std::runtime_error("null pointer");
        if (count == 0) return 0;
        if (spp < 1 || spp > 1024 || (spp & (spp - 1))) throw std::runtime_error("spp must be a power of two <= 1024");
        if (count > kMaxPosesPerLaunch) throw std::runtime_error("at most 256 poses per call");
        EyeDev& e = denoiseEye(r, d);
        cudaStream_t st = r.stream();
        uploadPoses12(d.poses, poses12, count, st);
        const uint64_t rows = static_cast<uint64_t>(count) * e.N;
        std::vector<uint32_t> iota(rows);
        for (uint64_t i = 0; i < rows; ++i) iota[i] = static_cast<uint32_t>(i);
        DevBuf<uint32_t> ent;
        DevBuf<float> part, s;
        DevBuf<RayRecord> rec;
        ent.ensure(rows);
        s.ensure(rows * 3);
        part.ensure(std::max<size_t>(1, adaptivePartialFloats(rows, static_cast<uint32_t>(spp))));
        rec.ensure(rows * static_cast<uint64_t>(spp));
        check(cudaMemcpyAsync(ent.ptr, iota.data(), rows * 4, cudaMemcpyHostToDevice, st), "cudaMemcpy");
        const uint32_t* ep = ent.ptr;
        float* pp = part.ptr;
        const uint32_t c = static_cast<uint32_t>(spp);
        const AdaptiveLaunch L = planAdaptive(&ep, &rows, &c, &pp, 1);
        DevEye ce;
        r.withCuts(ce, static_cast<uint32_t>(count), e.maxRel);
        if (ce.cuts)
          check(launchCuts(r.dev, d.poses.ptr, static_cast<uint32_t>(count), ce.cutRadius, ce.maxRel, ce.cuts, st),
                "cuts");
        check(launchAdaptive(r.dev, e.omm.ptr, e.N, d.poses.ptr, L, seed, s.ptr, r.errWord(), rec.ptr, st, ce.cuts),
              "adaptive render");
        check(cudaMemcpyAsync(records, rec.ptr, rows * spp * sizeof(RayRecord), cudaMemcpyDeviceToHost, st),
              "cudaMemcpy");
        check(cudaMemcpyAsync(sums, s.ptr, rows * 12, cudaMemcpyDeviceToHost, st), "cudaMemcpy");
        r.checkErrWord();
        return 0;
      },
      -1);
}

int crSetBvhBuilder(int kind) {
  if (kind != 0 && kind != 1) {
    setError("crSetBvhBuilder: builder must be 0 (host SAH) or 1 (GPU linear BVH)");
    return -1;
  }
  R().builder = kind;
  return 0;
}

int crGetBvhBuilder(void) { return R().builder; }

int crSetBvhWidth(int width) {
  return guarded(
      "crSetBvhWidth",
      [&]() -> int {
        if (width != 2 && width != 4 && width != 8) throw std::runtime_error("BVH width must be 2, 4 or 8");
        Renderer& r = R();
        if (r.bvhWidth != width) ++r.generation;  // recorded batches search the tree they were made with
        r.bvhWidth = width;
        return 0;
      },
      -1);
}

int crGetBvhWidth(void) { return R().bvhWidth; }

int crGetWideBvhHost(int width, float* nodesOut, size_t capFloats, uint32_t* nodeCount, float* trisOut) {
  return guarded(
      "crGetWideBvhHost",
      [&]() -> int {
        Renderer& r = R();
        if (!r.loaded || !r.pendingBvh) throw std::runtime_error("needs a scene loaded with the host builder, not yet uploaded");
        const HostBvh& b = *r.pendingBvh;
        std::vector<float> w;
        WideBvhStats st;
        collapseWideBvh(b.nodes.data(), static_cast<uint32_t>(b.nodes.size() / 16), b.tris.data(),
                        static_cast<uint32_t>(b.tris.size() / 12), width, w, st);
        if (nodeCount) *nodeCount = st.nodes;
        if (nodesOut) {
          if (capFloats < w.size()) throw std::runtime_error("output too small");
          std::memcpy(nodesOut, w.data(), w.size() * 4);
        }
        if (trisOut)
          for (size_t t = 0; t < b.tris.size() / 12; ++t)
            for (int v = 0; v < 3; ++v)
              for (int a = 0; a < 3; ++a) trisOut[9 * t + 3 * v + a] = b.tris[12 * t + 4 * v + a];
        return 0;
      },
      -1);
}

int crGetWideBvhStats(uint32_t* nodes, uint32_t* depth, double* meanChildren) {
  return guarded(
      "crGetWideBvhStats",
      [&]() -> int {
        Renderer& r = R();
        if (!r.loaded) throw std::runtime_error("no scene loaded");
        r.ensureUploaded();
        if (nodes) *nodes = r.dev.width == 2 ? 0u : r.wideStats.nodes;
        if (depth) *depth = r.dev.width == 2 ? 0u : r.wideStats.maxDepth;
        if (meanChildren) *meanChildren = r.dev.width == 2 ? 0.0 : r.wideStats.meanChildren;
        return 0;
      },
      -1);
}

int crSetStream(void* stream) {
  R().userStream = static_cast<cudaStream_t>(stream);
  return 0;
}

int crSynchronize(void) {
  return guarded(
      "crSynchronize",
      [&]() -> int {
        Renderer& r = R();
        check(cudaStreamSynchronize(r.stream()), "synchronize");
        r.checkErrWord();
        return 0;
      },
      -1);
}

int crRenderFrameRecorded(void* records) {
  return guarded(
      "crRenderFrameRecorded",
      [&]() -> int {
        Renderer& r = R();
        if (!r.compoundActive()) throw std::runtime_error("current camera is not a compound eye");
        if (!records) throw std::runtime_error("null record buffer");
        Camera& c = r.cam();
        EyeDev& e = r.syncEye(r.current);
        const size_t n = static_cast<size_t>(e.N) * e.spp;
        DevBuf<RayRecord> rec;
        rec.ensure(std::max<size_t>(1, n));
        float p16[16];
        Renderer::packPose(c, p16);
        r.poses.ensure(4);
        check(cudaMemcpyAsync(r.poses.ptr, p16, sizeof(p16), cudaMemcpyHostToDevice, r.stream()), "cudaMemcpy");
        r.renderDevicePoses(e, r.poses.ptr, 1, e.sums.ptr, rec.ptr);
        e.haveSums = true;
        if (n) check(cudaMemcpyAsync(records, rec.ptr, n * sizeof(RayRecord), cudaMemcpyDeviceToHost, r.stream()), "cudaMemcpy");
        r.checkErrWord();
        rec.release();
        return 0;
      },
      -1);
}

size_t crGetTriangleCount(void) { return R().loaded ? R().scene.triangleCount() : 0; }

int crGetSceneTriangles(float* verts, float* colours, unsigned char* shading) {
  Renderer& r = R();
  if (!r.loaded) {
    setError("crGetSceneTriangles: no scene loaded");
    return -1;
  }
  const SceneData& s = r.scene;
  if (verts) std::memcpy(verts, s.triVerts.data(), s.triVerts.size() * sizeof(float));
  if (colours) std::memcpy(colours, s.triColours.data(), s.triColours.size() * sizeof(float));
  if (shading) std::memcpy(shading, s.triShading.data(), s.triShading.size());
  return 0;
}

size_t crGetTextureCount(void) { return R().loaded ? R().scene.textures.size() : 0; }
size_t crGetTexelCount(void) { return R().loaded ? R().scene.texels.size() : 0; }

int crGetSceneTextures(int* table, unsigned int* texels) {
  Renderer& r = R();
  if (!r.loaded) {
    setError("crGetSceneTextures: no scene loaded");
    return -1;
  }
  const SceneData& s = r.scene;
  if (table)
    for (size_t i = 0; i < s.textures.size(); ++i) {
      table[3 * i] = static_cast<int>(s.textures[i].offset);
      table[3 * i + 1] = s.textures[i].width;
      table[3 * i + 2] = s.textures[i].height;
    }
  if (texels && !s.texels.empty()) std::memcpy(texels, s.texels.data(), s.texels.size() * sizeof(uint32_t));
  return 0;
}

int crCompareTextureSampling(const unsigned int* texels, int width, int height, const float* uv, int n,
                             float* rgbaRenderer, float* rgbaHardware) {
  return guarded(
      "crCompareTextureSampling",
      [&]() -> int {
        check(sampleTextureBoth(texels, width, height, uv, n, rgbaRenderer, rgbaHardware), "texture sampling");
        return 0;
      },
      -1);
}

int crGetOmmatidia(float* out) {
  return guarded(
      "crGetOmmatidia",
      [&]() -> int {
        Renderer& r = R();
        if (!r.compoundActive()) throw std::runtime_error("current camera is not a compound eye");
        if (!out) throw std::runtime_error("null output");
        const std::vector<Ommatidium>& o = r.scene.cameras[r.current].omm;
        if (!o.empty()) std::memcpy(out, o.data(), o.size() * sizeof(Ommatidium));
        return 0;
      },
      -1);
}

int crGetCameraLocalSpace(float* a) {
  return guarded(
      "crGetCameraLocalSpace",
      [&]() -> int {
        const LocalSpace& ls = R().cam().ls;
        const f3 v[3] = {ls.x, ls.y, ls.z};
        for (int k = 0; k < 3; ++k) {
          a[3 * k] = v[k].x;
          a[3 * k + 1] = v[k].y;
          a[3 * k + 2] = v[k].z;
        }
        return 0;
      },
      -1);
}

int crGetRandomStates(uint32_t* out) {
  return guarded(
      "crGetRandomStates",
      [&]() -> int {
        Renderer& r = R();
        if (!r.compoundActive()) throw std::runtime_error("current camera is not a compound eye");
        EyeDev& e = r.eyes[r.current];
        if (!e.configured || !e.rng.ptr) return -1;
        const size_t n = static_cast<size_t>(kRngPlanes) * e.N * e.spp;
        check(cudaMemcpyAsync(out, e.rng.ptr, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, r.stream()), "cudaMemcpy");
        check(cudaStreamSynchronize(r.stream()), "state download");
        return 0;
      },
      -1);
}

int crGetBvhStats(uint32_t* innerNodes, uint32_t* leaves, uint32_t* maxDepth) {
  Renderer& r = R();
  if (!r.loaded) return -1;
  if (innerNodes) *innerNodes = r.bvhStats.innerNodes;
  if (leaves) *leaves = r.bvhStats.leaves;
  if (maxDepth) *maxDepth = r.bvhStats.maxDepth;
  return 0;
}

}  // extern "C"

void* getWindowPointer() { return nullptr; }
