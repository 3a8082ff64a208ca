// Host binned-SAH BVH2 builder; see bvh.hpp for the device layout.
#include "bvh.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

namespace cr {
namespace {

struct Box {
  float lo[3] = {INFINITY, INFINITY, INFINITY};
  float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void grow(const float* p) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], p[k]);
      hi[k] = std::max(hi[k], p[k]);
    }
  }
  void grow(const Box& b) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], b.lo[k]);
      hi[k] = std::max(hi[k], b.hi[k]);
    }
  }
  bool empty() const { return lo[0] > hi[0]; }
  double area() const {
    if (empty()) return 0.0;
    const double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return 2.0 * (dx * dy + dy * dz + dz * dx);
  }
};

struct Ref {
  Box box;
  float c[3];
  uint32_t id;
};

constexpr int kBins = 32;
constexpr double kCostTraverse = 1.2;
constexpr double kCostTriangle = 1.0;

struct Builder {
  std::vector<Ref>& refs;
  std::vector<Box> nodeBox;  // per node: own bounds (for SAH stats)
  std::vector<int32_t> child;  // 2 per node
  std::vector<Box> childBox;   // 2 per node
  std::vector<uint32_t> triOrder;
  BvhBuildStats stats;

  int32_t leafCode(uint32_t first, uint32_t count) {
    if (count < 1 || count > static_cast<uint32_t>(kMaxLeafSize)) throw std::logic_error("bad leaf size");
    if (first >= (1u << 28)) throw std::runtime_error("scene too large for the leaf encoding (2^28 triangles)");
    return ~static_cast<int32_t>((first << 3) | (count - 1));
  }

  uint32_t newNode() {
    child.push_back(0);
    child.push_back(0);
    childBox.emplace_back();
    childBox.emplace_back();
    return static_cast<uint32_t>(child.size() / 2 - 1);
  }

  int32_t makeLeaf(size_t begin, size_t end) {
    const uint32_t first = static_cast<uint32_t>(triOrder.size());
    for (size_t i = begin; i < end; ++i) triOrder.push_back(refs[i].id);
    ++stats.leaves;
    return leafCode(first, static_cast<uint32_t>(end - begin));
  }

  // Returns the child code for refs[begin, end).
  int32_t build(size_t begin, size_t end, uint32_t depth, Box& outBox) {
    Box bounds, cb;
    for (size_t i = begin; i < end; ++i) {
      bounds.grow(refs[i].box);
      cb.grow(refs[i].c);
    }
    outBox = bounds;
    stats.maxDepth = std::max(stats.maxDepth, depth);
    const size_t n = end - begin;
    if (n == 1) return makeLeaf(begin, end);

    // Binned SAH over the centroid bounds.
    double bestCost = INFINITY;
    int bestAxis = -1, bestSplit = -1;
    for (int axis = 0; axis < 3; ++axis) {
      const float ext = cb.hi[axis] - cb.lo[axis];
      if (!(ext > 0.0f)) continue;
      Box bb[kBins];
      uint32_t cnt[kBins] = {0};
      const double scale = kBins / static_cast<double>(ext);
      for (size_t i = begin; i < end; ++i) {
        int b = static_cast<int>((refs[i].c[axis] - cb.lo[axis]) * scale);
        b = std::min(std::max(b, 0), kBins - 1);
        ++cnt[b];
        bb[b].grow(refs[i].box);
      }
      double rightArea[kBins];
      uint32_t rightCnt[kBins];
      Box acc;
      uint32_t c = 0;
      for (int b = kBins - 1; b > 0; --b) {
        acc.grow(bb[b]);
        c += cnt[b];
        rightArea[b] = acc.area();
        rightCnt[b] = c;
      }
      Box left;
      uint32_t lc = 0;
      for (int b = 1; b < kBins; ++b) {
        left.grow(bb[b - 1]);
        lc += cnt[b - 1];
        if (lc == 0 || rightCnt[b] == 0) continue;
        const double cost = left.area() * lc + rightArea[b] * rightCnt[b];
        if (cost < bestCost) {
          bestCost = cost;
          bestAxis = axis;
          bestSplit = b;
        }
      }
    }
    const double area = bounds.area();
    const double leafCost = kCostTriangle * static_cast<double>(n);
    const double splitCost = area > 0.0 ? kCostTraverse + kCostTriangle * bestCost / area : INFINITY;
    if (n <= static_cast<size_t>(kMaxLeafSize) && (bestAxis < 0 || leafCost <= splitCost)) return makeLeaf(begin, end);

    size_t mid;
    if (bestAxis < 0) {
      mid = begin + n / 2;  // all centroids coincide: split by position in the list
    } else {
      const double scale = kBins / static_cast<double>(cb.hi[bestAxis] - cb.lo[bestAxis]);
      auto it = std::partition(refs.begin() + static_cast<std::ptrdiff_t>(begin), refs.begin() + static_cast<std::ptrdiff_t>(end),
                               [&](const Ref& r) {
                                 int b = static_cast<int>((r.c[bestAxis] - cb.lo[bestAxis]) * scale);
                                 b = std::min(std::max(b, 0), kBins - 1);
                                 return b < bestSplit;
                               });
      mid = static_cast<size_t>(it - refs.begin());
      if (mid == begin || mid == end) mid = begin + n / 2;
    }
    const uint32_t node = newNode();
    ++stats.innerNodes;
    Box lb, rb;
    const int32_t c0 = build(begin, mid, depth + 1, lb);
    const int32_t c1 = build(mid, end, depth + 1, rb);
    child[2 * node] = c0;
    child[2 * node + 1] = c1;
    childBox[2 * node] = lb;
    childBox[2 * node + 1] = rb;
    return static_cast<int32_t>(node);
  }
};

// Centre and half-extent of a box such that [c - e, c + e] contains [lo, hi]
// exactly: e is computed in double and rounded up.
void centreExtent(const Box& b, float* c, float* e) {
  for (int k = 0; k < 3; ++k) {
    c[k] = 0.5f * b.lo[k] + 0.5f * b.hi[k];
    const double need = std::max(static_cast<double>(b.hi[k]) - c[k], static_cast<double>(c[k]) - b.lo[k]);
    float ef = static_cast<float>(need);
    if (static_cast<double>(ef) < need) ef = std::nextafter(ef, INFINITY);
    e[k] = ef;
  }
}

void packNode(float* dst, const Box& a, const Box& b, int32_t c0, int32_t c1) {
  float ca[3], ea[3], cb[3], eb[3];
  centreExtent(a, ca, ea);
  centreExtent(b, cb, eb);
  dst[0] = ca[0];
  dst[1] = ca[1];
  dst[2] = ca[2];
  dst[3] = ea[0];
  dst[4] = ea[1];
  dst[5] = ea[2];
  dst[6] = cb[0];
  dst[7] = cb[1];
  dst[8] = cb[2];
  dst[9] = eb[0];
  dst[10] = eb[1];
  dst[11] = eb[2];
  std::memcpy(&dst[12], &c0, 4);
  std::memcpy(&dst[13], &c1, 4);
  dst[14] = 0.f;
  dst[15] = 0.f;
}

}  // namespace

void buildBvh(const float* verts, const float* colours, const uint8_t* shading, uint32_t triCount,
              HostBvh& out) {
  out = HostBvh{};
  if (triCount == 0) return;
  std::vector<Ref> refs(triCount);
  for (uint32_t t = 0; t < triCount; ++t) {
    Ref& r = refs[t];
    for (int k = 0; k < 3; ++k) r.box.grow(&verts[9 * t + 3 * k]);
    for (int a = 0; a < 3; ++a) r.c[a] = 0.5f * r.box.lo[a] + 0.5f * r.box.hi[a];
    r.id = t;
  }
  Builder b{refs, {}, {}, {}, {}, {}};
  b.child.reserve(2 * triCount);
  b.childBox.reserve(2 * triCount);
  b.triOrder.reserve(triCount);

  // The root is always an inner node; a scene that fits in one leaf gets a
  // second child whose box lies far outside any reachable ray interval.
  const uint32_t root = b.newNode();
  ++b.stats.innerNodes;
  Box whole;
  for (const Ref& r : refs) whole.grow(r.box);
  if (triCount <= static_cast<uint32_t>(kMaxLeafSize)) {
    b.child[0] = b.makeLeaf(0, triCount);
    b.childBox[0] = whole;
    Box far;
    for (int k = 0; k < 3; ++k) far.lo[k] = far.hi[k] = 1e30f;
    b.child[1] = b.child[0];
    b.childBox[1] = far;
  } else {
    // Split the root exactly as any other node, then move that node's
    // content into slot 0.
    Box rb;
    b.child.pop_back();
    b.child.pop_back();
    b.childBox.pop_back();
    b.childBox.pop_back();
    --b.stats.innerNodes;
    const int32_t code = b.build(0, triCount, 0, rb);
    if (code != 0) throw std::logic_error("root of a multi-leaf scene must be node 0");
  }
  (void)root;

  const size_t nodeCount = b.child.size() / 2;
  out.nodes.resize(nodeCount * 16);
  double sah = 0.0;
  const double rootArea = whole.area() > 0 ? whole.area() : 1.0;
  for (size_t i = 0; i < nodeCount; ++i) {
    packNode(&out.nodes[16 * i], b.childBox[2 * i], b.childBox[2 * i + 1], b.child[2 * i], b.child[2 * i + 1]);
    for (int c = 0; c < 2; ++c) {
      const double a = b.childBox[2 * i + c].area() / rootArea;
      const int32_t code = b.child[2 * i + c];
      if (code < 0) sah += a * kCostTriangle * static_cast<double>((~code & 7) + 1);
      else sah += a * kCostTraverse;
    }
  }
  b.stats.sahCost = sah + kCostTraverse;
  out.order = b.triOrder;
  out.tris.resize(static_cast<size_t>(triCount) * 12);
  out.shade.resize(static_cast<size_t>(triCount) * 12);
  for (uint32_t j = 0; j < triCount; ++j) {
    const uint32_t t = out.order[j];
    float* d = &out.tris[12 * static_cast<size_t>(j)];
    for (int k = 0; k < 3; ++k) {
      d[4 * k + 0] = verts[9 * t + 3 * k + 0];
      d[4 * k + 1] = verts[9 * t + 3 * k + 1];
      d[4 * k + 2] = verts[9 * t + 3 * k + 2];
      d[4 * k + 3] = 0.f;
    }
    std::memcpy(&d[3], &t, 4);
    float* s = &out.shade[12 * static_cast<size_t>(j)];
    std::memcpy(s, &colours[12 * static_cast<size_t>(t)], 12 * sizeof(float));
    s[3] = static_cast<float>(shading[t]);
  }
  out.stats = b.stats;
}

}  // namespace cr
