// Collapse of the two-wide BVH into a 4- or 8-wide BVH with quantised child
// boxes (layout in wbvh.hpp).  Host code, run once per scene and width.
#include "wbvh.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <utility>

namespace cr {
namespace {

struct Box {
  float lo[3], hi[3];
  void grow(const Box& b) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], b.lo[a]);
      hi[a] = std::max(hi[a], b.hi[a]);
    }
  }
  double area() const {
    const double x = double(hi[0]) - lo[0], y = double(hi[1]) - lo[1], z = double(hi[2]) - lo[2];
    return 2.0 * (x * y + y * z + z * x);
  }
};

Box emptyBox() {
  Box b;
  for (int a = 0; a < 3; ++a) {
    b.lo[a] = INFINITY;
    b.hi[a] = -INFINITY;
  }
  return b;
}

// Exact boxes of every two-wide node from its triangles (min / max of float
// vertices, no rounding), children before parents.
std::vector<Box> exactBoxes(const float* nodes, uint32_t inner, const float* tris, uint32_t triCount) {
  std::vector<Box> box(inner, emptyBox());
  auto leafBox = [&](int ref) {
    const uint32_t code = ~static_cast<uint32_t>(ref);
    const uint32_t first = code >> 3, count = (code & 7u) + 1u;
    if (first + count > triCount) throw std::runtime_error("wide BVH: leaf outside the triangle array");
    Box b = emptyBox();
    for (uint32_t t = first; t < first + count; ++t)
      for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) {
          const float x = tris[12 * static_cast<size_t>(t) + 4 * v + a];
          b.lo[a] = std::min(b.lo[a], x);
          b.hi[a] = std::max(b.hi[a], x);
        }
    return b;
  };
  // Post-order over an explicit stack (a linear BVH can be deep).
  std::vector<std::pair<uint32_t, bool>> st;
  st.push_back({0u, false});
  while (!st.empty()) {
    auto [n, expanded] = st.back();
    st.pop_back();
    int c[2];
    std::memcpy(c, nodes + 16 * static_cast<size_t>(n) + 12, sizeof(c));
    if (!expanded) {
      st.push_back({n, true});
      for (int k = 0; k < 2; ++k)
        if (c[k] >= 0) {
          if (static_cast<uint32_t>(c[k]) >= inner) throw std::runtime_error("wide BVH: node outside the array");
          st.push_back({static_cast<uint32_t>(c[k]), false});
        }
      continue;
    }
    Box b = emptyBox();
    for (int k = 0; k < 2; ++k) b.grow(c[k] >= 0 ? box[c[k]] : leafBox(c[k]));
    box[n] = b;
  }
  return box;
}

}  // namespace

void collapseWideBvh(const float* nodes, uint32_t inner, const float* tris, uint32_t triCount, int W,
                     std::vector<float>& out, WideBvhStats& stats) {
  if (W != 4 && W != 8) throw std::runtime_error("wide BVH width must be 4 or 8");
  out.clear();
  stats = WideBvhStats{};
  if (inner == 0) return;
  const std::vector<Box> box = exactBoxes(nodes, inner, tris, triCount);
  auto childRefs = [&](uint32_t n, int* c) { std::memcpy(c, nodes + 16 * static_cast<size_t>(n) + 12, 2 * sizeof(int)); };
  auto leafBox = [&](int ref) {
    const uint32_t code = ~static_cast<uint32_t>(ref);
    const uint32_t first = code >> 3, count = (code & 7u) + 1u;
    Box b = emptyBox();
    for (uint32_t t = first; t < first + count; ++t)
      for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) {
          const float x = tris[12 * static_cast<size_t>(t) + 4 * v + a];
          b.lo[a] = std::min(b.lo[a], x);
          b.hi[a] = std::max(b.hi[a], x);
        }
    return b;
  };
  auto refBox = [&](int ref) { return ref >= 0 ? box[ref] : leafBox(ref); };

  const uint32_t F = wideNodeFloat4s(W) * 4;  // floats per wide node
  // Breadth-first: wide node j is made from two-wide node src[j].
  std::vector<uint32_t> src{0u}, depth{0u};
  size_t totalChildren = 0;
  for (size_t j = 0; j < src.size(); ++j) {
    // Children: open the inner child of largest surface area until W.
    std::vector<int> kids;
    int c[2];
    childRefs(src[j], c);
    kids.push_back(c[0]);
    kids.push_back(c[1]);
    while (static_cast<int>(kids.size()) < W) {
      int best = -1;
      double bestArea = -1.0;
      for (size_t k = 0; k < kids.size(); ++k)
        if (kids[k] >= 0 && box[kids[k]].area() > bestArea) {
          bestArea = box[kids[k]].area();
          best = static_cast<int>(k);
        }
      if (best < 0) break;
      const int open = kids[best];
      childRefs(static_cast<uint32_t>(open), c);
      kids[best] = c[0];
      kids.insert(kids.begin() + best + 1, c[1]);
    }
    totalChildren += kids.size();
    // Refs: inner children become wide nodes (appended to the queue).
    std::vector<int32_t> refs(kids.size());
    std::vector<Box> kb(kids.size());
    for (size_t k = 0; k < kids.size(); ++k) {
      kb[k] = refBox(kids[k]);
      if (kids[k] >= 0) {
        refs[k] = static_cast<int32_t>(src.size());
        src.push_back(static_cast<uint32_t>(kids[k]));
        depth.push_back(depth[j] + 1);
        stats.maxDepth = std::max(stats.maxDepth, depth[j] + 1);
      } else {
        refs[k] = kids[k];
      }
    }
    // Quantisation: origin at the node box's lower corner, per axis the
    // smallest power-of-two scale with 255 steps covering the box; child
    // planes rounded outward, in exact (double) arithmetic.
    Box nb = emptyBox();
    for (const Box& b : kb) nb.grow(b);
    float p[3];
    uint32_t ebits[3];
    double scale[3];
    for (int a = 0; a < 3; ++a) {
      p[a] = nb.lo[a];
      const double ext = double(nb.hi[a]) - double(p[a]);
      int e = -126;
      if (ext > 0.0) {
        e = static_cast<int>(std::ceil(std::log2(ext / 255.0)));
        while (std::ldexp(255.0, e) < ext) ++e;
        while (e > -126 && std::ldexp(255.0, e - 1) >= ext) --e;
        e = std::max(-126, std::min(127, e));
      }
      scale[a] = std::ldexp(1.0, e);
      ebits[a] = static_cast<uint32_t>(e + 127);
    }
    uint8_t qlo[3][8], qhi[3][8];
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 8; ++k) {
        qlo[a][k] = 255;  // empty slot: an inverted box
        qhi[a][k] = 0;
      }
    for (size_t k = 0; k < kb.size(); ++k)
      for (int a = 0; a < 3; ++a) {
        const double l = std::floor((double(kb[k].lo[a]) - p[a]) / scale[a]);
        const double h = std::ceil((double(kb[k].hi[a]) - p[a]) / scale[a]);
        if (!(l >= 0.0 && h <= 255.0 && l <= h)) throw std::runtime_error("wide BVH: quantisation out of range");
        qlo[a][k] = static_cast<uint8_t>(l);
        qhi[a][k] = static_cast<uint8_t>(h);
      }
    float node[24] = {};
    node[0] = p[0];
    node[1] = p[1];
    node[2] = p[2];
    const uint32_t meta = ebits[0] | (ebits[1] << 8) | (ebits[2] << 16) | (static_cast<uint32_t>(kb.size()) << 24);
    std::memcpy(&node[3], &meta, 4);
    auto word = [&](const uint8_t* q, int first) {
      return static_cast<uint32_t>(q[first]) | (static_cast<uint32_t>(q[first + 1]) << 8) |
             (static_cast<uint32_t>(q[first + 2]) << 16) | (static_cast<uint32_t>(q[first + 3]) << 24);
    };
    uint32_t w[12];
    int nw = 0;
    if (W == 4) {
      w[nw++] = word(qlo[0], 0);
      w[nw++] = word(qlo[1], 0);
      w[nw++] = word(qlo[2], 0);
      w[nw++] = word(qhi[0], 0);
      w[nw++] = word(qhi[1], 0);
      w[nw++] = word(qhi[2], 0);
      w[nw++] = 0;
      w[nw++] = 0;
    } else {
      for (int half = 0; half < 2; ++half) {  // lo then hi, axes x y z, children 0-3 then 4-7
        const uint8_t(*q)[8] = half == 0 ? qlo : qhi;
        for (int a = 0; a < 3; ++a) {
          w[nw++] = word(q[a], 0);
          w[nw++] = word(q[a], 4);
        }
      }
    }
    std::memcpy(&node[4], w, 4 * nw);
    int32_t r[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t k = 0; k < refs.size(); ++k) r[k] = refs[k];
    std::memcpy(&node[4 + nw], r, 4 * W);
    out.insert(out.end(), node, node + F);
  }
  stats.nodes = static_cast<uint32_t>(src.size());
  stats.meanChildren = static_cast<double>(totalChildren) / static_cast<double>(src.size());
}

}  // namespace cr
