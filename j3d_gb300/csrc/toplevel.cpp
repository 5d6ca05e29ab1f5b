// toplevel.cpp -- the per-frame top level over a scene's objects.
//
// qbvh_two_level_with_transformations (canvas.cpp:762) is built every frame
// over all scene objects with their 4x4 transforms, and closest-hit and
// shadow queries go through it (canvas.cpp:786, 854). Here the top level is
// a small BVH over the objects' world-space boxes, built on the host when the
// instance table is written (a few microseconds for hundreds of objects) and
// uploaded with the table; the traversal kernels walk it with the world ray,
// take an object's BVH with the object-space ray at a top-level leaf, and come
// back. Node layout = the meshes' nodes of the same width W (J3DG_NODE_F4:
// planes [6][W], refs [W]); a leaf holds one object: ref = J3DG_LEAF_BIT |
// object << 3.
//
// Culling at the top level never changes a result: the boxes are padded
// outward (relative 2^-20 of each box's magnitude plus outward rounding to
// float) and the kernels pad the world ray's slab test by
// (max|origin| + pad_scale) 2^-12, far above the rounding between the world
// ray and the object-space ray (a few ulps of |origin| + |box|) through a
// rigid transform, so every object-space hit lies inside its object's
// padded top-level box and no object holding a candidate is culled.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

#include "internal.h"
#include "toplevel.h"

namespace j3dg {

namespace {

struct Box {
  double lo[3], hi[3];
};

struct Builder {
  const std::vector<Box>& box;
  std::vector<uint32_t> idx;
  float* nodes;  // 4 J3DG_NODE_F4(W) floats per node
  uint32_t W, cap, n_nodes = 0, depth = 0;

  Builder(const std::vector<Box>& b, uint32_t width, float* out, uint32_t node_cap)
      : box(b), nodes(out), W(width), cap(node_cap) {
    idx.resize(b.size());
    std::iota(idx.begin(), idx.end(), 0u);
  }

  static Box unite(const std::vector<Box>& bx, const uint32_t* first, const uint32_t* last) {
    Box u;
    for (int a = 0; a < 3; ++a) {
      u.lo[a] = std::numeric_limits<double>::infinity();
      u.hi[a] = -std::numeric_limits<double>::infinity();
    }
    for (const uint32_t* p = first; p != last; ++p)
      for (int a = 0; a < 3; ++a) {
        u.lo[a] = std::min(u.lo[a], bx[*p].lo[a]);
        u.hi[a] = std::max(u.hi[a], bx[*p].hi[a]);
      }
    return u;
  }

  // splits [b, e) at its centroid median along the widest centroid axis
  uint32_t split(uint32_t b, uint32_t e) {
    double clo[3], chi[3];
    for (int a = 0; a < 3; ++a) {
      clo[a] = std::numeric_limits<double>::infinity();
      chi[a] = -std::numeric_limits<double>::infinity();
    }
    for (uint32_t i = b; i < e; ++i)
      for (int a = 0; a < 3; ++a) {
        const double c = box[idx[i]].lo[a] + box[idx[i]].hi[a];
        clo[a] = std::min(clo[a], c);
        chi[a] = std::max(chi[a], c);
      }
    int ax = 0;
    for (int a = 1; a < 3; ++a)
      if (chi[a] - clo[a] > chi[ax] - clo[ax]) ax = a;
    const uint32_t m = b + (e - b) / 2;
    std::nth_element(idx.begin() + b, idx.begin() + m, idx.begin() + e, [&](uint32_t x, uint32_t y) {
      const double cx = box[x].lo[ax] + box[x].hi[ax], cy = box[y].lo[ax] + box[y].hi[ax];
      return cx < cy || (cx == cy && x < y);
    });
    return m;
  }

  // splits [b, e) into up to `groups` ranges (a power of 2) by repeated
  // median splits; g receives the range boundaries
  void groups_of(uint32_t b, uint32_t e, uint32_t groups, std::vector<uint32_t>& g) {
    if (groups == 1 || e - b < 2) {
      g.push_back(b);
      return;
    }
    const uint32_t m = split(b, e);
    groups_of(b, m, groups / 2, g);
    groups_of(m, e, groups / 2, g);
  }

  // returns the ref of the subtree over idx[b, e)
  uint32_t build(uint32_t b, uint32_t e, uint32_t level) {
    if (e - b == 1) return J3DG_LEAF_BIT | (idx[b] << 3);
    const uint32_t node = n_nodes++;
    depth = std::max(depth, level + 1);
    std::vector<uint32_t> g;
    groups_of(b, e, W, g);
    g.push_back(e);
    const int ng = (int)g.size() - 1;
    const uint32_t F = 4 * J3DG_NODE_F4(W);
    float* N = nodes + (size_t)F * node;
    for (uint32_t k = 0; k < F; ++k) N[k] = 0.f;
    for (uint32_t c = 0; c < W; ++c) {
      N[0 * W + c] = N[2 * W + c] = N[4 * W + c] = std::numeric_limits<float>::infinity();
      N[1 * W + c] = N[3 * W + c] = N[5 * W + c] = -std::numeric_limits<float>::infinity();
      const uint32_t empty = J3DG_EMPTY_REF;
      std::memcpy(N + 6 * W + c, &empty, 4);
    }
    for (int c = 0; c < ng; ++c) {
      const Box u = unite(box, idx.data() + g[c], idx.data() + g[c + 1]);
      const uint32_t ref = build(g[c], g[c + 1], level + 1);
      for (int a = 0; a < 3; ++a) {
        N[(2 * a) * W + c] = (float)u.lo[a];  // already representable: boxes are rounded outward to float
        N[(2 * a + 1) * W + c] = (float)u.hi[a];
      }
      std::memcpy(N + 6 * W + c, &ref, 4);
    }
    return node;
  }
};

// x rounded to float towards -inf / +inf
float down(double x) {
  float f = (float)x;
  return (double)f > x ? std::nextafter(f, -std::numeric_limits<float>::infinity()) : f;
}
float up(double x) {
  float f = (float)x;
  return (double)f < x ? std::nextafter(f, std::numeric_limits<float>::infinity()) : f;
}

}  // namespace

TopLevel build_top_level(const float* const* mesh_lo, const float* const* mesh_hi, const float* const* cs, uint32_t n,
                         uint32_t W, float* nodes, uint32_t node_cap) {
  TopLevel t;
  t.n_inst = n;
  if (n == 0) return t;
  std::vector<Box> box(n);
  double scale = 0.0;
  for (uint32_t i = 0; i < n; ++i) {
    Box& b = box[i];
    for (int a = 0; a < 3; ++a) {
      b.lo[a] = std::numeric_limits<double>::infinity();
      b.hi[a] = -std::numeric_limits<double>::infinity();
    }
    const float* M = cs[i];
    for (int k = 0; k < 8; ++k) {
      const double p[3] = {(k & 1) ? mesh_hi[i][0] : mesh_lo[i][0], (k & 2) ? mesh_hi[i][1] : mesh_lo[i][1],
                           (k & 4) ? mesh_hi[i][2] : mesh_lo[i][2]};
      for (int a = 0; a < 3; ++a) {
        const double w = (double)M[a] * p[0] + (double)M[4 + a] * p[1] + (double)M[8 + a] * p[2] + (double)M[12 + a];
        b.lo[a] = std::min(b.lo[a], w);
        b.hi[a] = std::max(b.hi[a], w);
      }
    }
    for (int a = 0; a < 3; ++a) {
      const double mag = std::max(std::fabs(b.lo[a]), std::fabs(b.hi[a]));
      b.lo[a] = down(b.lo[a] - mag * 0x1p-20);
      b.hi[a] = up(b.hi[a] + mag * 0x1p-20);
      scale = std::max(scale, std::max(std::fabs(b.lo[a]), std::fabs(b.hi[a])));
    }
  }
  t.pad_scale = up(scale);
  if (!std::isfinite(t.pad_scale)) return t;  // non-finite boxes: no top level (objects are walked in turn)
  if (n > node_cap + 1 || n > (1u << 28) || (W != 2 && W != 4 && W != 8)) return t;
  Builder B(box, W, nodes, node_cap);
  t.root = B.build(0, n, 0);
  t.n_nodes = B.n_nodes;
  t.depth = B.depth;
  t.ok = true;
  return t;
}

}  // namespace j3dg
