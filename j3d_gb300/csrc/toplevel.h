// toplevel.h -- host build of the per-frame top level over a scene's objects
// (the two-level structure of canvas.cpp:762); see toplevel.cpp.
#pragma once
#include <stdint.h>

namespace j3dg {

struct TopLevel {
  bool ok = false;        // false: no top level (the kernels walk the objects in turn)
  uint32_t root = 0;      // inner node 0, or the leaf of the only object
  uint32_t n_nodes = 0;
  uint32_t depth = 0;     // inner-node levels
  uint32_t n_inst = 0;
  float pad_scale = 0.f;  // max |coordinate| of the padded object boxes
};

// A BVH of width W (2, 4, 8; the meshes' node layout, J3DG_NODE_F4) over the
// n objects' padded world boxes. nodes: room for node_cap nodes; n objects
// need n - 1 at most.
TopLevel build_top_level(const float* const* mesh_lo, const float* const* mesh_hi, const float* const* cs, uint32_t n,
                         uint32_t W, float* nodes, uint32_t node_cap);

}  // namespace j3dg
