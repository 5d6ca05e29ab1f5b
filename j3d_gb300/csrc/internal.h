// internal.h -- host-side definitions of the opaque C-ABI objects.
#pragma once
#include <stdint.h>

#include <atomic>

#include <string>

#include "../../include/j3dg.h"

// Wide-node child reference: inner node index, or a leaf of up to 8
// consecutive triangles of the leaf-ordered triangle array.
#define J3DG_LEAF_BIT 0x80000000u
#define J3DG_EMPTY_REF 0xffffffffu
#define J3DG_MAX_LEAF 8u
#define J3DG_MAX_TRIANGLES (1u << 28)
// Traversal stack entries per thread; builds whose depth could overflow it
// are refused at build time, so the device check never fires on valid BVHs.
#define J3DG_STACK 96
#define J3DG_MAX_DEPTH ((J3DG_STACK - 1) / 3)
// Wide nodes of width W (2, 4 or 8 children): the child boxes as floats
// [6][W] (planes lo.x, hi.x, lo.y, hi.y, lo.z, hi.z; child c of plane p at
// p W + c), then the W child refs, padded to whole 64-byte lines: 64 B
// (W = 2), 128 B (W = 4), 256 B (W = 8). A level pushes up to W - 1 stack
// entries, so the deepest tree a width allows is J3DG_MAX_DEPTH_W(W).
#define J3DG_NODE_F4(W) (((7 * (W)) + 15) / 16 * 4)
#define J3DG_MAX_DEPTH_W(W) ((J3DG_STACK - 1) / ((W) - 1))

struct j3dg_ctx {
  int device = 0;
  void* stream = nullptr;        // cudaStream_t
  void* copy_stream = nullptr;   // cudaStream_t of asynchronous canvas downloads
  uint32_t* d_status = nullptr;  // device status word
  void* d_inst = nullptr;        // device instance table (DevInst[])
  uint32_t inst_cap = 0;
  void* h_inst = nullptr;        // pinned staging for the instance table
  int sm_count = 0;
  // library calls that took the context stream: a frame overlaps the kernel
  // before it only when that kernel is the previous frame (nothing between)
  uint64_t stream_ops = 0;
  std::string last_error;
  std::atomic<uint32_t> live{0};  // meshes, canvases, ... made from this context and not destroyed
};

// Member of every object made from a context: counts the object in the
// context's `live` from attach() until the object is deleted, so that
// j3dg_ctx_destroy can refuse to free a context that objects still use.
struct CtxHold {
  j3dg_ctx* ctx = nullptr;
  CtxHold() = default;
  CtxHold(const CtxHold&) = delete;
  CtxHold& operator=(const CtxHold&) = delete;
  void attach(j3dg_ctx* c) {
    ctx = c;
    if (c) c->live.fetch_add(1);
  }
  ~CtxHold() {
    if (ctx) ctx->live.fetch_sub(1);
  }
};

struct j3dg_mesh {
  j3dg_ctx* ctx = nullptr;
  CtxHold hold;
  uint32_t nv = 0, nt = 0;
  float min_bb[3] = {0, 0, 0}, max_bb[3] = {0, 0, 0};
  float scale = 0.f;  // max |coordinate| of the bbox corners
  uint32_t leaf_size = 4;
  uint32_t width = 4;        // children per BVH node: 2, 4 or 8
  uint32_t build_flags = 0;  // j3dg_build_opts::flags
  uint32_t n_nodes = 0, max_depth = 0, root_ref = 0;
  float build_ms = 0.f;
  uint64_t device_bytes = 0;
  void* d_nodes = nullptr;    // float4[8 * n_nodes]
  void* d_tris = nullptr;     // float4[3 * nt], leaf order, v0.w = triangle id
  void* d_normals = nullptr;  // float4[nt], by triangle id
  void* d_slot_of = nullptr;  // uint32[nt]: leaf-order position of each triangle id
  void* d_index = nullptr;    // uint32[3 * nt], the caller's triangles
  void* d_verts = nullptr;    // float[3 * nv], kept by rebuildable meshes (J3DG_BUILD_REBUILDABLE)
  void* d_colors = nullptr;   // float[3 * nv] or null
  void* d_uv = nullptr;       // float[6 * nt] or null
  void* d_tex = nullptr;      // uint32[tex_w * tex_h] or null
  uint32_t tex_w = 0, tex_h = 0;
};

struct j3dg_matcap {
  j3dg_ctx* ctx = nullptr;
  CtxHold hold;
  uint32_t w = 0, h = 0, cavity = 0;
  uint32_t* d_pixels = nullptr;
};

struct j3dg_canvas {
  j3dg_ctx* ctx = nullptr;
  CtxHold hold;
  uint32_t w = 0, h = 0;
  j3dg_camera camera;
  float projection[16], projection_inv[16];
  j3dg_canvas_settings settings;
  void* d_pixels = nullptr;      // j3dg_pixel[w*h]
  uint32_t* d_image = nullptr;   // w*h
  uint32_t* d_background = nullptr;
  void* d_queue = nullptr;       // 48 B per pixel: raster keys, jobs and tables during a frame, splat keys after
  uint32_t* d_work = nullptr;    // per-frame work counters (kCanvasWorkWords)
  uint32_t* d_stamps = nullptr;  // w*h: number of the traced frame that last wrote each pixel
  uint32_t seq = 0;              // traced frames launched on this canvas
  uint32_t stamp_seq = 0;        // every pixel carries this frame number (0: not known, no overlap)
  bool expect_stamps = false;    // the next traced frame waits for stamp_seq (j3dg_canvas_expect_frame)
  int last_primary = 1;          // J3DG_PRIMARY_TRACE or J3DG_PRIMARY_RASTER
  // asynchronous download: ev_ready marks the work queued before it, ev_copied its end
  void* ev_ready = nullptr;
  void* ev_copied = nullptr;
  bool copy_pending = false;
};

// Decoded mesh / point-cloud file on the device (ingest.cu).
struct j3dg_geometry {
  j3dg_ctx* ctx = nullptr;
  CtxHold hold;
  uint64_t nv = 0, nt = 0;
  float* d_v = nullptr;      // 3 nv
  uint32_t* d_t = nullptr;   // 3 nt
  uint32_t* d_c = nullptr;   // nv packed RGBA8, or null
  float* d_n = nullptr;      // 3 nv, or null
  float* d_uv = nullptr;     // 6 nt, or null
  j3dg_geometry_info info;
};

// Point cloud on the device (pointcloud.cu).
struct j3dg_pointcloud {
  j3dg_ctx* ctx = nullptr;
  CtxHold hold;
  uint64_t n = 0;
  float* d_v = nullptr;      // 3 n
  uint32_t* d_c = nullptr;   // n packed RGBA8, or null
  float min_bb[3] = {0, 0, 0}, max_bb[3] = {0, 0, 0};
};
