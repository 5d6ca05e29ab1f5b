// render.cuh -- launch parameters and launchers of the per-frame kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/j3dg.h"

namespace j3dg {

struct DevInst;

// Primary hits by conservative rasterisation (FrameParams::raster): per
// instance, the object -> clip matrix of the frame's camera and the slab
// padding of the camera's rays in object space.
struct RasterInst {
  float M[16];     // clip = proj * cs_inv * inst.cs (column-major)
  float pad;       // make_ray's padding for rays from the camera
  uint32_t first;  // first work item of the instance (prefix of nt)
  uint32_t nt;
  uint32_t unused;
};
// rlist: [0] large triangles listed, [1] list overflow, then the count of
// candidates queued in each stripe of the queue, one 128-byte line apart (so
// that the stripes' atomics go to different L2 lines); entries from
// kRasterListHeader
static const uint32_t kRasterStripes = 64;
static const uint32_t kRasterCounterStride = 32;
static const uint32_t kRasterListHeader = 32 + kRasterStripes * kRasterCounterStride;
__host__ __device__ inline uint32_t raster_stripe_counter(uint32_t s) { return 32 + s * kRasterCounterStride; }
static const uint32_t kRasterEntryWords = 8;  // inst, slot, x0, y0, x1, y1, -, -

struct FrameParams {
  const DevInst* inst;
  uint32_t n_inst;
  uint32_t top;    // 1: the instance table carries a top level and the kernels walk it
  uint32_t width;  // children per BVH node of the frame's meshes (2, 4, 8)
  uint32_t w, h;
  int x0, y0, x1, y1;
  float cs[16], cs_inv[16], pinv[16];
  float pivot[3];
  float diagonal;
  float near_plane;
  j3dg_pixel* gbuf;
  uint32_t* im;
  const uint32_t* background;
  const uint32_t* matcap;
  uint32_t mw, mh, cavity;
  uint32_t shadow, textured, vertexcolors, shading;
  int shade_mode;  // 0: G-buffer only; 1: also plain shading into im (misses <- background)
  // [0..3] rasterised frames: [0] primary items taken, [1] shadow jobs queued,
  // [2] taken; k_frame: [4 + seq % kFrameDepth] items taken,
  // [4 + kFrameDepth + seq % kFrameDepth] warps done (the frame's last warp
  // zeroes both)
  uint32_t* work;
  uint32_t* status;
  unsigned long long* counters;  // optional [node visits, triangle tests]
  // raster != 0: launch_render first fills keys[w*h] with the minimum of
  // (t bits << 32 | inst << id_bits | triangle id) over each pixel's
  // accepted triangles (id_bits 32: one instance), and k_frame takes the
  // primary hit from there instead of tracing
  uint32_t raster;
  uint32_t id_bits;
  uint32_t raster_total;  // triangles of all instances
  uint32_t rlist_cap;     // large-triangle entries that fit rlist
  float proj[16];         // the canvas projection
  unsigned long long* keys;
  RasterInst* rinst;      // n_inst entries
  uint32_t* rlist;        // counters, then the large-triangle entries (kRasterListHeader)
  // Frames of one canvas may overlap (k_frame launched as a programmatic
  // dependent of the canvas's previous frame): seq is the frame's number
  // (>= 1), stamps (w*h, or null: not written) the number of the frame that
  // last wrote each pixel, stored after the pixel's last write, and a frame
  // with wait_seq != 0 waits before its first write of a pixel until the
  // pixel carries wait_seq, so that every pixel's writes stay in frame order.
  uint32_t* stamps;
  uint32_t seq, wait_seq;
  // frame kernels of the context, in launch order: launch is this one's
  // number (>= 1), ring[launch % kFrameDepth] the number of the last frame
  // kernel that released that entry (at its end, once every frame before it
  // had completed)
  uint32_t* ring;
  uint32_t launch;
};
static const uint32_t kFrameDepth = 4;                     // frame kernels in flight at most
static const uint32_t kCanvasWorkWords = 4 + 2 * kFrameDepth;  // FrameParams::work

cudaError_t launch_render(const FrameParams& P, cudaStream_t st);
// all frames in one persistent launch; offsets = prefix sums of primary_items
// total_items = offsets[n_frames] (the sum of primary_items of the frames)
// (every frame's meshes have BVH width `width`)
cudaError_t launch_render_batch(const FrameParams* d_params, const uint32_t* d_offsets, uint32_t n_frames,
                                uint32_t total_items, uint32_t* work, int block_threads, bool top, int width,
                                cudaStream_t st);
uint32_t primary_items(const FrameParams& P);
// mode: 0 plain, 1 edges, 2 wireframe, 3 one-bit
cudaError_t launch_shade(const FrameParams& P, const j3dg_pixel* G, int mode, int fill_background, cudaStream_t st);
// primary rays of the frame's rectangle, row-major (the rays k_frame traces)
cudaError_t launch_primary_rays(const FrameParams& P, j3dg_ray* out, cudaStream_t st);
// a frame from primary hits found elsewhere (one j3dg_hit per ray of
// launch_primary_rays): hit records, shadow rays, plain shading; P needs the
// raster scratch layout (keys, jobs, list) of its canvas
cudaError_t launch_frame_from_hits(const FrameParams& P, const j3dg_hit* hits, cudaStream_t st);
cudaError_t launch_copy_u32(uint32_t* dst, const uint32_t* src, size_t n, cudaStream_t st);
cudaError_t launch_clear_ids(j3dg_pixel* G, size_t n, cudaStream_t st);
cudaError_t launch_init_pixels(j3dg_pixel* G, size_t n, cudaStream_t st);
cudaError_t launch_rays(const DevInst* inst, uint32_t n_inst, bool top, int width, const j3dg_ray* rays, uint32_t n,
                        j3dg_hit* hits, bool any, uint32_t* counter, uint32_t* status, unsigned long long* counters,
                        cudaStream_t st);

}  // namespace j3dg
