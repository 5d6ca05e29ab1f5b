// render_dispatch.cu -- the per-frame launchers of render.cuh. render.cu is
// compiled once per BVH width (namespaces w2, w4, w8); the launchers that
// trace call the build for the width of the frame's meshes, the others the
// w4 build.
#include "render.cuh"

namespace j3dg {

#define J3DG_RENDER_DECLS                                                                                         \
  cudaError_t launch_render(const FrameParams& P, cudaStream_t st);                                               \
  cudaError_t launch_render_batch(const FrameParams* d_params, const uint32_t* d_offsets, uint32_t n_frames,      \
                                  uint32_t total_items, uint32_t* work, int block_threads, bool top, int width,   \
                                  cudaStream_t st);                                                               \
  uint32_t primary_items(const FrameParams& P);                                                                   \
  cudaError_t launch_shade(const FrameParams& P, const j3dg_pixel* G, int mode, int fill_background,             \
                           cudaStream_t st);                                                                      \
  cudaError_t launch_primary_rays(const FrameParams& P, j3dg_ray* out, cudaStream_t st);                          \
  cudaError_t launch_frame_from_hits(const FrameParams& P, const j3dg_hit* hits, cudaStream_t st);                \
  cudaError_t launch_copy_u32(uint32_t* dst, const uint32_t* src, size_t n, cudaStream_t st);                     \
  cudaError_t launch_clear_ids(j3dg_pixel* G, size_t n, cudaStream_t st);                                         \
  cudaError_t launch_init_pixels(j3dg_pixel* G, size_t n, cudaStream_t st);                                       \
  cudaError_t launch_rays(const DevInst* inst, uint32_t n_inst, bool top, int width, const j3dg_ray* rays,        \
                          uint32_t n, j3dg_hit* hits, bool any, uint32_t* counter, uint32_t* status,              \
                          unsigned long long* counters, cudaStream_t st);

namespace w2 {
J3DG_RENDER_DECLS
}
namespace w4 {
J3DG_RENDER_DECLS
}
namespace w8 {
J3DG_RENDER_DECLS
}

cudaError_t launch_render(const FrameParams& P, cudaStream_t st) {
  if (P.width == 2) return w2::launch_render(P, st);
  if (P.width == 8) return w8::launch_render(P, st);
  if (P.width != 4) return cudaErrorInvalidValue;
  return w4::launch_render(P, st);
}

cudaError_t launch_render_batch(const FrameParams* d_params, const uint32_t* d_offsets, uint32_t n_frames,
                                uint32_t total_items, uint32_t* work, int block_threads, bool top, int width,
                                cudaStream_t st) {
  if (width == 2) return w2::launch_render_batch(d_params, d_offsets, n_frames, total_items, work, block_threads, top, 2, st);
  if (width == 8) return w8::launch_render_batch(d_params, d_offsets, n_frames, total_items, work, block_threads, top, 8, st);
  if (width != 4) return cudaErrorInvalidValue;
  return w4::launch_render_batch(d_params, d_offsets, n_frames, total_items, work, block_threads, top, 4, st);
}

cudaError_t launch_frame_from_hits(const FrameParams& P, const j3dg_hit* hits, cudaStream_t st) {
  if (P.width == 2) return w2::launch_frame_from_hits(P, hits, st);
  if (P.width == 8) return w8::launch_frame_from_hits(P, hits, st);
  if (P.width != 4) return cudaErrorInvalidValue;
  return w4::launch_frame_from_hits(P, hits, st);
}

cudaError_t launch_rays(const DevInst* inst, uint32_t n_inst, bool top, int width, const j3dg_ray* rays, uint32_t n,
                        j3dg_hit* hits, bool any, uint32_t* counter, uint32_t* status, unsigned long long* counters,
                        cudaStream_t st) {
  if (width == 2) return w2::launch_rays(inst, n_inst, top, 2, rays, n, hits, any, counter, status, counters, st);
  if (width == 8) return w8::launch_rays(inst, n_inst, top, 8, rays, n, hits, any, counter, status, counters, st);
  if (width != 4) return cudaErrorInvalidValue;
  return w4::launch_rays(inst, n_inst, top, 4, rays, n, hits, any, counter, status, counters, st);
}

uint32_t primary_items(const FrameParams& P) { return w4::primary_items(P); }
cudaError_t launch_shade(const FrameParams& P, const j3dg_pixel* G, int mode, int fill_background, cudaStream_t st) {
  return w4::launch_shade(P, G, mode, fill_background, st);
}
cudaError_t launch_primary_rays(const FrameParams& P, j3dg_ray* out, cudaStream_t st) {
  return w4::launch_primary_rays(P, out, st);
}
cudaError_t launch_copy_u32(uint32_t* dst, const uint32_t* src, size_t n, cudaStream_t st) {
  return w4::launch_copy_u32(dst, src, n, st);
}
cudaError_t launch_clear_ids(j3dg_pixel* G, size_t n, cudaStream_t st) { return w4::launch_clear_ids(G, n, st); }
cudaError_t launch_init_pixels(j3dg_pixel* G, size_t n, cudaStream_t st) { return w4::launch_init_pixels(G, n, st); }

}  // namespace j3dg
