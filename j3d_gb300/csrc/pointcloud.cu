// pointcloud.cu -- point clouds on the device and their splat onto a
// rendered canvas (canvas::render_pointclouds_on_image, canvas.cpp:952-1030).
//
// The depth test is a 64-bit atomicMax per point on a key per pixel:
//   high 32 bits: the bits of 1/depth (non-negative floats order like their
//                 bit patterns), larger = nearer;
//   low 32 bits:  0xfffffffe - vertex id for a point of the cloud being
//                 drawn, 0xffffffff for what is already on the canvas.
// A point therefore wins only with a strictly greater 1/depth, and among
// equal depths the smallest vertex id wins -- the order a sequential
// rasteriser with a strict depth test gives. After each cloud a resolve pass
// writes the winners' G-buffer fields and colours and marks them as canvas
// (low bits all ones), so later clouds test against them. The keys live in
// the canvas's frame scratch, which is idle between frames.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "../../include/j3dg.h"
#include "device_common.cuh"
#include "internal.h"

namespace j3dg {
int ctx_fail(j3dg_ctx* c, int code, const std::string& msg);
void canvas_writable(j3dg_canvas* cv);
}

namespace {

using j3dg::fa;
using j3dg::fm;
using j3dg::mat_vec;

cudaStream_t S(j3dg_ctx* c) {
  ++c->stream_ops;
  return (cudaStream_t)c->stream;
}

int fail(j3dg_ctx* c, int code, const std::string& msg) { return j3dg::ctx_fail(c, code, msg); }

int cuda_fail(j3dg_ctx* c, cudaError_t e, const char* where) {
  if (e == cudaErrorMemoryAllocation) return fail(c, J3DG_ERR_OUT_OF_MEMORY, std::string(where) + ": out of device memory");
  return fail(c, J3DG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CKP(x, where)                                  \
  do {                                                 \
    cudaError_t e_ = (x);                              \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, where); \
  } while (0)

bool is_device_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

const uint32_t kMaxPoints = 0xfffffff0u;
const int kBoundsBlocks = 1024;

// compute_bb (mesh.cpp:39-58): per-block min/max, finished on the host.
__global__ void k_bounds(const float* __restrict__ V, uint64_t n, float* __restrict__ partial) {
  __shared__ float s[6][256];
  float mn[3] = {V[0], V[1], V[2]}, mx[3] = {V[0], V[1], V[2]};
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float v = V[3 * i + k];
      mn[k] = v < mn[k] ? v : mn[k];
      mx[k] = mx[k] < v ? v : mx[k];
    }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    s[k][threadIdx.x] = mn[k];
    s[3 + k][threadIdx.x] = mx[k];
  }
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float a = s[k][threadIdx.x + w], b = s[3 + k][threadIdx.x + w];
        s[k][threadIdx.x] = a < s[k][threadIdx.x] ? a : s[k][threadIdx.x];
        s[3 + k][threadIdx.x] = s[3 + k][threadIdx.x] < b ? b : s[3 + k][threadIdx.x];
      }
    __syncthreads();
  }
  if (threadIdx.x < 6) partial[6 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

// canvas.cpp:961-968: 1/depth of the mesh pixels, 0 elsewhere.
__global__ void k_zinit(const j3dg_pixel* __restrict__ G, uint64_t n, unsigned long long* __restrict__ keys) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t db = G[i].db_id;
  const uint32_t z = db != 0 ? __float_as_uint(__fdiv_rn(1.f, G[i].depth)) : 0u;
  keys[i] = ((unsigned long long)z << 32) | 0xffffffffull;
}

struct SplatParams {
  float obj_cs[16];    // pc::cs
  float cs_inv[16];    // scene coordinate_system_inv
  float proj[16];      // canvas projection
  float near_plane;
  float half_w, half_h;
  uint32_t w, h;
};

// One point: camera space through the cloud's cs and the scene's inverse
// pose, then the pixel whose primary ray (s = 2(x+.5)/w - 1 through the
// inverse projection) passes nearest: s_x = P0 x / d + P8, s_y = P5 y / d + P9
// with d = -z the view-space depth the G-buffer stores.
__global__ void k_splat(const float* __restrict__ V, uint64_t n, const SplatParams p,
                        unsigned long long* __restrict__ keys) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const float4 w4 = mat_vec(p.obj_cs, V[3 * i], V[3 * i + 1], V[3 * i + 2], 1.f);
    const float4 c4 = mat_vec(p.cs_inv, w4.x, w4.y, w4.z, w4.w);
    const float d = -c4.z;
    if (!(d > p.near_plane)) continue;
    const float inv_d = __fdiv_rn(1.f, d);
    const float sx = fa(fm(fm(p.proj[0], c4.x), inv_d), p.proj[8]);
    const float sy = fa(fm(fm(p.proj[5], c4.y), inv_d), p.proj[9]);
    const float fx = fm(fa(sx, 1.f), p.half_w);
    const float fy = fm(fa(sy, 1.f), p.half_h);
    if (!(fx >= 0.f && fx < (float)p.w && fy >= 0.f && fy < (float)p.h)) continue;
    const uint32_t col = min((uint32_t)fx, p.w - 1), row = min((uint32_t)fy, p.h - 1);
    const unsigned long long key = ((unsigned long long)__float_as_uint(inv_d) << 32) | (0xfffffffeu - (uint32_t)i);
    unsigned long long* slot = keys + (size_t)row * p.w + col;
    if (key > *slot) atomicMax(slot, key);  // a stale read only skips keys that lose anyway
  }
}

__global__ void k_resolve(unsigned long long* __restrict__ keys, uint64_t npix, const uint32_t* __restrict__ colors,
                          uint64_t n_points, uint32_t db_id, int one_bit, j3dg_pixel* __restrict__ G,
                          uint32_t* __restrict__ im, uint32_t* status) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const unsigned long long key = keys[i];
  const uint32_t low = (uint32_t)key;
  if (low == 0xffffffffu) return;
  const uint32_t id = 0xfffffffeu - low;
  if (id >= n_points) {
    atomicOr(status, J3DG_DEV_BAD_INDEX);
    return;
  }
  const float inv_d = __uint_as_float((uint32_t)(key >> 32));
  G[i].object_id = id;
  G[i].depth = __fdiv_rn(1.f, inv_d);
  G[i].db_id = db_id;
  im[i] = (colors && !one_bit) ? colors[id] : 0xffffffffu;
  keys[i] = key | 0xffffffffull;
}

int make_pc(j3dg_ctx* c, uint64_t n, j3dg_pointcloud** out, j3dg_pointcloud** pc) {
  if (n == 0) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "pointcloud: no points");
  if (n > kMaxPoints) return fail(c, J3DG_ERR_UNSUPPORTED, "pointcloud: more than 2^32 - 16 points");
  *pc = new (std::nothrow) j3dg_pointcloud();
  if (!*pc) return J3DG_ERR_OUT_OF_MEMORY;
  (*pc)->ctx = c;
  (*pc)->hold.attach(c);
  (*pc)->n = n;
  *out = nullptr;
  return J3DG_OK;
}

void free_pc(j3dg_pointcloud* pc) {
  cudaFree(pc->d_v);
  cudaFree(pc->d_c);
  delete pc;
}

int finish_pc(j3dg_ctx* c, j3dg_pointcloud* pc) {
  float* d_part = nullptr;
  const int blocks = (int)std::min<uint64_t>(kBoundsBlocks, (pc->n + 255) / 256);
  CKP(cudaMalloc(&d_part, sizeof(float) * 6 * blocks), "pointcloud bounds");
  k_bounds<<<blocks, 256, 0, S(c)>>>(pc->d_v, pc->n, d_part);
  cudaError_t e = cudaGetLastError();
  std::vector<float> part(6 * (size_t)blocks);
  if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), d_part, sizeof(float) * part.size(), cudaMemcpyDeviceToHost, S(c));
  if (e == cudaSuccess) e = cudaStreamSynchronize(S(c));
  cudaFree(d_part);
  if (e != cudaSuccess) return cuda_fail(c, e, "pointcloud bounds");
  for (int k = 0; k < 3; ++k) {
    pc->min_bb[k] = part[k];
    pc->max_bb[k] = part[3 + k];
  }
  for (int b = 1; b < blocks; ++b)
    for (int k = 0; k < 3; ++k) {
      pc->min_bb[k] = std::min(pc->min_bb[k], part[6 * b + k]);
      pc->max_bb[k] = std::max(pc->max_bb[k], part[6 * b + 3 + k]);
    }
  return J3DG_OK;
}

}  // namespace

extern "C" {

int j3dg_pointcloud_create(j3dg_ctx* c, const float* V, uint64_t n, const uint32_t* colors, j3dg_pointcloud** out) {
  if (!c || !V || !out) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_pointcloud* pc = nullptr;
  if (int rc = make_pc(c, n, out, &pc)) return rc;
  cudaSetDevice(c->device);
  cudaError_t e = cudaMalloc((void**)&pc->d_v, sizeof(float) * 3 * n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(pc->d_v, V, sizeof(float) * 3 * n, is_device_ptr(V) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                        S(c));
  if (e == cudaSuccess && colors) {
    e = cudaMalloc((void**)&pc->d_c, sizeof(uint32_t) * n);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(pc->d_c, colors, sizeof(uint32_t) * n,
                          is_device_ptr(colors) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, S(c));
  }
  int rc = e == cudaSuccess ? finish_pc(c, pc) : cuda_fail(c, e, "pointcloud_create");
  if (rc != J3DG_OK) {
    cudaStreamSynchronize(S(c));
    free_pc(pc);
    return rc;
  }
  *out = pc;
  return J3DG_OK;
}

int j3dg_pointcloud_from_geometry(j3dg_ctx* c, const j3dg_geometry* g, j3dg_pointcloud** out) {
  if (!c || !g || !out) return J3DG_ERR_INVALID_ARGUMENT;
  if (g->ctx != c) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "pointcloud_from_geometry: geometry of another context");
  return j3dg_pointcloud_create(c, g->d_v, g->nv, g->d_c, out);
}

int j3dg_pointcloud_destroy(j3dg_pointcloud* pc) {
  if (!pc) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(pc->ctx->device);
  cudaStreamSynchronize(S(pc->ctx));
  free_pc(pc);
  return J3DG_OK;
}

int j3dg_pointcloud_get_bounds(const j3dg_pointcloud* pc, float min_bb[3], float max_bb[3]) {
  if (!pc || !min_bb || !max_bb) return J3DG_ERR_INVALID_ARGUMENT;
  memcpy(min_bb, pc->min_bb, sizeof(pc->min_bb));
  memcpy(max_bb, pc->max_bb, sizeof(pc->max_bb));
  return J3DG_OK;
}

int j3dg_canvas_render_pointclouds(j3dg_canvas* cv, const j3dg_scene* s, const j3dg_pointcloud_instance* pcs,
                                   uint32_t n_pcs) {
  if (!cv || !s || (n_pcs && !pcs)) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = cv->ctx;
  for (uint32_t k = 0; k < n_pcs; ++k)
    if (!pcs[k].pointcloud || pcs[k].pointcloud->ctx != c)
      return fail(c, J3DG_ERR_INVALID_ARGUMENT, "render_pointclouds: point cloud missing or of another context");
  const uint64_t npix = (uint64_t)cv->w * cv->h;
  if (n_pcs == 0 || npix == 0) return J3DG_OK;
  cudaSetDevice(c->device);
  j3dg::canvas_writable(cv);
  // the canvas's frame scratch (48 bytes per pixel) is idle between frames
  unsigned long long* keys = (unsigned long long*)cv->d_queue;
  const unsigned pix_blocks = (unsigned)((npix + 255) / 256);
  k_zinit<<<pix_blocks, 256, 0, S(c)>>>((const j3dg_pixel*)cv->d_pixels, npix, keys);
  CKP(cudaGetLastError(), "render_pointclouds");
  SplatParams p;
  memcpy(p.cs_inv, s->coordinate_system_inv, sizeof(p.cs_inv));
  memcpy(p.proj, cv->projection, sizeof(p.proj));
  p.near_plane = cv->camera.near_clipping_plane;
  p.w = cv->w;
  p.h = cv->h;
  p.half_w = 0.5f * (float)cv->w;
  p.half_h = 0.5f * (float)cv->h;
  for (uint32_t k = 0; k < n_pcs; ++k) {
    const j3dg_pointcloud* pc = pcs[k].pointcloud;
    memcpy(p.obj_cs, pcs[k].cs, sizeof(p.obj_cs));
    const unsigned blocks = (unsigned)std::min<uint64_t>((uint64_t)c->sm_count * 8, (pc->n + 255) / 256);
    k_splat<<<blocks, 256, 0, S(c)>>>(pc->d_v, pc->n, p, keys);
    CKP(cudaGetLastError(), "render_pointclouds");
    k_resolve<<<pix_blocks, 256, 0, S(c)>>>(keys, npix, pc->d_c, pc->n, pcs[k].db_id, cv->settings.one_bit,
                                            (j3dg_pixel*)cv->d_pixels, cv->d_image, c->d_status);
    CKP(cudaGetLastError(), "render_pointclouds");
  }
  return J3DG_OK;
}

}  // extern "C"
