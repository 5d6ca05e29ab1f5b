// api.cu -- the extern "C" boundary of libj3dgpu.so (declared in include/j3dg.h).
//
// Objects own device memory; every call runs on the context's one stream.
// Bulk arrays may be host or device pointers (cudaPointerGetAttributes).
// No C++ exception crosses the boundary and there is no CPU fallback.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <cfloat>
#include <new>
#include <string>
#include <vector>
#include <atomic>
#include <thread>

#include "../../include/j3dg.h"
#include "device_common.cuh"
#include "internal.h"
#include "toplevel.h"
#include "query.cuh"
#include "render.cuh"

namespace j3dg {
int build_bvh(j3dg_mesh* m, const float* dV, const uint32_t* dT, cudaStream_t st, uint32_t* d_status,
              cudaEvent_t done, std::string& err);
struct RebuildLane;
int rebuild_lane_alloc(uint32_t nt_max, uint32_t nv_max, uint32_t W, bool ploc, bool lbvh, cudaStream_t st,
                       RebuildLane** out, std::string& err);
void rebuild_lane_free(RebuildLane* L, cudaStream_t st);
cudaError_t rebuild_enqueue(RebuildLane* L, const j3dg_mesh* m, cudaStream_t st, cudaStream_t side, uint32_t* d_status);
}

using j3dg::DevInst;
using j3dg::DevTop;
using j3dg::FrameParams;

namespace {

// ring of instance-table slots: host staging (pinned) -> device
const uint32_t kInstSlots = 8;

// bytes the device's default pool keeps reserved between calls (build scratch)
const uint64_t kKeepReserved = 24ull << 30;

// canvas scratch per pixel: raster keys, shadow jobs and tables during a
// frame; the point-cloud splat's depth keys after it
const size_t kQueueBytesPerPixel = 48, kQueueBytesFixed = 16384;

struct CtxExtra {
  std::vector<DevInst> last;  // the table in the most recent slot
  int last_slot = -1;
  bool last_top = false;      // whether that table's top level is walked
  uint32_t next_slot = 0;
  cudaEvent_t slot_ev[kInstSlots];
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  unsigned long long* d_counters = nullptr;
  uint32_t* d_ray_counter = nullptr;  // work counter of ray-batch queries
  bool counting = false;
  int batch_threads = 128;            // block shape of batched launches
  int primary_mode = J3DG_PRIMARY_AUTO;
  bool top_level = true;              // scenes of several objects walk a top level
  bool frame_overlap = true;          // a canvas's traced frame may start while its previous one finishes
  uint64_t frame_ops = ~0ull;         // stream_ops right after the last traced frame was launched
  uint32_t* d_frame_ring = nullptr;   // FrameParams::ring (kFrameDepth words)
  uint32_t frame_launches = 0;        // frame kernels launched (FrameParams::launch)
  // canvas buffers: stream-ordered allocations from a pool that keeps freed
  // memory reserved, so a server that evicts and re-creates canvases under
  // an HBM cap neither synchronizes the device (as cudaFree does) nor waits
  // for the driver to map memory again
  cudaMemPool_t canvas_pool = nullptr;
  // device addresses of the no-allocation voxel grid's scratch (a file-scope
  // array of the library), looked up once when the context is created
  uint32_t* noalloc_keys = nullptr;
  uint8_t* noalloc_staging = nullptr;
  std::string noalloc_error;
};

int fail(j3dg_ctx* c, int code, const std::string& msg) {
  if (c) c->last_error = msg;
  return code;
}

int cuda_fail(j3dg_ctx* c, cudaError_t e, const char* where) {
  if (e == cudaErrorMemoryAllocation) return fail(c, J3DG_ERR_OUT_OF_MEMORY, std::string(where) + ": out of device memory");
  return fail(c, J3DG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(c, x, where)                          \
  do {                                           \
    cudaError_t e_ = (x);                        \
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

cudaStream_t S(j3dg_ctx* c) {
  ++c->stream_ops;
  return (cudaStream_t)c->stream;
}

// Context layout: the opaque j3dg_ctx plus CtxExtra allocated together.
struct CtxAll {
  j3dg_ctx ctx;
  CtxExtra ex;
  char* h_slots = nullptr;  // pinned, kInstSlots tables of inst_cap objects
};

CtxAll* all(j3dg_ctx* c) { return reinterpret_cast<CtxAll*>(c); }

DevInst to_dev(const j3dg_instance& in) {
  DevInst d;
  memset(&d, 0, sizeof(d));
  const j3dg_mesh* m = in.mesh;
  d.nodes = (const float4*)m->d_nodes;
  d.tris = (const float4*)m->d_tris;
  d.normals = (const float4*)m->d_normals;
  d.slot_of = (const uint32_t*)m->d_slot_of;
  d.index = (const uint32_t*)m->d_index;
  d.colors = (const float*)m->d_colors;
  d.uv = (const float*)m->d_uv;
  d.tex = (const uint32_t*)m->d_tex;
  d.tex_w = m->tex_w;
  d.tex_h = m->tex_h;
  d.root_ref = m->root_ref;
  d.n_nodes = m->n_nodes;
  d.nt = m->nt;
  d.db_id = in.db_id;
  d.scale = m->scale;
  d.width = m->width;
  memcpy(d.cs, in.cs, sizeof(d.cs));
  j3dg_invert_orthonormal(in.cs, d.inv);  // canvas.cpp:734
  return d;
}

// Instance table, on the device and in its pinned staging alike:
// [DevTop][DevInst x cap][top-level BVH4 nodes x cap], 256-byte aligned. The
// kernels receive &DevInst[0] and find the header just in front of it.
size_t table_bytes(uint32_t cap) {
  const size_t node = sizeof(float4) * J3DG_NODE_F4(8);  // the widest node
  const size_t b = sizeof(DevTop) + sizeof(DevInst) * (size_t)cap + node * (size_t)std::max(cap, 1u);
  return (b + 255) & ~size_t(255);
}

// Objects of a scene from which the kernels walk a top level (the two-level
// structure of canvas.cpp:762); a single object is walked directly.
const uint32_t kTopMinObjects = 2;

// Writes the table of the n objects t / objs (capacity cap >= n) into the host
// image h of a table whose device copy lives at d: the header, the objects
// and the top level over their world boxes. Returns the device address of
// DevInst[0]; top tells whether the kernels should walk the top level (it
// exists, the scene has kTopMinObjects objects or more, and the deepest
// object tree under it still fits the traversal stack).
const DevInst* write_table(char* h, char* d, const DevInst* t, const j3dg_instance* objs, uint32_t n, uint32_t cap,
                           bool& top, bool* fits = nullptr) {
  DevTop* H = reinterpret_cast<DevTop*>(h);
  DevInst* I = reinterpret_cast<DevInst*>(h + sizeof(DevTop));
  const size_t off_nodes = sizeof(DevTop) + sizeof(DevInst) * (size_t)cap;
  memcpy(I, t, sizeof(DevInst) * n);
  std::vector<const float*> lo(n), hi(n), cs(n);
  uint32_t deepest = 0;
  for (uint32_t i = 0; i < n; ++i) {
    lo[i] = objs[i].mesh->min_bb;
    hi[i] = objs[i].mesh->max_bb;
    cs[i] = objs[i].cs;
    deepest = std::max(deepest, objs[i].mesh->max_depth);
  }
  const uint32_t W = objs[0].mesh->width;
  const j3dg::TopLevel tl = j3dg::build_top_level(lo.data(), hi.data(), cs.data(), n, W,
                                                  reinterpret_cast<float*>(h + off_nodes), std::max(cap, 1u));
  memset(H, 0, sizeof(DevTop));
  if (tl.ok) {
    H->nodes = reinterpret_cast<const float4*>(d + off_nodes);
    H->root = tl.root;
    H->n_nodes = tl.n_nodes;
    H->n_inst = n;
    H->pad_scale = tl.pad_scale;
  }
  const bool walkable = tl.ok && tl.depth + deepest <= J3DG_MAX_DEPTH_W(W);
  top = walkable && n >= kTopMinObjects;
  if (fits) *fits = walkable;
  return reinterpret_cast<const DevInst*>(d + sizeof(DevTop));
}

// Uploads the instance table (skipped when unchanged); returns its device
// address and whether its top level is walked.
int upload_instances(j3dg_ctx* c, const j3dg_instance* objs, uint32_t n, const DevInst** out, bool* top = nullptr) {
  CtxAll* A = all(c);
  CtxExtra& X = A->ex;
  std::vector<DevInst> t(n);
  for (uint32_t i = 0; i < n; ++i) {
    if (!objs[i].mesh) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "instance without a mesh");
    if (objs[i].mesh->ctx != c) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "mesh belongs to another context");
    if (objs[i].mesh->width != objs[0].mesh->width)
      return fail(c, J3DG_ERR_UNSUPPORTED, "the objects of one scene must share a BVH width");
    t[i] = to_dev(objs[i]);
  }
  if (top) *top = false;
  if (n == 0) {
    *out = nullptr;
    return J3DG_OK;
  }
  if (n > c->inst_cap) {
    // grow both rings (waits for in-flight copies)
    CK(c, cudaStreamSynchronize(S(c)), "instance table");
    uint32_t cap = std::max(n, 2 * c->inst_cap);
    void* d = nullptr;
    char* h = nullptr;
    CK(c, cudaMalloc(&d, table_bytes(cap) * kInstSlots), "instance table");
    if (cudaMallocHost((void**)&h, table_bytes(cap) * kInstSlots) != cudaSuccess) {
      cudaFree(d);
      return fail(c, J3DG_ERR_OUT_OF_MEMORY, "instance table: pinned host allocation failed");
    }
    cudaFree(c->d_inst);
    cudaFreeHost(A->h_slots);
    c->d_inst = d;
    A->h_slots = h;
    c->inst_cap = cap;
    X.last.clear();
    X.last_slot = -1;
  }
  const size_t tb = table_bytes(c->inst_cap);
  if (X.last_slot >= 0 && X.last.size() == n && memcmp(X.last.data(), t.data(), sizeof(DevInst) * n) == 0) {
    *out = reinterpret_cast<const DevInst*>(static_cast<char*>(c->d_inst) + (size_t)X.last_slot * tb + sizeof(DevTop));
    if (top) *top = X.last_top;
    return J3DG_OK;
  }
  uint32_t slot = X.next_slot;
  X.next_slot = (X.next_slot + 1) % kInstSlots;
  CK(c, cudaEventSynchronize(X.slot_ev[slot]), "instance table");
  char* h = A->h_slots + (size_t)slot * tb;
  char* d = static_cast<char*>(c->d_inst) + (size_t)slot * tb;
  bool walk_top = false;
  *out = write_table(h, d, t.data(), objs, n, c->inst_cap, walk_top);
  walk_top = walk_top && X.top_level;
  CK(c, cudaMemcpyAsync(d, h, tb, cudaMemcpyHostToDevice, S(c)), "instance table");
  CK(c, cudaEventRecord(X.slot_ev[slot], S(c)), "instance table");
  X.last = t;
  X.last_slot = (int)slot;
  X.last_top = walk_top;
  if (top) *top = walk_top;
  return J3DG_OK;
}

int check_status(j3dg_ctx* c) {
  uint32_t st = 0;
  CK(c, cudaMemcpyAsync(&st, c->d_status, sizeof(st), cudaMemcpyDeviceToHost, S(c)), "status");
  CK(c, cudaStreamSynchronize(S(c)), "status");
  if (st) {
    CK(c, cudaMemsetAsync(c->d_status, 0, sizeof(uint32_t), S(c)), "status");
    CK(c, cudaStreamSynchronize(S(c)), "status");
    return fail(c, J3DG_ERR_DEVICE_STATUS, "device status word 0x" + std::to_string(st) +
                                               " (1 stack overflow, 2 visit cap, 4 bad index, 8 hit overflow, "
                                               "16 frame wait timeout)");
  }
  return J3DG_OK;
}

// Copies n bytes to dst (host or device) from device src, then synchronizes.
int copy_out(j3dg_ctx* c, void* dst, const void* src, size_t n) {
  cudaMemcpyKind k = is_device_ptr(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  CK(c, cudaMemcpyAsync(dst, src, n, k, S(c)), "copy out");
  return check_status(c);
}

void free_mesh_buffers(j3dg_mesh* m) {
  // the BVH arrays come from the stream-ordered pool, whose cudaFree does not
  // wait for the device: finish every stream's work on them first
  cudaDeviceSynchronize();
  cudaFree(m->d_nodes);
  cudaFree(m->d_tris);
  cudaFree(m->d_normals);
  cudaFree(m->d_slot_of);
  cudaFree(m->d_index);
  cudaFree(m->d_colors);
  cudaFree(m->d_uv);
  cudaFree(m->d_tex);
  cudaFree(m->d_verts);
  m->d_nodes = m->d_tris = m->d_normals = m->d_slot_of = m->d_index = m->d_colors = m->d_uv = m->d_tex = nullptr;
  m->d_verts = nullptr;
}

int shade_mode_of(const j3dg_canvas_settings& s) {
  // canvas.cpp:584-669: one-bit, then wireframe, then edges, else plain
  if (s.one_bit) return 3;
  if (s.wireframe) return 2;
  if (s.edges) return 1;
  return 0;
}

// the numbers of the canvas's next traced frame (never 0) and of the
// context's next frame kernel (never 0)
void next_frame_seq(FrameParams& P, j3dg_canvas* cv) {
  if (++cv->seq == 0u) ++cv->seq;
  P.seq = cv->seq;
  CtxExtra& X = all(cv->ctx)->ex;
  if (++X.frame_launches == 0u) ++X.frame_launches;
  P.launch = X.frame_launches;
  P.ring = X.d_frame_ring;
}

void fill_frame(FrameParams& P, j3dg_canvas* cv, const j3dg_scene* s, const DevInst* inst, const j3dg_matcap* m) {
  memset(&P, 0, sizeof(P));
  P.inst = inst;
  P.n_inst = s ? s->n_objects : 0;
  P.width = (s && s->n_objects && s->objects[0].mesh) ? s->objects[0].mesh->width : 4u;
  P.w = cv->w;
  P.h = cv->h;
  P.x0 = 0;
  P.y0 = 0;
  P.x1 = (int)cv->w - 1;
  P.y1 = (int)cv->h - 1;
  if (s) {
    memcpy(P.cs, s->coordinate_system, sizeof(P.cs));
    memcpy(P.cs_inv, s->coordinate_system_inv, sizeof(P.cs_inv));
    memcpy(P.pivot, s->pivot, sizeof(P.pivot));
    P.diagonal = s->diagonal;
  }
  memcpy(P.pinv, cv->projection_inv, sizeof(P.pinv));
  P.near_plane = cv->camera.near_clipping_plane;
  P.gbuf = (j3dg_pixel*)cv->d_pixels;
  P.im = cv->d_image;
  P.background = cv->d_background;
  if (m) {
    P.matcap = m->d_pixels;
    P.mw = m->w;
    P.mh = m->h;
    P.cavity = m->cavity;
  }
  P.shadow = cv->settings.shadow;
  P.textured = cv->settings.textured;
  P.vertexcolors = cv->settings.vertexcolors;
  P.shading = cv->settings.shading;
  P.status = cv->ctx->d_status;
  P.work = cv->d_work;
  CtxExtra& X = all(cv->ctx)->ex;
  P.counters = X.counting ? X.d_counters : nullptr;
}

// Rasterised primary hits (FrameParams::raster) when the frame allows them:
// every object's box in front of the camera (so no triangle's box reaches
// the camera plane), keys that hold (object, triangle id), and room for the
// tables in the canvas's 48-byte-per-pixel scratch. The automatic mode, if
// kAutoRaster enabled it, would also want at most kRasterTrisPerPixel
// triangles per pixel of the rectangle (reading every triangle once then
// costs less than tracing every pixel).
const double kRasterTrisPerPixel = 24.0;
// the automatic mode traces: on the 28M-triangle torus at 1920x1080 the
// rasterised frame measured slower than the traced one (with and without
// shadow rays), so it is only taken on request
const bool kAutoRaster = false;

uint32_t bits_for(uint32_t v) {  // bits that hold 0..v
  uint32_t b = 1;
  while (b < 32 && (v >> b) != 0) ++b;
  return b;
}

// The canvas scratch as the raster stages use it: keys (8 B per pixel),
// shadow jobs (32 B per pixel), the n objects' table, the large-triangle
// list. Returns false if the scratch is too small.
bool raster_layout(FrameParams& P, j3dg_canvas* cv, uint32_t n, uint32_t id_bits, uint32_t total) {
  const size_t npx = (size_t)cv->w * cv->h, bytes = kQueueBytesPerPixel * npx + kQueueBytesFixed;
  const size_t off_inst = (40 * npx + 255) & ~size_t(255);
  const size_t off_list = (off_inst + sizeof(j3dg::RasterInst) * n + 255) & ~size_t(255);
  const size_t min_entries = 16;
  if (off_list + sizeof(uint32_t) * (j3dg::kRasterListHeader + min_entries * j3dg::kRasterEntryWords) > bytes)
    return false;
  const size_t cap = ((bytes - off_list) / sizeof(uint32_t) - j3dg::kRasterListHeader) / j3dg::kRasterEntryWords;
  char* q = (char*)cv->d_queue;
  P.raster = 1;
  P.id_bits = id_bits;
  P.raster_total = total;
  P.rlist_cap = (uint32_t)std::min<size_t>(cap, 0xffffffffu);
  memcpy(P.proj, cv->projection, sizeof(P.proj));
  P.keys = (unsigned long long*)q;
  P.rinst = (j3dg::RasterInst*)(q + off_inst);
  P.rlist = (uint32_t*)(q + off_list);
  return true;
}

void setup_raster(FrameParams& P, j3dg_canvas* cv, const j3dg_scene* s) {
  const int mode = all(cv->ctx)->ex.primary_mode;
  cv->last_primary = J3DG_PRIMARY_TRACE;
  if (mode == J3DG_PRIMARY_TRACE || !s || s->n_objects == 0 || P.x1 < P.x0 || P.y1 < P.y0) return;
  const uint32_t n = s->n_objects;
  uint64_t total = 0;
  uint32_t max_nt = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const j3dg_mesh* m = s->objects[i].mesh;
    if (!m || !m->d_slot_of || m->nt == 0) return;
    total += m->nt;
    max_nt = std::max(max_nt, m->nt);
  }
  if (total >= (1ull << 32)) return;
  uint32_t id_bits = 32;
  if (n > 1) {
    id_bits = bits_for(max_nt - 1);
    if (id_bits + bits_for(n - 1) > 32) return;
  }
  // camera-space depth -(cs_inv * object cs * corner).z of every box corner
  const double min_depth = 1e-3 * std::max((double)s->diagonal, 1e-30);
  const float* ci = s->coordinate_system_inv;
  for (uint32_t i = 0; i < n; ++i) {
    const j3dg_instance& o = s->objects[i];
    const j3dg_mesh* m = o.mesh;
    for (int k = 0; k < 8; ++k) {
      const double c[3] = {(k & 1) ? m->max_bb[0] : m->min_bb[0], (k & 2) ? m->max_bb[1] : m->min_bb[1],
                           (k & 4) ? m->max_bb[2] : m->min_bb[2]};
      double wld[3];
      for (int r = 0; r < 3; ++r)
        wld[r] = (double)o.cs[r] * c[0] + (double)o.cs[4 + r] * c[1] + (double)o.cs[8 + r] * c[2] + (double)o.cs[12 + r];
      const double z = (double)ci[2] * wld[0] + (double)ci[6] * wld[1] + (double)ci[10] * wld[2] + (double)ci[14];
      if (!(-z > min_depth)) return;
    }
  }
  const uint64_t px = (uint64_t)(P.x1 - P.x0 + 1) * (uint64_t)(P.y1 - P.y0 + 1);
  if (mode == J3DG_PRIMARY_AUTO && (!kAutoRaster || (double)total > kRasterTrisPerPixel * (double)px)) return;
  if (raster_layout(P, cv, n, id_bits, (uint32_t)total)) cv->last_primary = J3DG_PRIMARY_RASTER;
}

}  // namespace
namespace j3dg {
void canvas_writable(j3dg_canvas* cv);
}  // namespace j3dg
namespace {

// Frees the canvas buffers in stream order on the context stream (after a
// download still running on the copy stream, which the stream waits for).
void canvas_release(j3dg_canvas* cv) {
  j3dg_ctx* c = cv->ctx;
  j3dg::canvas_writable(cv);
  void* bufs[6] = {cv->d_pixels, cv->d_image, cv->d_background, cv->d_queue, cv->d_work, cv->d_stamps};
  for (void* b : bufs)
    if (b) cudaFreeAsync(b, S(c));
  cv->d_pixels = cv->d_queue = nullptr;
  cv->d_image = cv->d_background = cv->d_work = cv->d_stamps = nullptr;
  cv->stamp_seq = 0;
}

int canvas_alloc(j3dg_canvas* cv, uint32_t w, uint32_t h) {
  j3dg_ctx* c = cv->ctx;
  canvas_release(cv);
  cv->w = w;
  cv->h = h;
  size_t n = (size_t)w * h;
  if (n) {
    cudaMemPool_t pool = all(c)->ex.canvas_pool;
    CK(c, cudaMallocFromPoolAsync(&cv->d_pixels, sizeof(j3dg_pixel) * n, pool, S(c)), "canvas");
    CK(c, cudaMallocFromPoolAsync((void**)&cv->d_image, sizeof(uint32_t) * n, pool, S(c)), "canvas");
    CK(c, cudaMallocFromPoolAsync((void**)&cv->d_background, sizeof(uint32_t) * n, pool, S(c)), "canvas");
    CK(c, cudaMallocFromPoolAsync(&cv->d_queue, kQueueBytesPerPixel * n + kQueueBytesFixed, pool, S(c)), "canvas");
    CK(c, cudaMallocFromPoolAsync((void**)&cv->d_work, j3dg::kCanvasWorkWords * sizeof(uint32_t), pool, S(c)),
       "canvas");
    CK(c, cudaMallocFromPoolAsync((void**)&cv->d_stamps, sizeof(uint32_t) * n, pool, S(c)), "canvas");
    CK(c, cudaMemsetAsync(cv->d_work, 0, j3dg::kCanvasWorkWords * sizeof(uint32_t), S(c)), "canvas");
    CK(c, cudaMemsetAsync(cv->d_stamps, 0, sizeof(uint32_t) * n, S(c)), "canvas");
    CK(c, cudaMemsetAsync(cv->d_image, 0, sizeof(uint32_t) * n, S(c)), "canvas");
    CK(c, cudaMemsetAsync(cv->d_background, 0, sizeof(uint32_t) * n, S(c)), "canvas");
    CK(c, j3dg::launch_init_pixels((j3dg_pixel*)cv->d_pixels, n, S(c)), "canvas");
  }
  // canvas.cpp:131-133: default camera and its projection
  j3dg_make_projection_matrix(&cv->camera, (int)w, (int)h, cv->projection);
  j3dg_invert_projection_matrix(cv->projection, cv->projection_inv);
  return J3DG_OK;
}

}  // namespace

namespace j3dg {

int ctx_fail(j3dg_ctx* c, int code, const std::string& msg) { return fail(c, code, msg); }

// Before work that writes the canvas: the context stream waits (on the
// device) for a download of the canvas still running on the copy stream.
void canvas_writable(j3dg_canvas* cv) {
  cv->stamp_seq = 0;  // a write without stamps: the next traced frame does not overlap
  if (!cv->copy_pending) return;
  cudaStreamWaitEvent(S(cv->ctx), (cudaEvent_t)cv->ev_copied, 0);
  cv->copy_pending = false;
}

// node-visit / triangle-test counters while counting is on, else null
unsigned long long* ctx_counters(j3dg_ctx* c) { return all(c)->ex.counting ? all(c)->ex.d_counters : nullptr; }

// The device instance table of one mesh with the identity transform.
int mesh_devinst(j3dg_ctx* c, const j3dg_mesh* mesh, const DevInst** out) {
  if (mesh->ctx != c) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "mesh of another context");
  j3dg_instance one;
  one.mesh = mesh;
  for (int i = 0; i < 16; ++i) one.cs[i] = (i % 5 == 0) ? 1.f : 0.f;
  one.db_id = 0;
  one.reserved = 0;
  return upload_instances(c, &one, 1, out);
}

// Plain closest hit of device rays against one mesh into device hits (async).
int ray_query_device(j3dg_ctx* c, const j3dg_mesh* mesh, const j3dg_ray* d_rays, uint32_t n, j3dg_hit* d_hits) {
  const DevInst* dinst = nullptr;
  if (int rc = mesh_devinst(c, mesh, &dinst)) return rc;
  CK(c, launch_rays(dinst, 1, false, (int)mesh->width, d_rays, n, d_hits, false, all(c)->ex.d_ray_counter, c->d_status,
                    nullptr, S(c)),
     "ray query");
  return J3DG_OK;
}

}  // namespace j3dg

extern "C" {

int j3dg_abi_version(void) { return J3DG_ABI_VERSION; }

const char* j3dg_status_string(int s) {
  switch (s) {
    case J3DG_OK: return "ok";
    case J3DG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case J3DG_ERR_CUDA: return "CUDA error";
    case J3DG_ERR_OUT_OF_MEMORY: return "out of device memory";
    case J3DG_ERR_NO_DEVICE: return "no CUDA device";
    case J3DG_ERR_DEVICE_STATUS: return "device status raised";
    case J3DG_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

const char* j3dg_last_error(const j3dg_ctx* c) { return c ? c->last_error.c_str() : "no context"; }

int j3dg_ctx_create(int device, j3dg_ctx** out) {
  if (!out) return J3DG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return J3DG_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return J3DG_ERR_INVALID_ARGUMENT;
  CtxAll* A = new (std::nothrow) CtxAll();
  if (!A) return J3DG_ERR_OUT_OF_MEMORY;
  j3dg_ctx* c = &A->ctx;
  c->device = device;
  c->h_inst = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete A;
    return J3DG_ERR_CUDA;
  }
  cudaStream_t st;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    delete A;
    return J3DG_ERR_CUDA;
  }
  c->stream = st;
  cudaStream_t cst;
  if (cudaStreamCreateWithFlags(&cst, cudaStreamNonBlocking) != cudaSuccess) {
    cudaStreamDestroy(st);
    delete A;
    return J3DG_ERR_CUDA;
  }
  c->copy_stream = cst;
  // the device's default stream-ordered pool (BVH build scratch, query
  // buffers) keeps up to kKeepReserved bytes mapped between calls: a build
  // then reuses the previous build's pages instead of mapping its scratch
  // (~20 GB for 28M triangles) again after every synchronisation released them
  {
    cudaMemPool_t dflt = nullptr;
    uint64_t keep_bytes = kKeepReserved;
    if (cudaDeviceGetDefaultMemPool(&dflt, device) == cudaSuccess)
      cudaMemPoolSetAttribute(dflt, cudaMemPoolAttrReleaseThreshold, &keep_bytes);
    cudaGetLastError();
  }
  cudaMemPoolProps props;
  memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  uint64_t keep = UINT64_MAX;
  bool ok = cudaMemPoolCreate(&A->ex.canvas_pool, &props) == cudaSuccess &&
            cudaMemPoolSetAttribute(A->ex.canvas_pool, cudaMemPoolAttrReleaseThreshold, &keep) == cudaSuccess &&
            cudaMalloc((void**)&c->d_status, sizeof(uint32_t)) == cudaSuccess &&
            cudaMemset(c->d_status, 0, sizeof(uint32_t)) == cudaSuccess &&
            cudaMalloc((void**)&A->ex.d_counters, 4 * sizeof(unsigned long long)) == cudaSuccess &&
            cudaMalloc((void**)&A->ex.d_ray_counter, sizeof(uint32_t)) == cudaSuccess &&
            cudaMalloc((void**)&A->ex.d_frame_ring, j3dg::kFrameDepth * sizeof(uint32_t)) == cudaSuccess &&
            cudaMemset(A->ex.d_frame_ring, 0, j3dg::kFrameDepth * sizeof(uint32_t)) == cudaSuccess &&
            cudaMemset(A->ex.d_counters, 0, 2 * sizeof(unsigned long long)) == cudaSuccess &&
            cudaEventCreate(&A->ex.ev0) == cudaSuccess && cudaEventCreate(&A->ex.ev1) == cudaSuccess;
  for (uint32_t i = 0; ok && i < kInstSlots; ++i) ok = cudaEventCreateWithFlags(&A->ex.slot_ev[i], cudaEventDisableTiming) == cudaSuccess;
  if (ok) {
    c->inst_cap = 16;
    ok = cudaMalloc(&c->d_inst, table_bytes(c->inst_cap) * kInstSlots) == cudaSuccess &&
         cudaMallocHost((void**)&A->h_slots, table_bytes(c->inst_cap) * kInstSlots) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    j3dg_ctx_destroy(c);
    return J3DG_ERR_CUDA;
  }
  // the no-allocation voxel grid's scratch: its address on this device, and
  // the module holding it loaded now rather than in the first call; a failed
  // lookup only disables j3dg_voxelize_noalloc (which then reports it)
  j3dg::voxel_scratch(&A->ex.noalloc_keys, &A->ex.noalloc_staging, A->ex.noalloc_error);
  *out = c;
  return J3DG_OK;
}

int j3dg_ctx_destroy(j3dg_ctx* c) {
  if (!c) return J3DG_ERR_INVALID_ARGUMENT;
  if (const uint32_t n = c->live.load())
    return fail(c, J3DG_ERR_INVALID_ARGUMENT,
                "context still used by " + std::to_string(n) + " object(s): destroy them first");
  CtxAll* A = all(c);
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(S(c));
  if (c->copy_stream) cudaStreamSynchronize((cudaStream_t)c->copy_stream);
  cudaFree(c->d_status);
  cudaFree(c->d_inst);
  cudaFree(A->ex.d_counters);
  cudaFree(A->ex.d_ray_counter);
  cudaFree(A->ex.d_frame_ring);
  if (A->h_slots) cudaFreeHost(A->h_slots);
  for (uint32_t i = 0; i < kInstSlots; ++i)
    if (A->ex.slot_ev[i]) cudaEventDestroy(A->ex.slot_ev[i]);
  if (A->ex.ev0) cudaEventDestroy(A->ex.ev0);
  if (A->ex.ev1) cudaEventDestroy(A->ex.ev1);
  // canvases still alive keep their memory until they are destroyed
  if (A->ex.canvas_pool) cudaMemPoolDestroy(A->ex.canvas_pool);
  if (c->stream) cudaStreamDestroy(S(c));
  if (c->copy_stream) cudaStreamDestroy((cudaStream_t)c->copy_stream);
  delete A;
  return J3DG_OK;
}

int j3dg_ctx_synchronize(j3dg_ctx* c) {
  if (!c) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  return check_status(c);
}

int j3dg_ctx_device_status(j3dg_ctx* c, uint32_t* status) {
  if (!c || !status) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  CK(c, cudaMemcpyAsync(status, c->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, S(c)), "status");
  CK(c, cudaStreamSynchronize(S(c)), "status");
  return J3DG_OK;
}

void* j3dg_ctx_stream(j3dg_ctx* c) { return c ? c->stream : nullptr; }

// Instrumentation: per-frame node-visit and triangle-test counters.
int j3dg_ctx_set_counting(j3dg_ctx* c, int enable) {
  if (!c) return J3DG_ERR_INVALID_ARGUMENT;
  all(c)->ex.counting = enable != 0;
  return J3DG_OK;
}

int j3dg_ctx_set_primary_mode(j3dg_ctx* c, int mode) {
  if (!c || mode < J3DG_PRIMARY_AUTO || mode > J3DG_PRIMARY_RASTER) return J3DG_ERR_INVALID_ARGUMENT;
  all(c)->ex.primary_mode = mode;
  return J3DG_OK;
}

int j3dg_canvas_last_primary(const j3dg_canvas* cv) { return cv ? cv->last_primary : J3DG_ERR_INVALID_ARGUMENT; }

int j3dg_ctx_set_batch_block(j3dg_ctx* c, int threads) {
  if (!c || (threads != 64 && threads != 128 && threads != 256)) return J3DG_ERR_INVALID_ARGUMENT;
  all(c)->ex.batch_threads = threads;
  return J3DG_OK;
}

int j3dg_ctx_memory(j3dg_ctx* c, uint64_t out[6]) {
  if (!c || !out) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  size_t fr = 0, tot = 0;
  CK(c, cudaMemGetInfo(&fr, &tot), "memory");
  out[0] = fr;
  out[1] = tot;
  unsigned long long v = 0;
  CK(c, cudaMemPoolGetAttribute(all(c)->ex.canvas_pool, cudaMemPoolAttrReservedMemCurrent, &v), "memory");
  out[2] = v;
  CK(c, cudaMemPoolGetAttribute(all(c)->ex.canvas_pool, cudaMemPoolAttrUsedMemCurrent, &v), "memory");
  out[3] = v;
  cudaMemPool_t dflt = nullptr;
  CK(c, cudaDeviceGetDefaultMemPool(&dflt, c->device), "memory");
  CK(c, cudaMemPoolGetAttribute(dflt, cudaMemPoolAttrReservedMemCurrent, &v), "memory");
  out[4] = v;
  CK(c, cudaMemPoolGetAttribute(dflt, cudaMemPoolAttrUsedMemCurrent, &v), "memory");
  out[5] = v;
  return J3DG_OK;
}

int j3dg_ctx_set_top_level(j3dg_ctx* c, int enable) {
  if (!c) return J3DG_ERR_INVALID_ARGUMENT;
  all(c)->ex.top_level = enable != 0;
  all(c)->ex.last_slot = -1;  // the next table is written afresh
  return J3DG_OK;
}

int j3dg_ctx_read_counters(j3dg_ctx* c, uint64_t out[2], int reset) {
  if (!c || !out) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  unsigned long long h[2];
  CK(c, cudaMemcpyAsync(h, all(c)->ex.d_counters, sizeof(h), cudaMemcpyDeviceToHost, S(c)), "counters");
  if (reset) CK(c, cudaMemsetAsync(all(c)->ex.d_counters, 0, sizeof(h), S(c)), "counters");
  CK(c, cudaStreamSynchronize(S(c)), "counters");
  out[0] = h[0];
  out[1] = h[1];
  return J3DG_OK;
}

// ------------------------------------------------------------------ mesh


namespace {

// One mesh build on stream `st` with its own timing events (the body of
// j3dg_mesh_build; j3dg_mesh_build_many runs several on their own streams).
// The device status word is checked by the caller.
int mesh_build_on(j3dg_ctx* c, const float* V, uint32_t nv, const uint32_t* T, uint32_t nt,
                  const j3dg_build_opts* opts, cudaStream_t st, cudaEvent_t ev0, cudaEvent_t ev1, j3dg_mesh** out,
                  std::string& msg) {
  *out = nullptr;
  if (!V || !T || nv == 0 || nt == 0) {
    msg = "mesh_build: empty mesh";
    return J3DG_ERR_INVALID_ARGUMENT;
  }
  if (nt >= J3DG_MAX_TRIANGLES) {
    msg = "mesh_build: more than 2^28 triangles";
    return J3DG_ERR_UNSUPPORTED;
  }
  uint32_t leaf = opts && opts->leaf_size ? opts->leaf_size : 2u;
  if (leaf < 1 || leaf > J3DG_MAX_LEAF) {
    msg = "mesh_build: leaf_size must be 1..8";
    return J3DG_ERR_INVALID_ARGUMENT;
  }
  j3dg_mesh* m = new (std::nothrow) j3dg_mesh();
  if (!m) return J3DG_ERR_OUT_OF_MEMORY;
  m->ctx = c;
  m->hold.attach(c);
  m->nv = nv;
  m->nt = nt;
  m->leaf_size = leaf;
  m->build_flags = opts ? opts->flags : 0u;
  {
    const uint32_t f = m->build_flags;
    if (f & ~(uint32_t)(J3DG_BUILD_LBVH | J3DG_BUILD_WIDTH2 | J3DG_BUILD_WIDTH8 | J3DG_BUILD_REBUILDABLE)) {
      delete m;
      msg = "mesh_build: unknown build flags";
      return J3DG_ERR_INVALID_ARGUMENT;
    }
    if ((f & J3DG_BUILD_WIDTH2) && (f & J3DG_BUILD_WIDTH8)) {
      delete m;
      msg = "mesh_build: two BVH widths requested";
      return J3DG_ERR_INVALID_ARGUMENT;
    }
    m->width = (f & J3DG_BUILD_WIDTH2) ? 2u : ((f & J3DG_BUILD_WIDTH8) ? 8u : 4u);
    if (m->width != 4 && (f & J3DG_BUILD_LBVH)) {
      delete m;
      msg = "mesh_build: the LBVH builder makes 4-wide trees only";
      return J3DG_ERR_UNSUPPORTED;
    }
  }
  float* dV = nullptr;
  bool ownV = false;
  int rc = J3DG_OK;
  cudaError_t e = cudaMalloc(&m->d_index, sizeof(uint32_t) * 3 * (size_t)nt);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m->d_index, T, sizeof(uint32_t) * 3 * (size_t)nt,
                        is_device_ptr(T) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    if (is_device_ptr(V)) {
      dV = const_cast<float*>(V);
    } else {
      ownV = true;
      e = cudaMalloc((void**)&dV, sizeof(float) * 3 * (size_t)nv);
      if (e == cudaSuccess) e = cudaMemcpyAsync(dV, V, sizeof(float) * 3 * (size_t)nv, cudaMemcpyHostToDevice, st);
    }
  }
  if (e == cudaSuccess) e = cudaEventRecord(ev0, st);
  if (e != cudaSuccess) {
    rc = e == cudaErrorMemoryAllocation ? J3DG_ERR_OUT_OF_MEMORY : J3DG_ERR_CUDA;
    msg = std::string("mesh_build upload: ") + cudaGetErrorString(e);
  } else {
    std::string err;
    rc = j3dg::build_bvh(m, dV, (const uint32_t*)m->d_index, st, c->d_status, ev1, err);  // ev1: the BVH is ready
    if (rc == J3DG_OK && (m->build_flags & J3DG_BUILD_REBUILDABLE)) {  // the vertices a batch rebuilds from
      cudaError_t ev = cudaMalloc(&m->d_verts, sizeof(float) * 3 * (size_t)nv);
      if (ev == cudaSuccess)
        ev = cudaMemcpyAsync(m->d_verts, dV, sizeof(float) * 3 * (size_t)nv, cudaMemcpyDeviceToDevice, st);
      if (ev != cudaSuccess) {
        rc = ev == cudaErrorMemoryAllocation ? J3DG_ERR_OUT_OF_MEMORY : J3DG_ERR_CUDA;
        err = std::string("keeping the vertices: ") + cudaGetErrorString(ev);
      }
    }
    if (rc == J3DG_OK) {
      cudaEventSynchronize(ev1);
      cudaEventElapsedTime(&m->build_ms, ev0, ev1);
    } else {
      msg = "mesh_build: " + err;
    }
  }
  if (ownV) cudaFree(dV);
  if (rc != J3DG_OK) {
    free_mesh_buffers(m);
    delete m;
    return rc;
  }
  *out = m;
  return J3DG_OK;
}

}  // namespace

int j3dg_mesh_build(j3dg_ctx* c, const float* V, uint32_t nv, const uint32_t* T, uint32_t nt,
                    const j3dg_build_opts* opts, j3dg_mesh** out) {
  if (!c || !out) return J3DG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  cudaSetDevice(c->device);
  CtxExtra& X = all(c)->ex;
  std::string msg;
  j3dg_mesh* m = nullptr;
  int rc = mesh_build_on(c, V, nv, T, nt, opts, S(c), X.ev0, X.ev1, &m, msg);
  if (rc != J3DG_OK) return fail(c, rc, msg);
  if ((rc = check_status(c)) != J3DG_OK) {
    j3dg_mesh_destroy(m);
    return rc;
  }
  *out = m;
  return J3DG_OK;
}

int j3dg_mesh_build_many(j3dg_ctx* c, uint32_t n, const j3dg_mesh_source* src, const j3dg_build_opts* opts,
                         uint32_t max_concurrent, j3dg_mesh** out) {
  if (!c || (n && (!src || !out))) return J3DG_ERR_INVALID_ARGUMENT;
  for (uint32_t i = 0; i < n; ++i) out[i] = nullptr;
  if (n == 0) return J3DG_OK;
  cudaSetDevice(c->device);
  // the work queued on the context stream before this call comes first
  CK(c, cudaStreamSynchronize(S(c)), "mesh_build_many");
  const uint32_t K = std::max(1u, std::min(n, max_concurrent ? max_concurrent : 8u));
  std::vector<int> rcs(n, J3DG_OK);
  std::vector<std::string> msgs(n);
  std::atomic<uint32_t> next{0};
  std::vector<std::thread> workers;
  for (uint32_t k = 0; k < K; ++k)
    workers.emplace_back([&, k] {
      cudaSetDevice(c->device);
      cudaStream_t st = nullptr;
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      const bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
                      cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
      for (uint32_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) {
        const j3dg_build_opts* o = opts ? opts + i : nullptr;
        if (!ok) {
          rcs[i] = J3DG_ERR_CUDA;
          msgs[i] = "mesh_build_many: could not create a build stream";
          continue;
        }
        rcs[i] = mesh_build_on(c, src[i].vertices, src[i].n_vertices, src[i].triangles, src[i].n_triangles, o, st,
                               e0, e1, &out[i], msgs[i]);
      }
      if (st) cudaStreamSynchronize(st);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      if (st) cudaStreamDestroy(st);
    });
  for (auto& t : workers) t.join();
  int rc = J3DG_OK;
  std::string msg;
  for (uint32_t i = 0; i < n && rc == J3DG_OK; ++i)
    if (rcs[i] != J3DG_OK) {
      rc = rcs[i];
      msg = "mesh " + std::to_string(i) + ": " + msgs[i];
    }
  if (rc == J3DG_OK) rc = check_status(c);
  else fail(c, rc, msg);
  if (rc != J3DG_OK)
    for (uint32_t i = 0; i < n; ++i)
      if (out[i]) {
        j3dg_mesh_destroy(out[i]);
        out[i] = nullptr;
      }
  return rc;
}

int j3dg_mesh_destroy(j3dg_mesh* m) {
  if (!m) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(m->ctx->device);
  cudaStreamSynchronize(S(m->ctx));
  all(m->ctx)->ex.last_slot = -1;  // the cached instance table may name this mesh
  free_mesh_buffers(m);
  delete m;
  return J3DG_OK;
}

int j3dg_mesh_get_nodes(const j3dg_mesh* m, void* dst, uint64_t bytes) {
  if (!m || (!dst && bytes)) return J3DG_ERR_INVALID_ARGUMENT;
  const uint64_t have = sizeof(float4) * J3DG_NODE_F4(m->width) * (uint64_t)m->n_nodes;
  if (bytes > have) return fail(m->ctx, J3DG_ERR_INVALID_ARGUMENT, "mesh_get_nodes: more bytes than the node array");
  if (!bytes) return J3DG_OK;
  cudaSetDevice(m->ctx->device);
  CK(m->ctx, cudaStreamSynchronize(S(m->ctx)), "mesh_get_nodes");
  CK(m->ctx, cudaMemcpy(dst, m->d_nodes, bytes, cudaMemcpyDeviceToHost), "mesh_get_nodes");
  return J3DG_OK;
}

int j3dg_mesh_get_info(const j3dg_mesh* m, j3dg_mesh_info* info) {
  if (!m || !info) return J3DG_ERR_INVALID_ARGUMENT;
  info->n_vertices = m->nv;
  info->n_triangles = m->nt;
  memcpy(info->min_bb, m->min_bb, sizeof(info->min_bb));
  memcpy(info->max_bb, m->max_bb, sizeof(info->max_bb));
  info->n_nodes = m->n_nodes;
  info->max_depth = m->max_depth;
  info->device_bytes = m->device_bytes;
  info->build_ms = m->build_ms;
  info->width = m->width;
  return J3DG_OK;
}

int j3dg_mesh_get_triangle_normals(const j3dg_mesh* m, float* normals) {
  if (!m || !normals) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = m->ctx;
  cudaSetDevice(c->device);
  std::vector<float> tmp(4 * (size_t)m->nt);
  CK(c, cudaMemcpyAsync(tmp.data(), m->d_normals, sizeof(float) * 4 * (size_t)m->nt, cudaMemcpyDeviceToHost, S(c)),
     "normals");
  CK(c, cudaStreamSynchronize(S(c)), "normals");
  for (size_t i = 0; i < m->nt; ++i)
    for (int k = 0; k < 3; ++k) normals[3 * i + k] = tmp[4 * i + k];
  return J3DG_OK;
}

static int upload_owned(j3dg_ctx* c, void** dst, const void* src, size_t bytes, const char* what) {
  cudaFree(*dst);
  *dst = nullptr;
  if (!src) return J3DG_OK;
  CK(c, cudaMalloc(dst, bytes), what);
  CK(c, cudaMemcpyAsync(*dst, src, bytes, is_device_ptr(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, S(c)),
     what);
  CK(c, cudaStreamSynchronize(S(c)), what);
  all(c)->ex.last_slot = -1;
  return J3DG_OK;
}

int j3dg_mesh_set_vertex_colors(j3dg_mesh* m, const float* colors) {
  if (!m) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(m->ctx->device);
  cudaStreamSynchronize(S(m->ctx));
  return upload_owned(m->ctx, &m->d_colors, colors, sizeof(float) * 3 * (size_t)m->nv, "vertex colors");
}

int j3dg_mesh_set_uv(j3dg_mesh* m, const float* uv) {
  if (!m) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(m->ctx->device);
  cudaStreamSynchronize(S(m->ctx));
  return upload_owned(m->ctx, &m->d_uv, uv, sizeof(float) * 6 * (size_t)m->nt, "uv");
}

int j3dg_mesh_set_texture(j3dg_mesh* m, const uint32_t* tex, uint32_t w, uint32_t h) {
  if (!m || (tex && (w == 0 || h == 0))) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(m->ctx->device);
  cudaStreamSynchronize(S(m->ctx));
  m->tex_w = tex ? w : 0;
  m->tex_h = tex ? h : 0;
  return upload_owned(m->ctx, &m->d_tex, tex, sizeof(uint32_t) * (size_t)w * h, "texture");
}

// ------------------------------------------------------------ ray batches

static int ray_query(j3dg_ctx* c, const j3dg_instance* objs, uint32_t n_obj, const j3dg_ray* rays, uint32_t n,
                     j3dg_hit* hits, bool any) {
  if (!c || (n && (!rays || !hits)) || (n_obj && !objs)) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  const DevInst* dinst = nullptr;
  bool top = false;
  int rc = upload_instances(c, objs, n_obj, &dinst, &top);
  if (rc) return rc;
  if (n == 0) return J3DG_OK;
  const bool rays_dev = is_device_ptr(rays), hits_dev = is_device_ptr(hits);
  j3dg_ray* dr = const_cast<j3dg_ray*>(rays);
  j3dg_hit* dh = hits;
  if (!rays_dev) {
    CK(c, cudaMallocAsync((void**)&dr, sizeof(j3dg_ray) * (size_t)n, S(c)), "rays");
    CK(c, cudaMemcpyAsync(dr, rays, sizeof(j3dg_ray) * (size_t)n, cudaMemcpyHostToDevice, S(c)), "rays");
  }
  if (!hits_dev) CK(c, cudaMallocAsync((void**)&dh, sizeof(j3dg_hit) * (size_t)n, S(c)), "hits");
  CK(c, j3dg::launch_rays(dinst, n_obj, top, n_obj ? (int)objs[0].mesh->width : 4, dr, n, dh, any,
                          all(c)->ex.d_ray_counter, c->d_status, j3dg::ctx_counters(c),
                          S(c)),
     "find");
  if (!hits_dev) {
    CK(c, cudaMemcpyAsync(hits, dh, sizeof(j3dg_hit) * (size_t)n, cudaMemcpyDeviceToHost, S(c)), "hits");
    cudaFreeAsync(dh, S(c));
  }
  if (!rays_dev) cudaFreeAsync(dr, S(c));
  return check_status(c);
}

int j3dg_find_closest(j3dg_ctx* c, const j3dg_instance* objs, uint32_t n_obj, const j3dg_ray* rays, uint32_t n,
                      j3dg_hit* hits) {
  return ray_query(c, objs, n_obj, rays, n, hits, false);
}

int j3dg_find_any(j3dg_ctx* c, const j3dg_instance* objs, uint32_t n_obj, const j3dg_ray* rays, uint32_t n,
                  j3dg_hit* hits) {
  return ray_query(c, objs, n_obj, rays, n, hits, true);
}

int j3dg_find_all(j3dg_ctx* c, const j3dg_mesh* mesh, const j3dg_ray* rays, uint32_t n, uint32_t cap, j3dg_hit* hits,
                  uint32_t* counts) {
  if (!c || !mesh || (n && (!rays || !counts || (cap && !hits)))) return J3DG_ERR_INVALID_ARGUMENT;
  if (mesh->ctx != c) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "find_all: mesh of another context");
  if (mesh->width != 4) return fail(c, J3DG_ERR_UNSUPPORTED, "find_all: needs a 4-wide BVH");
  cudaSetDevice(c->device);
  j3dg_instance one;
  one.mesh = mesh;
  for (int i = 0; i < 16; ++i) one.cs[i] = (i % 5 == 0) ? 1.f : 0.f;
  one.db_id = 0;
  one.reserved = 0;
  const DevInst* dinst = nullptr;
  if (int rc = upload_instances(c, &one, 1, &dinst)) return rc;
  if (n == 0) return J3DG_OK;
  const bool rays_dev = is_device_ptr(rays), hits_dev = !cap || is_device_ptr(hits), counts_dev = is_device_ptr(counts);
  j3dg_ray* dr = const_cast<j3dg_ray*>(rays);
  j3dg_hit* dh = hits;
  uint32_t* dc = counts;
  if (!rays_dev) {
    CK(c, cudaMallocAsync((void**)&dr, sizeof(j3dg_ray) * (size_t)n, S(c)), "find_all");
    CK(c, cudaMemcpyAsync(dr, rays, sizeof(j3dg_ray) * (size_t)n, cudaMemcpyHostToDevice, S(c)), "find_all");
  }
  if (!hits_dev) CK(c, cudaMallocAsync((void**)&dh, sizeof(j3dg_hit) * (size_t)n * cap, S(c)), "find_all");
  if (!counts_dev) CK(c, cudaMallocAsync((void**)&dc, sizeof(uint32_t) * (size_t)n, S(c)), "find_all");
  CK(c, j3dg::launch_find_all(dinst, dr, n, cap, dh, dc, c->d_status, S(c)), "find_all");
  if (!hits_dev) {
    CK(c, cudaMemcpyAsync(hits, dh, sizeof(j3dg_hit) * (size_t)n * cap, cudaMemcpyDeviceToHost, S(c)), "find_all");
    cudaFreeAsync(dh, S(c));
  }
  if (!counts_dev) {
    CK(c, cudaMemcpyAsync(counts, dc, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToHost, S(c)), "find_all");
    cudaFreeAsync(dc, S(c));
  }
  if (!rays_dev) cudaFreeAsync(dr, S(c));
  return check_status(c);
}

int j3dg_voxelize(j3dg_ctx* c, const j3dg_mesh* mesh, uint32_t max_dim, uint32_t dims[3], uint8_t* voxels,
                  uint64_t capacity) {
  if (!c || !mesh || !dims) return J3DG_ERR_INVALID_ARGUMENT;
  if (max_dim == 0 || max_dim > 1024) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "voxelize: max_dim must be 1..1024");
  if (mesh->ctx != c) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "voxelize: mesh of another context");
  if (mesh->width != 4) return fail(c, J3DG_ERR_UNSUPPORTED, "voxelize: needs a 4-wide BVH");
  cudaSetDevice(c->device);
  // vox.cpp:286-299
  const float* mn = mesh->min_bb;
  const float* mx = mesh->max_bb;
  int L = 0;
  if ((mx[1] - mn[1]) > (mx[L] - mn[L])) L = 1;
  if ((mx[2] - mn[2]) > (mx[L] - mn[L])) L = 2;
  j3dg::VoxParams V;
  memset(&V, 0, sizeof(V));
  for (int j = 0; j < 3; ++j) {
    V.dim[j] = (uint32_t)((float)max_dim * (mx[j] - mn[j]) / (mx[L] - mn[L]));
    if (V.dim[j] == 0) V.dim[j] = 1;
    dims[j] = V.dim[j];
    V.mn[j] = mn[j];
    V.mx[j] = mx[j];
  }
  const uint64_t total = (uint64_t)V.dim[0] * V.dim[1] * V.dim[2];
  if (!voxels) return J3DG_OK;
  if (capacity < total) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "voxelize: capacity below dims product");
  for (int d = 0; d < 3; ++d) V.rays[d] = V.dim[(d + 1) % 3] * V.dim[(d + 2) % 3];
  V.rays_total = V.rays[0] + V.rays[1] + V.rays[2];
  V.use_texture = mesh->d_uv && mesh->d_tex && mesh->tex_w && mesh->tex_h;
  V.use_colors = !V.use_texture && mesh->d_colors;
  j3dg_instance one;
  one.mesh = mesh;
  for (int i = 0; i < 16; ++i) one.cs[i] = (i % 5 == 0) ? 1.f : 0.f;
  one.db_id = 0;
  one.reserved = 0;
  const DevInst* dinst = nullptr;
  if (int rc = upload_instances(c, &one, 1, &dinst)) return rc;
  uint32_t* keys = nullptr;
  uint8_t* dout = voxels;
  const bool out_dev = is_device_ptr(voxels);
  CK(c, cudaMallocAsync((void**)&keys, sizeof(uint32_t) * total, S(c)), "voxelize");
  if (!out_dev) CK(c, cudaMallocAsync((void**)&dout, total, S(c)), "voxelize");
  CK(c, j3dg::launch_voxelize(dinst, V, keys, dout, c->d_status, S(c)), "voxelize");
  if (!out_dev) {
    CK(c, cudaMemcpyAsync(voxels, dout, total, cudaMemcpyDeviceToHost, S(c)), "voxelize");
    cudaFreeAsync(dout, S(c));
  }
  cudaFreeAsync(keys, S(c));
  return check_status(c);
}

// Voxel grid without device allocation: the scratch is the library's
// file-scope array (query.cu); the instance table uses the context's ring,
// which holds one object without growing.
int j3dg_voxelize_noalloc(j3dg_ctx* c, const j3dg_mesh* mesh, uint32_t max_dim, uint32_t dims[3], uint8_t* voxels,
                          uint64_t capacity) {
  if (!c || !mesh || !dims) return J3DG_ERR_INVALID_ARGUMENT;
  if (max_dim == 0 || max_dim > 1024) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "voxelize_noalloc: max_dim must be 1..1024");
  if (mesh->ctx != c) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "voxelize_noalloc: mesh of another context");
  if (mesh->width != 4) return fail(c, J3DG_ERR_UNSUPPORTED, "voxelize_noalloc: needs a 4-wide BVH");
  cudaSetDevice(c->device);
  const float* mn = mesh->min_bb;
  const float* mx = mesh->max_bb;
  int L = 0;
  if ((mx[1] - mn[1]) > (mx[L] - mn[L])) L = 1;
  if ((mx[2] - mn[2]) > (mx[L] - mn[L])) L = 2;
  j3dg::VoxParams V;
  memset(&V, 0, sizeof(V));
  for (int j = 0; j < 3; ++j) {
    V.dim[j] = (uint32_t)((float)max_dim * (mx[j] - mn[j]) / (mx[L] - mn[L]));
    if (V.dim[j] == 0) V.dim[j] = 1;
    dims[j] = V.dim[j];
    V.mn[j] = mn[j];
    V.mx[j] = mx[j];
  }
  const uint64_t total = (uint64_t)V.dim[0] * V.dim[1] * V.dim[2];
  if (total > J3DG_NOALLOC_MAX_VOXELS)
    return fail(c, J3DG_ERR_INVALID_ARGUMENT,
                "voxelize_noalloc: the grid needs " + std::to_string(total) + " voxels, the scratch holds " +
                    std::to_string(J3DG_NOALLOC_MAX_VOXELS) + " (use j3dg_voxelize or a smaller max_dim)");
  if (!voxels) return J3DG_OK;
  if (capacity < total) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "voxelize_noalloc: capacity below dims product");
  uint32_t* keys = all(c)->ex.noalloc_keys;
  uint8_t* staging = all(c)->ex.noalloc_staging;
  if (!keys) return fail(c, J3DG_ERR_CUDA, all(c)->ex.noalloc_error);
  for (int d = 0; d < 3; ++d) V.rays[d] = V.dim[(d + 1) % 3] * V.dim[(d + 2) % 3];
  V.rays_total = V.rays[0] + V.rays[1] + V.rays[2];
  V.use_texture = mesh->d_uv && mesh->d_tex && mesh->tex_w && mesh->tex_h;
  V.use_colors = !V.use_texture && mesh->d_colors;
  j3dg_instance one;
  one.mesh = mesh;
  for (int i = 0; i < 16; ++i) one.cs[i] = (i % 5 == 0) ? 1.f : 0.f;
  one.db_id = 0;
  one.reserved = 0;
  const DevInst* dinst = nullptr;
  if (int rc = upload_instances(c, &one, 1, &dinst)) return rc;
  const bool out_dev = is_device_ptr(voxels);
  CK(c, j3dg::launch_voxelize(dinst, V, keys, out_dev ? voxels : staging, c->d_status, S(c)), "voxelize_noalloc");
  if (!out_dev) CK(c, cudaMemcpyAsync(voxels, staging, total, cudaMemcpyDeviceToHost, S(c)), "voxelize_noalloc");
  return check_status(c);
}

// --------------------------------------------------------------- matcap

int j3dg_matcap_create(j3dg_ctx* c, const uint32_t* px, uint32_t w, uint32_t h, uint32_t cavity, j3dg_matcap** out) {
  if (!c || !px || !out || w == 0 || h == 0) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  j3dg_matcap* m = new (std::nothrow) j3dg_matcap();
  if (!m) return J3DG_ERR_OUT_OF_MEMORY;
  m->ctx = c;
  m->hold.attach(c);
  m->w = w;
  m->h = h;
  m->cavity = cavity;
  void* d = nullptr;
  int rc = upload_owned(c, &d, px, sizeof(uint32_t) * (size_t)w * h, "matcap");
  if (rc) {
    delete m;
    return rc;
  }
  m->d_pixels = (uint32_t*)d;
  *out = m;
  return J3DG_OK;
}

int j3dg_matcap_destroy(j3dg_matcap* m) {
  if (!m) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(m->ctx->device);
  cudaStreamSynchronize(S(m->ctx));
  cudaFree(m->d_pixels);
  delete m;
  return J3DG_OK;
}

// --------------------------------------------------------------- canvas

int j3dg_canvas_create(j3dg_ctx* c, uint32_t w, uint32_t h, j3dg_canvas** out) {
  if (!c || !out) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  j3dg_canvas* cv = new (std::nothrow) j3dg_canvas();
  if (!cv) return J3DG_ERR_OUT_OF_MEMORY;
  cv->ctx = c;
  cv->hold.attach(c);
  j3dg_make_default_camera(&cv->camera);
  memset(&cv->settings, 0, sizeof(cv->settings));
  int rc = canvas_alloc(cv, w, h);
  if (rc) {
    j3dg_canvas_destroy(cv);
    return rc;
  }
  *out = cv;
  return J3DG_OK;
}

int j3dg_canvas_destroy(j3dg_canvas* cv) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(cv->ctx->device);
  canvas_release(cv);  // stream-ordered: no wait on the host
  if (cv->ev_ready) cudaEventDestroy((cudaEvent_t)cv->ev_ready);
  if (cv->ev_copied) cudaEventDestroy((cudaEvent_t)cv->ev_copied);
  delete cv;
  return J3DG_OK;
}

int j3dg_canvas_resize(j3dg_canvas* cv, uint32_t w, uint32_t h) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(cv->ctx->device);
  j3dg_make_default_camera(&cv->camera);  // canvas.cpp:131
  return canvas_alloc(cv, w, h);
}

int j3dg_canvas_set_camera(j3dg_canvas* cv, const j3dg_camera* cam) {
  if (!cv || !cam) return J3DG_ERR_INVALID_ARGUMENT;
  cv->camera = *cam;
  j3dg_make_projection_matrix(&cv->camera, (int)cv->w, (int)cv->h, cv->projection);
  j3dg_invert_projection_matrix(cv->projection, cv->projection_inv);
  return J3DG_OK;
}

int j3dg_canvas_get_projection(const j3dg_canvas* cv, float* P, float* Pinv) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  if (P) memcpy(P, cv->projection, sizeof(cv->projection));
  if (Pinv) memcpy(Pinv, cv->projection_inv, sizeof(cv->projection_inv));
  return J3DG_OK;
}

int j3dg_canvas_set_background_color(j3dg_canvas* cv, uint32_t top, uint32_t bottom) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = cv->ctx;
  cudaSetDevice(c->device);
  std::vector<uint32_t> bg((size_t)cv->w * cv->h);
  j3dg_fill_background(bg.data(), cv->w, cv->h, top, bottom);
  if (bg.empty()) return J3DG_OK;
  CK(c, cudaMemcpyAsync(cv->d_background, bg.data(), sizeof(uint32_t) * bg.size(), cudaMemcpyHostToDevice, S(c)),
     "background");
  CK(c, cudaStreamSynchronize(S(c)), "background");
  return J3DG_OK;
}

int j3dg_canvas_update_settings(j3dg_canvas* cv, const j3dg_canvas_settings* s) {
  if (!cv || !s) return J3DG_ERR_INVALID_ARGUMENT;
  cv->settings = *s;
  return J3DG_OK;
}

static int scene_ok(j3dg_ctx* c, const j3dg_scene* s) {
  if (s && s->n_objects && !s->objects) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "scene with objects == NULL");
  return J3DG_OK;
}

int j3dg_canvas_update_canvas(j3dg_canvas* cv, int x0, int y0, int x1, int y1, const j3dg_scene* s) {
  if (!cv || !s) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = cv->ctx;
  if (int rc = scene_ok(c, s)) return rc;
  if (cv->w == 0 || cv->h == 0) return J3DG_OK;
  cudaSetDevice(c->device);
  j3dg::canvas_writable(cv);
  const DevInst* dinst = nullptr;
  bool top = false;
  if (int rc = upload_instances(c, s->objects, s->n_objects, &dinst, &top)) return rc;
  // canvas.cpp:681-698: clamp the rectangle
  const int w = (int)cv->w, h = (int)cv->h;
  auto clampv = [](int v, int hi) { return v < 0 ? 0 : (v >= hi ? hi - 1 : v); };
  x0 = clampv(x0, w);
  y0 = clampv(y0, h);
  x1 = clampv(x1, w);
  y1 = clampv(y1, h);
  FrameParams P;
  fill_frame(P, cv, s, dinst, nullptr);
  P.top = top ? 1u : 0u;
  next_frame_seq(P, cv);  // its counters; a rectangle writes no stamps and does not overlap
  P.x0 = x0;
  P.y0 = y0;
  P.x1 = x1;
  P.y1 = y1;
  P.shade_mode = 0;
  setup_raster(P, cv, s);
  CK(c, j3dg::launch_render(P, S(c)), "update_canvas");
  return J3DG_OK;
}

int j3dg_canvas_render_scene(j3dg_canvas* cv, const j3dg_scene* s) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = cv->ctx;
  if (int rc = scene_ok(c, s)) return rc;
  cudaSetDevice(c->device);
  j3dg::canvas_writable(cv);
  const size_t n = (size_t)cv->w * cv->h;
  CK(c, j3dg::launch_copy_u32(cv->d_image, cv->d_background, n, S(c)), "render_scene");
  if (!s) {
    CK(c, j3dg::launch_clear_ids((j3dg_pixel*)cv->d_pixels, n, S(c)), "render_scene");
    return J3DG_OK;
  }
  return j3dg_canvas_update_canvas(cv, 0, 0, (int)cv->w - 1, (int)cv->h - 1, s);
}

static int shade(j3dg_canvas* cv, const j3dg_pixel* G, const j3dg_matcap* m, int fill_background) {
  j3dg_ctx* c = cv->ctx;
  if (!m) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "canvas_to_image: no matcap");
  if (cv->w == 0 || cv->h == 0) return J3DG_OK;
  j3dg::canvas_writable(cv);
  FrameParams P;
  fill_frame(P, cv, nullptr, nullptr, m);
  CK(c, j3dg::launch_shade(P, G, shade_mode_of(cv->settings), fill_background, S(c)), "canvas_to_image");
  return J3DG_OK;
}

int j3dg_canvas_to_image(j3dg_canvas* cv, const j3dg_matcap* m) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(cv->ctx->device);
  return shade(cv, (const j3dg_pixel*)cv->d_pixels, m, 0);
}

int j3dg_canvas_to_image_from(j3dg_canvas* cv, const j3dg_pixel* px, const j3dg_matcap* m) {
  if (!cv || !px) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = cv->ctx;
  cudaSetDevice(c->device);
  if (is_device_ptr(px)) return shade(cv, px, m, 0);
  const size_t n = (size_t)cv->w * cv->h;
  j3dg_pixel* d = nullptr;
  CK(c, cudaMallocAsync((void**)&d, sizeof(j3dg_pixel) * n, S(c)), "canvas_to_image");
  CK(c, cudaMemcpyAsync(d, px, sizeof(j3dg_pixel) * n, cudaMemcpyHostToDevice, S(c)), "canvas_to_image");
  int rc = shade(cv, d, m, 0);
  cudaFreeAsync(d, S(c));
  return rc;
}

int j3dg_canvas_render_frame(j3dg_canvas* cv, const j3dg_scene* s, const j3dg_matcap* m) {
  if (!cv || !m) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = cv->ctx;
  if (int rc = scene_ok(c, s)) return rc;
  if (cv->w == 0 || cv->h == 0) return J3DG_OK;
  cudaSetDevice(c->device);
  const uint32_t prev_frame = cv->stamp_seq;  // every pixel carries it (0: unknown)
  CtxExtra& X = all(c)->ex;
  // the stream's last work is a traced frame (or a diagnostic asks for the wait)
  const bool after_frame = c->stream_ops == X.frame_ops || cv->expect_stamps;
  cv->expect_stamps = false;
  j3dg::canvas_writable(cv);
  const DevInst* dinst = nullptr;
  bool top = false;
  if (s)
    if (int rc = upload_instances(c, s->objects, s->n_objects, &dinst, &top)) return rc;
  const int mode = shade_mode_of(cv->settings);
  if (!s) {
    const size_t n = (size_t)cv->w * cv->h;
    CK(c, j3dg::launch_copy_u32(cv->d_image, cv->d_background, n, S(c)), "render_frame");
    CK(c, j3dg::launch_clear_ids((j3dg_pixel*)cv->d_pixels, n, S(c)), "render_frame");
    return J3DG_OK;
  }
  FrameParams P;
  fill_frame(P, cv, s, dinst, m);
  P.top = top ? 1u : 0u;
  setup_raster(P, cv, s);
  next_frame_seq(P, cv);
  // a traced frame in one kernel (plain shading) stamps its pixels and may
  // overlap the frame before it on the stream (with overlap on)
  const bool single = !P.raster && mode == 0 && X.frame_overlap;
  if (single) {
    P.stamps = cv->d_stamps;
    P.wait_seq = after_frame ? prev_frame : 0u;
  }
  if (mode == 0) {
    P.shade_mode = 1;  // one kernel: G-buffer, shadow, plain shading, background
    CK(c, j3dg::launch_render(P, S(c)), "render_frame");
  } else {
    P.shade_mode = 0;
    CK(c, j3dg::launch_render(P, S(c)), "render_frame");
    CK(c, j3dg::launch_shade(P, (const j3dg_pixel*)cv->d_pixels, mode, 1, S(c)), "render_frame");
  }
  cv->stamp_seq = single ? P.seq : 0u;
  X.frame_ops = single ? c->stream_ops : ~0ull;
  return J3DG_OK;
}

int j3dg_ctx_set_frame_overlap(j3dg_ctx* c, int enable) {
  if (!c) return J3DG_ERR_INVALID_ARGUMENT;
  all(c)->ex.frame_overlap = enable != 0;
  return J3DG_OK;
}

int j3dg_canvas_expect_frame(j3dg_canvas* cv, uint32_t seq) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  cv->stamp_seq = seq;
  cv->expect_stamps = true;
  return J3DG_OK;
}

// ------------------------------------------------------- learned frames

extern "C++" {
namespace j3dg {  // learned.cu
int learned_hits_device(j3dg_learned* l, const j3dg_ray* d_rays, uint32_t n, j3dg_hit* d_hits);
const j3dg_mesh* learned_mesh(const j3dg_learned* l);
j3dg_ctx* learned_ctx(const j3dg_learned* l);
}  // namespace j3dg
}

int j3dg_learned_render_frame(j3dg_learned* l, j3dg_canvas* cv, const j3dg_scene* s, const j3dg_matcap* m) {
  if (!l || !cv || !s || !m) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = cv->ctx;
  if (int rc = scene_ok(c, s)) return rc;
  if (j3dg::learned_ctx(l) != c || m->ctx != c) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "learned frame: objects of another context");
  if (s->n_objects != 1 || s->objects[0].mesh != j3dg::learned_mesh(l))
    return fail(c, J3DG_ERR_INVALID_ARGUMENT, "learned frame: the scene must hold the network's mesh as its only object");
  for (int i = 0; i < 16; ++i)
    if (s->objects[0].cs[i] != ((i % 5 == 0) ? 1.f : 0.f))
      return fail(c, J3DG_ERR_UNSUPPORTED, "learned frame: the network is trained in the mesh's space; its object "
                                          "transform must be the identity");
  if (cv->w == 0 || cv->h == 0) return J3DG_OK;
  cudaSetDevice(c->device);
  j3dg::canvas_writable(cv);
  const DevInst* dinst = nullptr;
  if (int rc = upload_instances(c, s->objects, 1, &dinst)) return rc;
  FrameParams P;
  fill_frame(P, cv, s, dinst, m);
  if (!raster_layout(P, cv, 1, 32, s->objects[0].mesh->nt))
    return fail(c, J3DG_ERR_INVALID_ARGUMENT, "learned frame: canvas scratch too small");
  cv->last_primary = J3DG_PRIMARY_TRACE;
  const int mode = shade_mode_of(cv->settings);
  P.shade_mode = mode == 0 ? 1 : 0;
  const size_t n = (size_t)cv->w * cv->h;
  if (n > 0xffffffffu) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "learned frame: canvas too large");
  // rays and hits: stream-ordered scratch from the context's canvas pool,
  // which keeps freed memory reserved (no device-wide synchronisation)
  char* scratch = nullptr;
  CK(c, cudaMallocFromPoolAsync((void**)&scratch, (sizeof(j3dg_ray) + sizeof(j3dg_hit)) * n, all(c)->ex.canvas_pool,
                                S(c)),
     "learned frame");
  j3dg_ray* rays = reinterpret_cast<j3dg_ray*>(scratch);
  j3dg_hit* hits = reinterpret_cast<j3dg_hit*>(scratch + sizeof(j3dg_ray) * n);
  int rc = J3DG_OK;
  cudaError_t e = j3dg::launch_primary_rays(P, rays, S(c));
  if (e == cudaSuccess) {
    rc = j3dg::learned_hits_device(l, rays, (uint32_t)n, hits);
    if (rc == J3DG_OK) e = j3dg::launch_frame_from_hits(P, hits, S(c));
    if (rc == J3DG_OK && e == cudaSuccess && mode != 0)
      e = j3dg::launch_shade(P, (const j3dg_pixel*)cv->d_pixels, mode, 1, S(c));
  }
  cudaFreeAsync(scratch, S(c));
  if (rc != J3DG_OK) return rc;
  CK(c, e, "learned frame");
  return J3DG_OK;
}

// ----------------------------------------------------------------- batches

namespace {

// Packed batch parameters: [FrameParams x n][offsets x (n+1), padded]
// [instance table of frame 0][table of frame 1]... (frames without objects
// take none); frame i's table holds caps[i] objects (table_bytes).
struct BatchLayout {
  size_t off_params = 0, off_offsets = 0, bytes = 0;
  std::vector<size_t> off_table;
  uint32_t n = 0;
  void set(uint32_t frames, const uint32_t* caps) {
    n = frames;
    off_params = 0;
    off_offsets = (sizeof(FrameParams) * n + 255) & ~size_t(255);
    size_t o = (off_offsets + sizeof(uint32_t) * (n + 1) + 255) & ~size_t(255);
    off_table.assign(n, 0);
    for (uint32_t i = 0; i < n; ++i) {
      off_table[i] = o;
      if (caps[i]) o += table_bytes(caps[i]);
    }
    bytes = o;
  }
};

int check_frames(j3dg_ctx* c, const j3dg_frame* f, uint32_t n, uint32_t& total_inst, uint32_t* width = nullptr) {
  total_inst = 0;
  uint32_t w = 0;
  for (uint32_t i = 0; i < n; ++i) {
    if (!f[i].canvas || !f[i].matcap) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "batch: frame without canvas or matcap");
    if (f[i].canvas->ctx != c || f[i].matcap->ctx != c) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "batch: object of another context");
    for (uint32_t j = 0; j < i; ++j)
      if (f[j].canvas == f[i].canvas) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "batch: a canvas appears twice");
    if (f[i].scene) {
      if (int rc = scene_ok(c, f[i].scene)) return rc;
      for (uint32_t k = 0; k < f[i].scene->n_objects; ++k) {
        if (!f[i].scene->objects[k].mesh || f[i].scene->objects[k].mesh->ctx != c)
          return fail(c, J3DG_ERR_INVALID_ARGUMENT, "batch: bad scene object");
        const uint32_t mw = f[i].scene->objects[k].mesh->width;
        if (w && mw != w) return fail(c, J3DG_ERR_UNSUPPORTED, "batch: the meshes of one batch must share a BVH width");
        w = mw;
      }
      total_inst += f[i].scene->n_objects;
    }
  }
  if (width) *width = w ? w : 4u;
  return J3DG_OK;
}

// Fills frame i of the host staging `h` for device base `d` (pointers
// inside point to `d`): its parameters and its instance table (sized for
// cap objects at creation). walk / fits: the frame's top level is worth
// walking (two or more objects) / fits the traversal stack.
void pack_frame(const j3dg_frame& f, uint32_t i, const BatchLayout& L, char* h, char* d, uint32_t cap, bool allow,
                bool& walk, bool& fits) {
  FrameParams* P = reinterpret_cast<FrameParams*>(h + L.off_params);
  const j3dg_scene* s = f.scene;
  const uint32_t ni = s ? s->n_objects : 0;
  const DevInst* dI = nullptr;
  walk = false;
  fits = true;
  if (ni) {
    std::vector<DevInst> t(ni);
    for (uint32_t j = 0; j < ni; ++j) t[j] = to_dev(s->objects[j]);
    dI = write_table(h + L.off_table[i], d + L.off_table[i], t.data(), s->objects, ni, cap, walk, &fits);
    walk = walk && allow;
  }
  fill_frame(P[i], f.canvas, s, dI, f.matcap);
  P[i].shade_mode = shade_mode_of(f.canvas->settings) == 0 ? 1 : 0;
}

// The launch walks top levels when some frame has two or more objects and
// every frame's top level fits the traversal stack (a frame with one object
// has a one-leaf top level, which the walk enters directly).
bool batch_top(const std::vector<char>& walk, const std::vector<char>& fits) {
  bool any = false, all = true;
  for (size_t i = 0; i < walk.size(); ++i) {
    any = any || walk[i];
    all = all && fits[i];
  }
  return any && all;
}

// Fills the whole staging; returns the total primary items of the frames.
uint32_t pack_frames(const j3dg_frame* f, uint32_t n, const BatchLayout& L, char* h, char* d, const uint32_t* cap,
                     bool allow, std::vector<char>& walk, std::vector<char>& fits, bool& top) {
  FrameParams* P = reinterpret_cast<FrameParams*>(h + L.off_params);
  uint32_t* off = reinterpret_cast<uint32_t*>(h + L.off_offsets);
  uint32_t items = 0;
  walk.assign(n, 0);
  fits.assign(n, 1);
  for (uint32_t i = 0; i < n; ++i) {
    bool w = false, ft = true;
    pack_frame(f[i], i, L, h, d, cap[i], allow, w, ft);
    walk[i] = w;
    fits[i] = ft;
    off[i] = items;
    items += f[i].canvas->w && f[i].canvas->h ? j3dg::primary_items(P[i]) : 0u;
  }
  off[n] = items;
  top = batch_top(walk, fits);
  for (uint32_t i = 0; i < n; ++i) P[i].top = top ? 1u : 0u;
  return items;
}

int enqueue_batch(j3dg_ctx* c, const j3dg_frame* f, uint32_t n, const BatchLayout& L, char* d, uint32_t items,
                  uint32_t* work, bool top, uint32_t width) {
  const FrameParams* dP = reinterpret_cast<const FrameParams*>(d + L.off_params);
  const uint32_t* dOff = reinterpret_cast<const uint32_t*>(d + L.off_offsets);
  CK(c, j3dg::launch_render_batch(dP, dOff, n, items, work, all(c)->ex.batch_threads, top, (int)width, S(c)),
     "batch");
  for (uint32_t i = 0; i < n; ++i) {
    const int mode = shade_mode_of(f[i].canvas->settings);
    if (mode != 0 && f[i].canvas->w && f[i].canvas->h) {
      FrameParams P;
      fill_frame(P, f[i].canvas, f[i].scene, nullptr, f[i].matcap);
      CK(c, j3dg::launch_shade(P, (const j3dg_pixel*)f[i].canvas->d_pixels, mode, 1, S(c)), "batch");
    }
  }
  return J3DG_OK;
}

}  // namespace

struct j3dg_batch {
  j3dg_ctx* ctx = nullptr;
  CtxHold hold;
  std::vector<j3dg_frame> frames;
  std::vector<std::vector<j3dg_instance>> objects;  // copies of each frame's objects
  std::vector<j3dg_scene> scenes;
  std::vector<uint32_t> caps;  // instance slots of each frame (its object count at creation)
  BatchLayout L;
  std::vector<char> walk, fits;  // per frame (pack_frame)
  bool top = false;              // the captured launch walks top levels
  uint32_t width = 4;            // the BVH width of every mesh of the batch
  char* h = nullptr;  // pinned staging
  char* d = nullptr;  // device copy
  uint32_t* work = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;
  // J3DG_BATCH_REBUILD: the meshes rebuilt ahead of the frames, by lane
  std::vector<j3dg::RebuildLane*> lanes;
  std::vector<std::vector<const j3dg_mesh*>> lane_meshes;
  std::vector<cudaStream_t> lane_streams;
  std::vector<cudaEvent_t> lane_events;  // [0]: the fork, then one join per lane
  cudaStream_t side = nullptr;           // captures the builds' loop bodies
};

int j3dg_render_batch(j3dg_ctx* c, const j3dg_frame* f, uint32_t n) {
  if (!c || (n && !f)) return J3DG_ERR_INVALID_ARGUMENT;
  if (n == 0) return J3DG_OK;
  cudaSetDevice(c->device);
  uint32_t total_inst = 0, width = 4;
  if (int rc = check_frames(c, f, n, total_inst, &width)) return rc;
  for (uint32_t i = 0; i < n; ++i) j3dg::canvas_writable(f[i].canvas);
  std::vector<uint32_t> caps(n);
  for (uint32_t i = 0; i < n; ++i) caps[i] = f[i].scene ? f[i].scene->n_objects : 0u;
  BatchLayout L;
  L.set(n, caps.data());
  char* d = nullptr;
  uint32_t* work = nullptr;
  std::vector<char> h(L.bytes);
  CK(c, cudaMallocAsync((void**)&d, L.bytes + 256, S(c)), "render_batch");
  work = reinterpret_cast<uint32_t*>(d + L.bytes);
  bool top = false;
  std::vector<char> walk, fits;
  const uint32_t items = pack_frames(f, n, L, h.data(), d, caps.data(), all(c)->ex.top_level, walk, fits, top);
  // pageable source: the copy is staged before the call returns
  CK(c, cudaMemcpyAsync(d, h.data(), L.bytes, cudaMemcpyHostToDevice, S(c)), "render_batch");
  int rc = enqueue_batch(c, f, n, L, d, items, work, top, width);
  cudaFreeAsync(d, S(c));
  return rc;
}

int j3dg_batch_create(j3dg_ctx* c, const j3dg_frame* f, uint32_t n, j3dg_batch** out) {
  return j3dg_batch_create2(c, f, n, 0u, out);
}

namespace {

// the distinct meshes of the frames' scenes, split into up to 8 lanes of
// about equal triangle counts (largest first, each to the lightest lane)
void rebuild_lanes(const j3dg_frame* f, uint32_t n, std::vector<std::vector<const j3dg_mesh*>>& lanes) {
  std::vector<const j3dg_mesh*> ms;
  for (uint32_t i = 0; i < n; ++i)
    if (f[i].scene)
      for (uint32_t k = 0; k < f[i].scene->n_objects; ++k) ms.push_back(f[i].scene->objects[k].mesh);
  std::sort(ms.begin(), ms.end());
  ms.erase(std::unique(ms.begin(), ms.end()), ms.end());
  std::stable_sort(ms.begin(), ms.end(), [](const j3dg_mesh* a, const j3dg_mesh* b) { return a->nt > b->nt; });
  const size_t K = std::min<size_t>(8, ms.size());
  lanes.assign(K, {});
  std::vector<uint64_t> load(K, 0);
  for (const j3dg_mesh* m : ms) {
    const size_t k = std::min_element(load.begin(), load.end()) - load.begin();
    lanes[k].push_back(m);
    load[k] += m->nt;
  }
}

}  // namespace

int j3dg_batch_create2(j3dg_ctx* c, const j3dg_frame* f, uint32_t n, uint32_t flags, j3dg_batch** out) {
  if (!c || !out || n == 0 || !f) return J3DG_ERR_INVALID_ARGUMENT;
  if (flags & ~J3DG_BATCH_REBUILD) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "batch_create2: unknown flags");
  *out = nullptr;
  cudaSetDevice(c->device);
  uint32_t total_inst = 0, width = 4;
  if (int rc = check_frames(c, f, n, total_inst, &width)) return rc;
  j3dg_batch* b = new (std::nothrow) j3dg_batch();
  if (!b) return J3DG_ERR_OUT_OF_MEMORY;
  b->ctx = c;
  b->width = width;
  b->hold.attach(c);
  b->frames.assign(f, f + n);
  b->objects.resize(n);
  b->scenes.resize(n);
  b->caps.assign(n, 0u);
  for (uint32_t i = 0; i < n; ++i) {
    b->caps[i] = f[i].scene ? f[i].scene->n_objects : 0u;
    if (f[i].scene) {
      b->scenes[i] = *f[i].scene;
      b->objects[i].assign(f[i].scene->objects, f[i].scene->objects + f[i].scene->n_objects);
      b->scenes[i].objects = b->objects[i].data();
      b->frames[i].scene = &b->scenes[i];
    }
  }
  b->L.set(n, b->caps.data());
  cudaError_t e = cudaMallocHost((void**)&b->h, b->L.bytes);
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->d, b->L.bytes + 256);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    j3dg_batch_destroy(b);
    return cuda_fail(c, e, "batch_create");
  }
  b->work = reinterpret_cast<uint32_t*>(b->d + b->L.bytes);
  int rc = J3DG_OK;
  if (flags & J3DG_BATCH_REBUILD) {
    rebuild_lanes(b->frames.data(), n, b->lane_meshes);
    for (const auto& lane : b->lane_meshes)
      for (const j3dg_mesh* m : lane)
        if (!m->d_verts && m->nt > m->leaf_size) {
          j3dg_batch_destroy(b);
          return fail(c, J3DG_ERR_UNSUPPORTED, "batch_create2: rebuilt meshes must be built with J3DG_BUILD_REBUILDABLE");
        }
    std::string err;
    for (const auto& lane : b->lane_meshes) {
      uint32_t nt_max = 2, nv_max = 3;
      bool ploc = false, lbvh = false;  // the builders the lane's meshes use
      for (const j3dg_mesh* m : lane) {
        nt_max = std::max(nt_max, m->nt);
        nv_max = std::max(nv_max, m->nv);
        if (m->nt > m->leaf_size) ((m->build_flags & J3DG_BUILD_LBVH) ? lbvh : ploc) = true;
      }
      j3dg::RebuildLane* L = nullptr;
      rc = j3dg::rebuild_lane_alloc(nt_max, nv_max, width, ploc || !lbvh, lbvh, S(c), &L, err);
      if (rc != J3DG_OK) {
        j3dg_batch_destroy(b);
        return fail(c, rc, "batch_create2: " + err);
      }
      b->lanes.push_back(L);
      cudaStream_t ls = nullptr;
      e = cudaStreamCreateWithFlags(&ls, cudaStreamNonBlocking);
      if (e == cudaSuccess) b->lane_streams.push_back(ls);
      cudaEvent_t ev = nullptr;
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      if (e == cudaSuccess) b->lane_events.push_back(ev);
      if (e != cudaSuccess) break;
    }
    cudaEvent_t fork = nullptr;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    if (e == cudaSuccess) b->lane_events.insert(b->lane_events.begin(), fork);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S(c));  // the scratch is allocated before the capture
    if (e != cudaSuccess) {
      j3dg_batch_destroy(b);
      return cuda_fail(c, e, "batch_create2");
    }
  }
  const uint32_t items =
      pack_frames(b->frames.data(), n, b->L, b->h, b->d, b->caps.data(), all(c)->ex.top_level, b->walk, b->fits, b->top);
  // capture: the rebuilds (forked lanes, joined before the frames), the
  // upload of the staged parameters, the launch and the shading passes
  cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  e = cudaStreamBeginCapture(S(c), mode);
  if (e == cudaSuccess && !b->lanes.empty()) {
    e = cudaEventRecord(b->lane_events[0], S(c));
    for (size_t k = 0; e == cudaSuccess && k < b->lanes.size(); ++k) {
      cudaStream_t ls = b->lane_streams[k];
      e = cudaStreamWaitEvent(ls, b->lane_events[0], 0);
      for (size_t i = 0; e == cudaSuccess && i < b->lane_meshes[k].size(); ++i)
        e = j3dg::rebuild_enqueue(b->lanes[k], b->lane_meshes[k][i], ls, b->side, c->d_status);
      if (e == cudaSuccess) e = cudaEventRecord(b->lane_events[k + 1], ls);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(S(c), b->lane_events[k + 1], 0);
    }
  }
  if (e == cudaSuccess) {
    e = cudaMemcpyAsync(b->d, b->h, b->L.bytes, cudaMemcpyHostToDevice, S(c));
    if (e == cudaSuccess) rc = enqueue_batch(c, b->frames.data(), n, b->L, b->d, items, b->work, b->top, b->width);
    cudaError_t e2 = cudaStreamEndCapture(S(c), &b->graph);
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaSuccess && rc == J3DG_OK) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (e != cudaSuccess || rc != J3DG_OK) {
    j3dg_batch_destroy(b);
    return rc != J3DG_OK ? rc : cuda_fail(c, e, "batch_create");
  }
  *out = b;
  return J3DG_OK;
}

int j3dg_batch_set_scene(j3dg_batch* b, uint32_t i, const j3dg_scene* s) {
  if (!b || i >= b->frames.size() || !s) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = b->ctx;
  if (int rc = scene_ok(c, s)) return rc;
  const uint32_t cap = b->caps[i];
  if (s->n_objects > cap) return fail(c, J3DG_ERR_INVALID_ARGUMENT, "batch_set_scene: more objects than at creation");
  for (uint32_t k = 0; k < s->n_objects; ++k) {
    if (!s->objects[k].mesh || s->objects[k].mesh->ctx != c)
      return fail(c, J3DG_ERR_INVALID_ARGUMENT, "batch_set_scene: bad scene object");
    if (s->objects[k].mesh->width != b->width)
      return fail(c, J3DG_ERR_UNSUPPORTED, "batch_set_scene: a mesh of another BVH width than the batch's");
  }
  cudaSetDevice(c->device);
  CK(c, cudaEventSynchronize(b->done), "batch_set_scene");  // the staging is read by the running launch
  const std::vector<j3dg_instance> old_objects = b->objects[i];
  const j3dg_scene old_scene = b->scenes[i];
  b->objects[i].assign(s->objects, s->objects + s->n_objects);
  b->scenes[i] = *s;
  b->scenes[i].objects = b->objects[i].data();
  // frame i keeps the instance slots it had at creation; the captured
  // launch keeps its top-level choice, so a scene that would change it is
  // refused (and the frame keeps its previous scene)
  j3dg_frame fr = b->frames[i];
  fr.scene = &b->scenes[i];
  const bool was_walk = b->walk[i], was_fits = b->fits[i];
  bool w = false, ft = true;
  pack_frame(fr, i, b->L, b->h, b->d, b->caps[i], all(c)->ex.top_level, w, ft);
  b->walk[i] = w;
  b->fits[i] = ft;
  if (batch_top(b->walk, b->fits) != b->top) {
    b->objects[i].assign(old_objects.begin(), old_objects.end());
    b->scenes[i] = old_scene;
    b->scenes[i].objects = b->objects[i].data();
    fr.scene = &b->scenes[i];
    pack_frame(fr, i, b->L, b->h, b->d, b->caps[i], all(c)->ex.top_level, w, ft);
    b->walk[i] = was_walk;
    b->fits[i] = was_fits;
    reinterpret_cast<FrameParams*>(b->h + b->L.off_params)[i].top = b->top ? 1u : 0u;
    return fail(c, J3DG_ERR_INVALID_ARGUMENT,
                "batch_set_scene: the new scene changes whether the batch walks top levels; create a new batch");
  }
  reinterpret_cast<FrameParams*>(b->h + b->L.off_params)[i].top = b->top ? 1u : 0u;
  return J3DG_OK;
}

int j3dg_batch_launch(j3dg_batch* b) {
  if (!b) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = b->ctx;
  cudaSetDevice(c->device);
  for (const auto& f : b->frames) j3dg::canvas_writable(f.canvas);
  CK(c, cudaGraphLaunch(b->exec, S(c)), "batch_launch");
  CK(c, cudaEventRecord(b->done, S(c)), "batch_launch");
  return J3DG_OK;
}

int j3dg_batch_destroy(j3dg_batch* b) {
  if (!b) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(S(b->ctx));
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (j3dg::RebuildLane* L : b->lanes) j3dg::rebuild_lane_free(L, S(b->ctx));
  cudaStreamSynchronize(S(b->ctx));
  for (cudaStream_t ls : b->lane_streams) cudaStreamDestroy(ls);
  for (cudaEvent_t ev : b->lane_events) cudaEventDestroy(ev);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->done) cudaEventDestroy(b->done);
  cudaFree(b->d);
  if (b->h) cudaFreeHost(b->h);
  delete b;
  return J3DG_OK;
}

int j3dg_canvas_get_pixels(j3dg_canvas* cv, j3dg_pixel* dst) {
  if (!cv || !dst) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(cv->ctx->device);
  return copy_out(cv->ctx, dst, cv->d_pixels, sizeof(j3dg_pixel) * (size_t)cv->w * cv->h);
}

int j3dg_canvas_get_image(j3dg_canvas* cv, uint32_t* dst) {
  if (!cv || !dst) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(cv->ctx->device);
  return copy_out(cv->ctx, dst, cv->d_image, sizeof(uint32_t) * (size_t)cv->w * cv->h);
}

int j3dg_canvas_download_async(j3dg_canvas* cv, j3dg_pixel* pixels, uint32_t* image) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = cv->ctx;
  cudaSetDevice(c->device);
  cudaStream_t cs = (cudaStream_t)c->copy_stream;
  if (!cv->ev_ready) {
    CK(c, cudaEventCreateWithFlags((cudaEvent_t*)&cv->ev_ready, cudaEventDisableTiming), "download_async");
    CK(c, cudaEventCreateWithFlags((cudaEvent_t*)&cv->ev_copied, cudaEventDisableTiming), "download_async");
  }
  const size_t n = (size_t)cv->w * cv->h;
  // an event record writes nothing: the stream's last work stays what it
  // was, so the next traced frame may still overlap the previous one
  CK(c, cudaEventRecord((cudaEvent_t)cv->ev_ready, (cudaStream_t)c->stream), "download_async");
  CK(c, cudaStreamWaitEvent(cs, (cudaEvent_t)cv->ev_ready, 0), "download_async");
  if (pixels && n)
    CK(c, cudaMemcpyAsync(pixels, cv->d_pixels, sizeof(j3dg_pixel) * n,
                          is_device_ptr(pixels) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, cs),
       "download_async");
  if (image && n)
    CK(c, cudaMemcpyAsync(image, cv->d_image, sizeof(uint32_t) * n,
                          is_device_ptr(image) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, cs),
       "download_async");
  CK(c, cudaEventRecord((cudaEvent_t)cv->ev_copied, cs), "download_async");
  cv->copy_pending = true;
  return J3DG_OK;
}

int j3dg_canvas_download_wait(j3dg_canvas* cv) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  if (!cv->ev_copied) return J3DG_OK;
  cudaSetDevice(cv->ctx->device);
  CK(cv->ctx, cudaEventSynchronize((cudaEvent_t)cv->ev_copied), "download_wait");
  cv->copy_pending = false;  // the copy has ended: the next write need not wait for it on the device
  return J3DG_OK;
}

int j3dg_canvas_set_pixels(j3dg_canvas* cv, const j3dg_pixel* src) {
  if (!cv || !src) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = cv->ctx;
  cudaSetDevice(c->device);
  j3dg::canvas_writable(cv);
  CK(c, cudaMemcpyAsync(cv->d_pixels, src, sizeof(j3dg_pixel) * (size_t)cv->w * cv->h,
                        is_device_ptr(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, S(c)),
     "set_pixels");
  CK(c, cudaStreamSynchronize(S(c)), "set_pixels");
  return J3DG_OK;
}

int j3dg_canvas_count_hits(j3dg_canvas* cv, uint64_t* hits, uint64_t* shadowed) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = cv->ctx;
  cudaSetDevice(c->device);
  unsigned long long* d = all(c)->ex.d_counters + 2;
  unsigned long long h[2] = {0, 0};
  CK(c, j3dg::launch_count_hits((const j3dg_pixel*)cv->d_pixels, (size_t)cv->w * cv->h, d, S(c)), "count_hits");
  CK(c, cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, S(c)), "count_hits");
  CK(c, cudaStreamSynchronize(S(c)), "count_hits");
  if (hits) *hits = h[0];
  if (shadowed) *shadowed = h[1];
  return J3DG_OK;
}

int j3dg_canvas_device_buffers(j3dg_canvas* cv, j3dg_pixel** px, uint32_t** im, uint32_t** bg) {
  if (!cv) return J3DG_ERR_INVALID_ARGUMENT;
  if (px) *px = (j3dg_pixel*)cv->d_pixels;
  if (im) *im = cv->d_image;
  if (bg) *bg = cv->d_background;
  return J3DG_OK;
}

}  // extern "C"
