// render.cu -- per-frame kernels: the ray-cast frame (primary rays, closest
// hit, G-buffer record, shadow rays, plain matcap shading), the
// neighbour-reading shading modes, and batched ray queries.
//
// A frame is one persistent kernel, k_frame: it replaces the per-pixel body
// of canvas::update_canvas (canvas.cpp:765-857) and, in plain mode, the
// background copy of canvas::render_scene (canvas.cpp:893-898) and
// canvas_to_image's plain shading (canvas.cpp:650-669).
// k_shade replaces canvas_to_image's edges, wireframe and one-bit modes
// (canvas.cpp:449-649), which read the right and upper neighbours.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "device_common.cuh"
#include "render.cuh"

// This file is compiled once per BVH width (2, 4, 8): J3DG_W selects the
// width its tracing kernels walk, and everything in it lives in namespace
// j3dg::w<J3DG_W>; render_dispatch.cu calls the variant a frame's meshes
// need (the width-independent launchers of the w4 build).
#ifndef J3DG_W
#define J3DG_W 4
#endif
#if J3DG_W == 2
#define J3DG_WNS w2
#elif J3DG_W == 4
#define J3DG_WNS w4
#elif J3DG_W == 8
#define J3DG_WNS w8
#else
#error "J3DG_W must be 2, 4 or 8"
#endif

namespace j3dg {
namespace J3DG_WNS {
static const int kWidth = J3DG_W;

// ------------------------------------------------------------ shading ----

__device__ __forceinline__ uint32_t tex_index(float f, uint32_t size) {
  if (!(f >= 0.f)) f = 0.f;
  float mx = (float)(size - 1);
  if (f > mx) f = mx;
  return (uint32_t)f;
}

// canvas.cpp:320-328
__device__ __forceinline__ uint32_t get_U(float u, uint32_t W) {
  return tex_index(floorf(fa(0.5f, fm(fm(fa(u, 1.f), (float)(W - 1)), 0.5f))), W);
}
__device__ __forceinline__ uint32_t get_V(float v, uint32_t H) {
  return tex_index(floorf(fa(0.5f, fm(fm(fa(-v, 1.f), (float)(H - 1)), 0.5f))), H);
}

// canvas.cpp:330-344
__device__ __forceinline__ uint32_t get_color(const uint32_t* __restrict__ mc, uint32_t mw, uint32_t U, uint32_t V,
                                              uint32_t shadow) {
  uint32_t clr = __ldg(mc + (size_t)V * mw + U);
  if (shadow) {
    uint32_t r = clr & 0xffu, g = (clr >> 8) & 0xffu, b = (clr >> 16) & 0xffu;
    clr = 0xff000000u | ((b >> 2) << 16) | ((g >> 2) << 8) | (r >> 2);
  }
  return clr;
}

// canvas.cpp:346-389 (acosf: CUDA's, within 1 LSB of the host's after rounding)
__device__ __forceinline__ uint32_t get_angle_color(float angle, const FrameParams& P, float u, float v,
                                                    uint32_t mark) {
  uint32_t clr = get_color(P.matcap, P.mw, get_U(u, P.mw), get_V(v, P.mh), mark);
  if (fabsf(angle) <= 1.f) {
    uint32_t r = clr & 0xffu, g = (clr >> 8) & 0xffu, b = (clr >> 16) & 0xffu;
    const float hp = 1.57079632679489f;
    float scale = __fdiv_rn(fs(hp, fabsf(fs(acosf(angle), hp))), hp);
    scale = __fsqrt_rn(fs(1.f, scale));
    uint32_t c = P.cavity;
    uint32_t r2 = c & 0xffu, g2 = (c >> 8) & 0xffu, b2 = (c >> 16) & 0xffu;
    float f = angle > 0.f ? 1.2f : 0.5f;
    float om = fs(1.f, scale);
    r = (uint32_t)fa(fm((float)r, om), fm(fm((float)r2, scale), f));
    g = (uint32_t)fa(fm((float)g, om), fm(fm((float)g2, scale), f));
    b = (uint32_t)fa(fm((float)b, om), fm(fm((float)b2, scale), f));
    r = r > 255u ? 255u : r;
    g = g > 255u ? 255u : g;
    b = b > 255u ? 255u : b;
    clr = 0xff000000u | (b << 16) | (g << 8) | r;
  }
  return clr;
}

// canvas.cpp:402-441 (_get_color)
__device__ __forceinline__ uint32_t pixel_color(const FrameParams& P, uint32_t mark, uint32_t pr, uint32_t pg,
                                                uint32_t pb, float u, float v) {
  if (mark & 2u) {
    if (P.shading) {
      float nz = __fsqrt_rn(fs(fs(1.f, fm(u, u)), fm(v, v)));
      float d = fa(fa(fa(fm(u, 0.f), fm(v, 0.f)), fm(nz, 1.f)), fm(0.f, 0.f));
      d = d < 0.f ? 0.f : (d > 1.f ? 1.f : d);
      float dif = fm(d, (mark & 1u) ? 0.3f : 1.f);
      return 0xff000000u | ((uint32_t)fm((float)pb, dif) << 16) | ((uint32_t)fm((float)pg, dif) << 8) |
             (uint32_t)fm((float)pr, dif);
    }
    if (mark & 1u) return 0xff000000u | ((pb >> 2) << 16) | ((pg >> 2) << 8) | (pr >> 2);
    return 0xff000000u | (pb << 16) | (pg << 8) | pr;
  }
  return get_color(P.matcap, P.mw, get_U(u, P.mw), get_V(v, P.mh), mark);
}

// ------------------------------------------------------------- render ----

// Pixel of work item `idx`: 8x4 tiles in row-major tile order over the
// rectangle, so the 32 rays of a warp's refill come from one tile.
__device__ __forceinline__ bool item_pixel(const FrameParams& P, uint32_t idx, int& x, int& y) {
  const uint32_t rw = (uint32_t)(P.x1 - P.x0 + 1);
  const uint32_t tiles_x = (rw + 7u) >> 3;
  const uint32_t tile = idx >> 5, within = idx & 31u;
  x = P.x0 + (int)((tile % tiles_x) * 8u + (within & 7u));
  y = P.y0 + (int)((tile / tiles_x) * 4u + (within >> 3));
  return x <= P.x1 && y <= P.y1;
}

__device__ __forceinline__ void write_miss(const FrameParams& P, size_t pix) {
  // canvas.cpp:859-866 (other fields keep their previous values)
  j3dg_pixel* rec = P.gbuf + pix;
  rec->db_id = 0u;
  rec->object_id = 0xffffffffu;
  rec->u = 0.f;
  rec->v = 0.f;
  rec->depth = FLT_MAX;
  if (P.shade_mode == 1) P.im[pix] = P.background ? __ldg(P.background + pix) : P.im[pix];
}

// ------------------------------------------- overlapped frames ----
//
// The kernel of a canvas's frame is launched as a programmatic dependent of
// the previous kernel on the stream, so it starts while that kernel's last
// rays finish (a frame's tail otherwise leaves most of the GPU idle).
//
// Hand-over: each warp, once the frame's items are all taken, lets the next
// frame start (griddepcontrol.launch_dependents) if the frame kFrameDepth - 1
// launches before this one has released its ring entry; nothing waits
// there, so at most kFrameDepth frames are in flight. A frame's last warp to
// finish zeroes the frame's counter slot, waits until the kernel before it
// has completed (griddepcontrol.wait) and then releases the frame's ring
// entry: a frame completes only after every frame before it, and a released
// entry means every frame up to it has completed. A warp that never handed
// over waits likewise before it exits (its block's exit then counts as the
// hand-over). A canvas's frames use counter slots seq % kFrameDepth, so a
// slot's previous user has completed before the slot is used again.
//
// Pixel order: the previous frame stores its number into the pixel's stamp
// with release order after its last write of the pixel, and this frame,
// before its first write, waits (acquire) until the pixel carries that
// number. The wait is bounded (half a second by the global timer, and an
// iteration cap): when it runs out it raises J3DG_DEV_WAIT_TIMEOUT and the
// frame stops waiting.
static const uint64_t kAwaitNs = 500000000ull;
static const uint32_t kAwaitSpins = 1u << 26;

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void await_pixel(const FrameParams& P, size_t pix) {
  if (P.wait_seq == 0u) return;
  const uint32_t* a = P.stamps + pix;
  if (ld_acquire(a) == P.wait_seq) return;
  const uint64_t t0 = global_ns();
  for (uint32_t k = 0; k < kAwaitSpins; ++k) {
    if (*reinterpret_cast<volatile const uint32_t*>(P.status) & J3DG_DEV_WAIT_TIMEOUT) return;  // one ran out
    __nanosleep(256);
    if (ld_acquire(a) == P.wait_seq) return;
    if (global_ns() - t0 > kAwaitNs) break;
  }
  atomicOr(P.status, J3DG_DEV_WAIT_TIMEOUT);
}

__device__ __forceinline__ void stamp_pixel(const FrameParams& P, size_t pix) {
  if (P.stamps) asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(P.stamps + pix), "r"(P.seq) : "memory");
}

// warp-uniform: the next frame may start (the frame kFrameDepth - 1
// launches before this one has released its ring entry)
__device__ __forceinline__ bool handover_allowed(const FrameParams& P) {
  if (!P.ring) return false;  // no ring: the block's exit hands over
  uint32_t rel = 0;
  if ((threadIdx.x & 31u) == 0) rel = ld_acquire(P.ring + ((P.launch + 1u) % kFrameDepth));
  rel = __shfl_sync(0xffffffffu, rel, 0);
  return rel + (kFrameDepth - 1u) >= P.launch;
}

// the frame's end for one warp (all lanes): the last warp zeroes the
// frame's counter slot, waits for the kernel before it and releases the
// frame's ring entry
__device__ __forceinline__ void frame_exit(const FrameParams& P, bool handed_over) {
  if (!handed_over) asm volatile("griddepcontrol.wait;" ::: "memory");
  if ((threadIdx.x & 31u) == 0) {
    const uint32_t slot = P.seq % kFrameDepth;
    uint32_t* const done = P.work + 4 + kFrameDepth + slot;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    if (atomicAdd(done, 1u) == warps - 1u) {
      atomicExch(P.work + 4 + slot, 0u);
      atomicExch(done, 0u);
      asm volatile("griddepcontrol.wait;" ::: "memory");
      if (P.ring)
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(P.ring + P.launch % kFrameDepth), "r"(P.launch)
                     : "memory");
    }
  }
}

// A frame in one persistent kernel: each lane runs primary ray -> (shadow ray)
// -> next pixel, refilled from the tile-ordered pixel list by warp-aggregated
// atomics (Aila and Laine 2009 dynamic fetch), so shadow rays overlap other
// lanes' primary rays and the frame has a single tail.
//   primary (canvas.cpp:765-834): G-buffer record, texture / vertex colour;
//   shadow  (canvas.cpp:836-857): any hit towards the light marks the pixel;
//   plain shading (canvas.cpp:650-669) when shade_mode == 1, misses get the
//   background (canvas.cpp:893-898).
#ifndef J3DG_TRACE_THREADS
#define J3DG_TRACE_THREADS 128
#endif
// blocks per SM the frame kernels are compiled for: 6 x 128 threads leave
// 85 registers a thread, which the step's working set fits without spills
// once the state read only at a pixel's start and finish is in shared
// memory (J3DG_COLD_SMEM); latency-bound traversal gains from the extra warps
#ifndef J3DG_TRACE_MINBLOCKS
#define J3DG_TRACE_MINBLOCKS 6
#endif
// A frame (or batch) of fewer primary items than J3DG_THROUGHPUT_ITEMS runs
// the latency build instead: 5 blocks per SM with the pixel state in
// registers. Measured on single frames: below about one 1920x1080 frame the
// extra warps of the throughput build lengthen the frame (a 512x512 frame
// of the 28M-triangle torus 0.80 -> 0.89 ms); from there on they shorten it.
#ifndef J3DG_LATENCY_MINBLOCKS
#define J3DG_LATENCY_MINBLOCKS 5
#endif
#ifndef J3DG_THROUGHPUT_ITEMS
#define J3DG_THROUGHPUT_ITEMS 2000000u
#endif
#ifndef J3DG_TRACE_ITERS
#define J3DG_TRACE_ITERS 16
#endif
// idle lanes that make a warp stop tracing and fetch new pixels (16: with
// overlapped frames and in batches; 12 was best for frames run one by one,
// by 0.6 %)
#ifndef J3DG_REFILL_AT
#define J3DG_REFILL_AT 16
#endif
// 1: a lane whose ray finished parks until the warp leaves the tracing loop,
// and the parked lanes run the finish code (hit record, shadow ray setup,
// shading) together there, instead of the whole warp running that long
// branch for one lane in most tracing steps
#ifndef J3DG_DEFER_FINISH
#define J3DG_DEFER_FINISH 1
#endif
static const int kTraceThreads = J3DG_TRACE_THREADS;
static const int kIters = J3DG_TRACE_ITERS;
// k_frame runs two warps per block, with the warps per SM of the builds
// above: when a frame's last rays keep a few warps busy, every block that is
// done frees its slot for the canvas's next frame (overlapped frames, below;
// 32 / 64 / 128 threads measured 0.610 / 0.591 / 0.594 ms per headline frame)
#ifndef J3DG_FRAME_THREADS
#define J3DG_FRAME_THREADS 64
#endif
static const int kFrameThreads = J3DG_FRAME_THREADS;
static const int kFrameBlocksT = J3DG_TRACE_MINBLOCKS * 128 / kFrameThreads;
static const int kFrameBlocksL = J3DG_LATENCY_MINBLOCKS * 128 / kFrameThreads;

// Pixel and colour state of a lane: read only at a pixel's start and
// finish. The throughput build keeps it in a per-block shared array
// (J3DG_COLD_SMEM bit 4), the latency build in registers.
struct PixState {
  size_t pix;
  uint32_t w0, frame;
  float su, sv;
};

template <bool kShared, int N>
__device__ __forceinline__ PixState& pix_state(PixState& local) {
  if constexpr (kShared) {
    __shared__ PixState s[N];
    return s[threadIdx.x];
  } else {
    return local;
  }
}

__device__ __forceinline__ uint32_t primary_count(const FrameParams& P) {
  const uint32_t rw = (uint32_t)(P.x1 - P.x0 + 1), rh = (uint32_t)(P.y1 - P.y0 + 1);
  return ((rw + 7u) >> 3) * ((rh + 3u) >> 2) * 32u;
}

// world ray of pixel (x, y): canvas.cpp:700-701, 773-782
__device__ __forceinline__ void primary_ray(const FrameParams& P, int x, int y, float4& o, float4& d) {
  o = mat_vec(P.cs, 0.f, 0.f, 0.f, 1.f);
  const float sx = fs(fm(2.f, __fdiv_rn(fa((float)x, 0.5f), (float)P.w)), 1.f);
  const float sy = fs(fm(2.f, __fdiv_rn(fa((float)y, 0.5f), (float)P.h)), 1.f);
  d = mat_vec(P.pinv, sx, sy, P.near_plane, 1.f);
  d = mat_vec(P.cs, d.x, d.y, d.z, 0.f);
}

__device__ __forceinline__ float primary_t_near(const FrameParams& P) { return __fdiv_rn(P.diagonal, 100.f); }

template <class Tracer>
__device__ __forceinline__ void primary_begin(const FrameParams& P, Tracer& T, int x, int y) {
  float4 o, d;
  primary_ray(P, x, y, o, d);
  T.begin(P.inst, P.n_inst, o.x, o.y, o.z, d.x, d.y, d.z, primary_t_near(P), FLT_MAX, false);
}


// canvas.cpp:836-838: the point light, three diagonals beyond the pivot
__device__ __forceinline__ float4 light_position(const FrameParams& P) {
  const float ld = fm(P.diagonal, 3.f);
  return mat_vec(P.cs, fa(P.pivot[0], ld), fa(P.pivot[1], ld), fa(P.pivot[2], ld), 1.f);
}

// Writes the hit record; returns true and sets up the shadow ray in T when
// one is needed. w0 / su / sv keep what the final colour needs.
template <class Tracer>
__device__ __forceinline__ bool primary_finish(const FrameParams& P, Tracer& T, size_t pix, uint32_t& w0, float& su,
                                               float& sv) {
  await_pixel(P, pix);
  const auto b = T.b;
  if (!b.found) {
    write_miss(P, pix);
    return false;
  }
  j3dg_pixel* rec = P.gbuf + pix;
  const DevInst& I = P.inst[b.inst()];
  // canvas.cpp:788-801
  const float4 N = __ldg(I.normals + b.tri());
  float4 n = mat_vec(P.cs_inv, N.x, N.y, N.z, 0.f);
  n = mat_vec(I.cs, n.x, n.y, n.z, n.w);
  uint32_t mark = 0, pr = 0, pg = 0, pb = 0;
  bool rgb = false;
  const float wgt = fs(fs(1.f, b.u()), b.v());
  if (P.textured && I.uv != nullptr && I.tex != nullptr) {
    // canvas.cpp:803-820
    const float* uv = I.uv + 6 * (size_t)b.tri();
    float c0 = fa(fa(fm(wgt, uv[0]), fm(b.u(), uv[2])), fm(b.v(), uv[4]));
    float c1 = fa(fa(fm(wgt, uv[1]), fm(b.u(), uv[3])), fm(b.v(), uv[5]));
    c0 = fmaxf(fminf(c0, 1.f), 0.f);
    c1 = fmaxf(fminf(c1, 1.f), 0.f);
    const int tw = (int)I.tex_w, th = (int)I.tex_h;
    int tx = (int)fm(c0, (float)tw), ty = (int)fm(c1, (float)th);
    tx = tx < 0 ? 0 : tx >= tw ? tw - 1 : tx;
    ty = ty < 0 ? 0 : ty >= th ? th - 1 : ty;
    const uint32_t c = __ldg(I.tex + (size_t)ty * I.tex_w + tx);
    pr = c & 0xffu;
    pg = (c >> 8) & 0xffu;
    pb = (c >> 16) & 0xffu;
    mark |= 2u;
    rgb = true;
  } else if (P.vertexcolors && I.colors != nullptr) {
    // canvas.cpp:821-834
    const uint32_t* Ti = I.index + 3 * (size_t)b.tri();
    const float* C0 = I.colors + 3 * (size_t)Ti[0];
    const float* C1 = I.colors + 3 * (size_t)Ti[1];
    const float* C2 = I.colors + 3 * (size_t)Ti[2];
    float c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) c[k] = fa(fa(fm(C0[k], wgt), fm(b.u(), C1[k])), fm(b.v(), C2[k]));
    pr = (uint8_t)fm(c[0], 255.f);
    pg = (uint8_t)fm(c[1], 255.f);
    pb = (uint8_t)fm(c[2], 255.f);
    mark |= 2u;
    rgb = true;
  }
  w0 = mark | (pr << 8) | (pg << 16) | (pb << 24);
  if (rgb)
    reinterpret_cast<uint32_t*>(rec)[0] = w0;
  else
    reinterpret_cast<uint8_t*>(rec)[0] = (uint8_t)mark;
  rec->u = n.x;
  rec->v = n.y;
  rec->depth = b.t;
  *reinterpret_cast<uint4*>(&rec->object_id) = make_uint4(b.tri(), __float_as_uint(b.u()), __float_as_uint(b.v()), I.db_id);
  su = n.x;
  sv = n.y;
  if (!P.shadow) {
    if (P.shade_mode == 1) P.im[pix] = pixel_color(P, mark, pr, pg, pb, n.x, n.y);
    return false;
  }
  // canvas.cpp:836-853: from the hit point towards the light
  const float4 light = light_position(P);
  const float4 A = __ldg(I.tris + 3 * (size_t)b.slot());
  const float4 B = __ldg(I.tris + 3 * (size_t)b.slot() + 1);
  const float4 C = __ldg(I.tris + 3 * (size_t)b.slot() + 2);
  const float4 V0 = mat_vec(I.cs, A.x, A.y, A.z, 1.f);
  const float4 V1 = mat_vec(I.cs, B.x, B.y, B.z, 1.f);
  const float4 V2 = mat_vec(I.cs, C.x, C.y, C.z, 1.f);
  const float px = fa(fa(fm(V0.x, wgt), fm(b.u(), V1.x)), fm(b.v(), V2.x));
  const float py = fa(fa(fm(V0.y, wgt), fm(b.u(), V1.y)), fm(b.v(), V2.y));
  const float pz = fa(fa(fm(V0.z, wgt), fm(b.u(), V1.z)), fm(b.v(), V2.z));
  T.begin(P.inst, P.n_inst, px, py, pz, fs(light.x, px), fs(light.y, py), fs(light.z, pz), 1e-3f, FLT_MAX, true);
  return true;
}

template <class Tracer>
__device__ __forceinline__ void shadow_finish(const FrameParams& P, const Tracer& T, size_t pix, uint32_t w0, float su,
                                              float sv) {
  uint32_t mark = w0 & 0xffu;
  if (T.b.found) {
    mark |= 1u;
    reinterpret_cast<uint8_t*>(P.gbuf + pix)[0] = (uint8_t)mark;
  }
  if (P.shade_mode == 1)
    P.im[pix] = pixel_color(P, mark, (w0 >> 8) & 0xffu, (w0 >> 16) & 0xffu, (w0 >> 24) & 0xffu, su, sv);
}

// ------------------------------------------------------- rasterisation ----
//
// Primary hits without traversal. A ray can only pass the bounds gate of a
// triangle if it passes through the triangle's box widened by the ray's
// slab padding, so every pixel whose ray can accept a triangle has its
// centre inside the screen rectangle of that widened box's projection
// (bounded by interval arithmetic over the box). Each triangle takes those
// pixels (the rectangle grown by kRasterMargin pixels, far above the
// rounding of either the projection or the pixel rays) as candidates; each
// candidate runs the traversal's own Moller-Trumbore + gate with the
// pixel's own ray, and accepted ones go into a per-pixel 64-bit atomicMin of
// (t, instance, triangle id). The traversal's closest hit is the minimum of
// that same key over the same accepted triangles, so the minima are equal.
// k_resolve rebuilds each hit from its key and runs the primary finish;
// k_shadow traces the shadow rays it queued. Triangles with more than
// kRasterSmall candidates (and any whose box reaches the camera plane) go
// to a list that k_raster_large covers pixel-parallel; if the list
// overflows, the raster kernels stand down and k_frame traces the frame.

static const uint32_t kRasterSmall = 64;
static const float kRasterMargin = 0.05f;
static const int kRasterThreads = 256;

// the best-hit record of one candidate test, in registers
struct LocalBest {
  float t;
  bool found;
  float u_, v_;
  uint32_t inst_, tri_, slot_;
  __device__ __forceinline__ float& u() { return u_; }
  __device__ __forceinline__ float& v() { return v_; }
  __device__ __forceinline__ uint32_t& inst() { return inst_; }
  __device__ __forceinline__ uint32_t& tri() { return tri_; }
  __device__ __forceinline__ uint32_t& slot() { return slot_; }
};

__device__ __forceinline__ uint32_t raster_key_low(const FrameParams& P, uint32_t inst, uint32_t id) {
  return P.id_bits >= 32u ? id : ((inst << P.id_bits) | id);
}

// candidate queue: (pixel index, inst << id_bits | slot), in the shadow
// jobs' space (free until k_resolve), 4 entries per canvas pixel, cut into
// kRasterStripes stripes with a counter each (warps append to the stripe of
// their index, so no counter is contended by every warp)
__device__ __forceinline__ uint2* raster_queue(const FrameParams& P) {
  return reinterpret_cast<uint2*>(P.keys + (size_t)P.w * P.h);
}
__device__ __forceinline__ uint32_t raster_stripe_cap(const FrameParams& P) {
  const size_t cap = 4 * (size_t)P.w * P.h / kRasterStripes;
  return cap < 0xffffffffu ? (uint32_t)cap : 0xffffffffu;
}

// pixel (x, y) against triangle `slot` of instance `inst`
__device__ __forceinline__ void raster_candidate(const FrameParams& P, uint32_t inst, uint32_t slot, int x, int y) {
  float4 o, d;
  primary_ray(P, x, y, o, d);
  const DevInst& I = P.inst[inst];
  // Tracer::start_object
  const float4 oo = mat_vec(I.inv, o.x, o.y, o.z, 1.f);
  const float4 dd = mat_vec(I.inv, d.x, d.y, d.z, 0.f);
  const Ray r = make_ray(oo.x, oo.y, oo.z, dd.x, dd.y, dd.z, primary_t_near(P), I.scale);
  LocalBest b;
  b.t = FLT_MAX;
  b.found = false;
  if (tri_test(r, I.tris, slot, inst, b, false)) {
    const unsigned long long key =
        ((unsigned long long)__float_as_uint(b.t) << 32) | (unsigned long long)raster_key_low(P, inst, b.tri_);
    atomicMin(P.keys + (size_t)y * P.w + x, key);
  }
}

// Per-instance object -> clip matrices and paddings; resets the list.
__global__ void k_raster_setup(const FrameParams P) {
  __shared__ float w2c[16];  // proj * cs_inv
  if (threadIdx.x < 16) {
    const int r = threadIdx.x & 3, c = threadIdx.x >> 2;
    float acc = 0.f;
    for (int k = 0; k < 4; ++k) acc += P.proj[4 * k + r] * P.cs_inv[4 * c + k];
    w2c[4 * c + r] = acc;
  }
  __syncthreads();
  const float4 eye = mat_vec(P.cs, 0.f, 0.f, 0.f, 1.f);
  for (uint32_t i = threadIdx.x; i < P.n_inst; i += blockDim.x) {
    const DevInst& I = P.inst[i];
    RasterInst& R = P.rinst[i];
    for (int e = 0; e < 16; ++e) {
      const int r = e & 3, c = e >> 2;
      float acc = 0.f;
      for (int k = 0; k < 4; ++k) acc += w2c[4 * k + r] * I.cs[4 * c + k];
      R.M[e] = acc;
    }
    // make_ray's padding for the camera's rays in this object's space
    const float4 oo = mat_vec(I.inv, eye.x, eye.y, eye.z, 1.f);
    const float mo = fmaxf(fmaxf(fabsf(oo.x), fabsf(oo.y)), fabsf(oo.z));
    R.pad = fm(fa(mo, I.scale), 0x1p-19f);
    R.nt = I.nt;
    R.unused = 0u;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t first = 0;
    for (uint32_t i = 0; i < P.n_inst; ++i) {
      P.rinst[i].first = first;
      first += P.inst[i].nt;
    }
    P.rlist[0] = 0u;  // large triangles listed
    P.rlist[1] = 0u;  // list overflow
  }
  if (threadIdx.x < kRasterStripes) P.rlist[raster_stripe_counter(threadIdx.x)] = 0u;  // candidates per stripe
}

__device__ __forceinline__ uint32_t raster_instance(const FrameParams& P, uint32_t g) {
  uint32_t lo = 0, hi = P.n_inst;  // last instance with first <= g
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (P.rinst[mid].first <= g)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Candidate rectangle of triangle `slot` of instance `inst` (inclusive
// pixel bounds, clamped to the frame's rectangle); false when empty. Clip x,
// y and w are linear over the widened box, so their ranges are the low
// corner's value plus the negative or positive parts of the three edge
// terms; x / w over [x range] x [w range] (w > 0) is bounded by the four
// corner quotients.
__device__ __forceinline__ bool raster_rect(const FrameParams& P, const RasterInst& R, const float4& a,
                                            const float4& b, const float4& c, int& x0, int& y0, int& x1, int& y1) {
  const float e = 2.f * R.pad;
  const float lx = min3f(a.x, b.x, c.x) - e, ly = min3f(a.y, b.y, c.y) - e, lz = min3f(a.z, b.z, c.z) - e;
  const float dx = max3f(a.x, b.x, c.x) + e - lx, dy = max3f(a.y, b.y, c.y) + e - ly,
              dz = max3f(a.z, b.z, c.z) + e - lz;
  const float* M = R.M;
  float xl = M[0] * lx + M[4] * ly + M[8] * lz + M[12], xh = xl;
  float yl = M[1] * lx + M[5] * ly + M[9] * lz + M[13], yh = yl;
  float wl = M[3] * lx + M[7] * ly + M[11] * lz + M[15], wh = wl;
  const float tx[3] = {M[0] * dx, M[4] * dy, M[8] * dz};
  const float ty[3] = {M[1] * dx, M[5] * dy, M[9] * dz};
  const float tw[3] = {M[3] * dx, M[7] * dy, M[11] * dz};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    xl += fminf(tx[k], 0.f);
    xh += fmaxf(tx[k], 0.f);
    yl += fminf(ty[k], 0.f);
    yh += fmaxf(ty[k], 0.f);
    wl += fminf(tw[k], 0.f);
    wh += fmaxf(tw[k], 0.f);
  }
  const float sx = 0.5f * (float)P.w, sy = 0.5f * (float)P.h;
  float px0 = 0.f, px1 = -1.f, py0 = 0.f, py1 = -1.f;
  if (wl > 0.f) {
    // approximate reciprocals: the margin covers their error many times over
    const float rl = __fdividef(1.f, wl), rh = __fdividef(1.f, wh);
    // pixel x's ray passes through ndc 2 (x + 0.5) / w - 1
    px0 = (fminf(xl * rl, xl * rh) + 1.f) * sx - 0.5f - kRasterMargin;
    px1 = (fmaxf(xh * rl, xh * rh) + 1.f) * sx - 0.5f + kRasterMargin;
    py0 = (fminf(yl * rl, yl * rh) + 1.f) * sy - 0.5f - kRasterMargin;
    py1 = (fmaxf(yh * rl, yh * rh) + 1.f) * sy - 0.5f + kRasterMargin;
  }
  if (!(wl > 0.f) || !(px0 <= px1) || !(py0 <= py1)) {  // reaches the camera plane (or not finite): all pixels
    x0 = P.x0;
    y0 = P.y0;
    x1 = P.x1;
    y1 = P.y1;
    return true;
  }
  // clamp in float first (the projected values may be huge)
  x0 = (int)ceilf(fmaxf(px0, (float)P.x0));
  x1 = (int)floorf(fminf(px1, (float)P.x1));
  y0 = (int)ceilf(fmaxf(py0, (float)P.y0));
  y1 = (int)floorf(fminf(py1, (float)P.y1));
  return x0 <= x1 && y0 <= y1;
}

// Persistent warps over chunks of 32 triangles (one per lane), the next
// chunk's vertices loaded while the current one is projected. Small
// candidate sets are queued for k_raster_test (or, when the warp's stripe is
// full, tested by the warp itself with candidates spread over its lanes);
// large ones are listed for k_raster_large.
#ifndef J3DG_RASTER_MINBLOCKS
#define J3DG_RASTER_MINBLOCKS 4
#endif
// kOne: a single instance, whose matrix and padding are read once per block
template <bool kOne>
__global__ void __launch_bounds__(kRasterThreads, J3DG_RASTER_MINBLOCKS) k_raster(const FrameParams P) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warp_g = (blockIdx.x * kRasterThreads + threadIdx.x) >> 5;
  const uint32_t n_warps = (gridDim.x * kRasterThreads) >> 5;
  const uint32_t n_chunks = (P.raster_total + 31u) >> 5;
  const uint32_t stripe = warp_g % kRasterStripes;
  uint32_t* const stripe_count = P.rlist + raster_stripe_counter(stripe);
  uint2* const queue = raster_queue(P) + (size_t)stripe * raster_stripe_cap(P);
  const uint32_t cap = raster_stripe_cap(P);
  float4 na = make_float4(0.f, 0.f, 0.f, 0.f), nb = na, nc = na;
  uint32_t n_inst = 0, n_slot = 0;
  bool n_ok = false;
  // kOne: the instance's matrix and padding in shared memory (broadcast reads)
  __shared__ RasterInst R1;
  if (kOne) {
    if (threadIdx.x < sizeof(RasterInst) / 4)
      reinterpret_cast<uint32_t*>(&R1)[threadIdx.x] = reinterpret_cast<const uint32_t*>(P.rinst)[threadIdx.x];
    __syncthreads();
  }
  const float4* const tris1 = kOne ? P.inst[0].tris : nullptr;
  const auto fetch = [&](uint32_t chunk) {
    const uint32_t g = (chunk << 5) + lane;
    n_ok = false;
    if (chunk < n_chunks && g < P.raster_total) {
      const float4* tr;
      if (kOne) {
        n_slot = g;
        tr = tris1 + 3 * (size_t)g;
        n_ok = g < R1.nt;
      } else {
        n_inst = raster_instance(P, g);
        const RasterInst& R = P.rinst[n_inst];
        n_slot = g - R.first;
        tr = P.inst[n_inst].tris + 3 * (size_t)n_slot;
        n_ok = n_slot < R.nt;
      }
      if (n_ok) {
        na = __ldg(tr);
        nb = __ldg(tr + 1);
        nc = __ldg(tr + 2);
      }
    }
  };
  fetch(warp_g);
  for (uint32_t chunk = warp_g; chunk < n_chunks; chunk += n_warps) {
    const float4 a = na, b = nb, c = nc;
    const uint32_t inst = n_inst, slot = n_slot;
    const bool ok = n_ok;
    fetch(chunk + n_warps);
    uint32_t cnt = 0;
    int rx = 0, ry = 0, rw = 1;
    int x0, y0, x1, y1;
    if (ok && raster_rect(P, kOne ? R1 : P.rinst[inst], a, b, c, x0, y0, x1, y1)) {
      const uint64_t area = (uint64_t)(x1 - x0 + 1) * (uint64_t)(y1 - y0 + 1);
      if (area <= kRasterSmall) {
        cnt = (uint32_t)area;
        rx = x0;
        ry = y0;
        rw = x1 - x0 + 1;
      } else {
        const uint32_t k = atomicAdd(P.rlist, 1u);
        if (k < P.rlist_cap) {
          uint32_t* E = P.rlist + kRasterListHeader + (size_t)k * kRasterEntryWords;
          *reinterpret_cast<uint4*>(E) = make_uint4(inst, slot, (uint32_t)x0, (uint32_t)y0);
          *reinterpret_cast<uint4*>(E + 4) = make_uint4((uint32_t)x1, (uint32_t)y1, 0u, 0u);
        } else {
          atomicOr(P.rlist + 1, 1u);
        }
      }
    }
    // candidate c of the warp belongs to the first lane whose inclusive
    // count exceeds c
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0) continue;
    uint32_t qbase = 0;
    if (lane == 31) qbase = atomicAdd(stripe_count, total);
    qbase = __shfl_sync(0xffffffffu, qbase, 31);
    {
      const uint32_t key = raster_key_low(P, inst, slot);
      uint32_t q = qbase + incl - cnt, pix = (uint32_t)ry * P.w + (uint32_t)rx;
      int dx = 0;
      for (uint32_t j = 0; j < cnt; ++j, ++q) {
        if (q < cap) queue[q] = make_uint2(pix + (uint32_t)dx, key);
        if (++dx == rw) {
          dx = 0;
          pix += P.w;
        }
      }
    }
    if (qbase + total <= cap) continue;
    for (uint32_t c0 = 0; c0 < total; c0 += 32) {
      const uint32_t cc = c0 + lane;
      int own = 0;
#pragma unroll
      for (int step = 16; step >= 1; step >>= 1) {
        const uint32_t v = __shfl_sync(0xffffffffu, incl, own + step - 1);
        if (v <= cc) own += step;
      }
      const uint32_t o_incl = __shfl_sync(0xffffffffu, incl, own), o_cnt = __shfl_sync(0xffffffffu, cnt, own);
      const uint32_t o_inst = __shfl_sync(0xffffffffu, inst, own), o_slot = __shfl_sync(0xffffffffu, slot, own);
      const int o_rx = __shfl_sync(0xffffffffu, rx, own), o_ry = __shfl_sync(0xffffffffu, ry, own);
      const int o_rw = __shfl_sync(0xffffffffu, rw, own);
      if (cc < total && qbase + cc >= cap) {
        const uint32_t j = cc - (o_incl - o_cnt);
        raster_candidate(P, o_inst, o_slot, o_rx + (int)(j % (uint32_t)o_rw), o_ry + (int)(j / (uint32_t)o_rw));
      }
    }
  }
}

// The queued (pixel, triangle) candidates, stripe by stripe.
__global__ void __launch_bounds__(kRasterThreads) k_raster_test(const FrameParams P) {
  if (P.rlist[1]) return;
  const uint32_t cap = raster_stripe_cap(P);
  const uint32_t mask = P.id_bits >= 32u ? 0xffffffffu : (1u << P.id_bits) - 1u;
  const uint2* queue = raster_queue(P);
  for (uint32_t s = 0; s < kRasterStripes; ++s) {
    const uint32_t n = min(P.rlist[raster_stripe_counter(s)], cap);
    for (uint32_t i = blockIdx.x * kRasterThreads + threadIdx.x; i < n; i += gridDim.x * kRasterThreads) {
      const uint2 c = queue[(size_t)s * cap + i];
      const uint32_t inst = P.id_bits >= 32u ? 0u : c.y >> P.id_bits;
      raster_candidate(P, inst, c.y & mask, (int)(c.x % P.w), (int)(c.x / P.w));
    }
  }
}

// Listed triangles: each block column walks the pixels of a rectangle.
__global__ void __launch_bounds__(kRasterThreads) k_raster_large(const FrameParams P) {
  const uint32_t n = min(P.rlist[0], P.rlist_cap);
  if (P.rlist[1]) return;  // overflowed: the frame is traced
  for (uint32_t e = blockIdx.y; e < n; e += gridDim.y) {
    const uint32_t* E = P.rlist + kRasterListHeader + (size_t)e * kRasterEntryWords;
    const uint4 a = *reinterpret_cast<const uint4*>(E);
    const uint4 b = *reinterpret_cast<const uint4*>(E + 4);
    const int x0 = (int)a.z, y0 = (int)a.w, x1 = (int)b.x, y1 = (int)b.y;
    const uint32_t rw = (uint32_t)(x1 - x0 + 1);
    const uint64_t area = (uint64_t)rw * (uint64_t)(y1 - y0 + 1);
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < area; p += (uint64_t)gridDim.x * blockDim.x)
      raster_candidate(P, a.x, a.y, x0 + (int)(p % rw), y0 + (int)(p / rw));
  }
}

// Primary hit of pixel (x, y) from its raster key: the traversal's state as
// if the ray had just finished. Returns false for a miss.
template <class Tracer>
__device__ __forceinline__ bool raster_resolve(const FrameParams& P, Tracer& T, int x, int y,
                                               unsigned long long key) {
  if (key == ~0ull) return false;
  const uint32_t lo = (uint32_t)key;
  const uint32_t inst = P.id_bits >= 32u ? 0u : lo >> P.id_bits;
  const uint32_t id = P.id_bits >= 32u ? lo : lo & ((1u << P.id_bits) - 1u);
  if (inst >= P.n_inst || id >= P.inst[inst].nt) {
    atomicOr(P.status, J3DG_DEV_BAD_INDEX);
    return false;
  }
  const DevInst& I = P.inst[inst];
  const uint32_t slot = __ldg(I.slot_of + id);
  if (slot >= I.nt) {
    atomicOr(P.status, J3DG_DEV_BAD_INDEX);
    return false;
  }
  primary_begin(P, T, x, y);
  if (inst != 0u) {
    T.inst = inst;
    T.start_object(P.inst);
  }
  T.b.t = FLT_MAX;
  T.b.found = false;
  if (!tri_test(T.r, I.tris, slot, inst, T.b, false)) {  // the raster accepted it with the same test
    atomicOr(P.status, J3DG_DEV_BAD_INDEX);
    return false;
  }
  return true;
}

// A hit pixel's shadow ray and what its final colour needs; the direction
// is recomputed from the light as primary_finish computes it.
struct ShadowJob {
  float px, py, pz;
  uint32_t pix;
  uint32_t w0;
  float su, sv;
  uint32_t unused;
};
static const int kResolveThreads = 256;

__device__ __forceinline__ ShadowJob* shadow_jobs(const FrameParams& P) {
  return reinterpret_cast<ShadowJob*>(P.keys + (size_t)P.w * P.h);
}

// One thread per pixel of the rectangle: the miss record, or the hit rebuilt
// from its key and the primary finish (G-buffer record, shading); hits that
// cast a shadow ray are queued for k_shadow.
__global__ void __launch_bounds__(kResolveThreads) k_resolve(const FrameParams P) {
  if (P.rlist[1]) return;  // the list overflowed: k_frame traces the frame
  TracerT<kResolveThreads, false, kWidth> T;
  const uint32_t rw = (uint32_t)(P.x1 - P.x0 + 1), rh = (uint32_t)(P.y1 - P.y0 + 1);
  const uint32_t i = blockIdx.x * kResolveThreads + threadIdx.x;
  bool queue = false;
  ShadowJob J;
  if (i < rw * rh) {
    const int x = P.x0 + (int)(i % rw), y = P.y0 + (int)(i / rw);
    const size_t pix = (size_t)y * P.w + x;
    if (raster_resolve(P, T, x, y, P.keys[pix])) {
      uint32_t w0 = 0;
      float su = 0.f, sv = 0.f;
      if (primary_finish(P, T, pix, w0, su, sv)) {
        queue = true;
        J = ShadowJob{T.wr(0), T.wr(1), T.wr(2), (uint32_t)pix, w0, su, sv, 0u};
      }
    } else {
      write_miss(P, pix);
    }
  }
  const uint32_t m = __ballot_sync(0xffffffffu, queue);
  if (m) {
    const uint32_t lane = threadIdx.x & 31u;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(P.work + 1, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (queue) shadow_jobs(P)[base + __popc(m & ((1u << lane) - 1u))] = J;
  }
}

// the queued shadow rays, traced by persistent warps
struct ShadowSrc {
  const FrameParams* P;
  const ShadowJob* jobs;
  uint32_t n;
  float4 light;
  __device__ __forceinline__ uint32_t count() const { return n; }
  template <class Tracer>
  __device__ __forceinline__ bool begin(Tracer& T, const DevInst* insts, uint32_t n_inst, uint32_t i) {
    const ShadowJob J = jobs[i];
    // primary_finish's shadow ray (canvas.cpp:836-853)
    if (T.begin(insts, n_inst, J.px, J.py, J.pz, fs(light.x, J.px), fs(light.y, J.py), fs(light.z, J.pz), 1e-3f,
                FLT_MAX, true)) {
      finish(T, i);
      return false;
    }
    return true;
  }
  template <class Tracer>
  __device__ __forceinline__ void finish(Tracer& T, uint32_t i) {
    const ShadowJob J = jobs[i];
    shadow_finish(*P, T, J.pix, J.w0, J.su, J.sv);
  }
};

template <bool TOP>
__global__ void __launch_bounds__(kTraceThreads, J3DG_TRACE_MINBLOCKS) k_shadow(const FrameParams P) {
  if (P.rlist[1]) return;
  ShadowSrc src{&P, shadow_jobs(P), P.work[1], light_position(P)};
  persistent_trace<kIters, kTraceThreads, TOP, kWidth>(src, P.inst, P.n_inst, P.work + 2, P.status, P.counters);
}

template <bool kThroughput, bool TOP>
__global__ void __launch_bounds__(kFrameThreads, kThroughput ? kFrameBlocksT : kFrameBlocksL)
    k_frame(const FrameParams P) {
  TracerT<kFrameThreads, TOP, kWidth> T;
  uint2 stack[J3DG_STACK];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t n = primary_count(P);
  uint32_t* const taken = P.work + 4 + P.seq % kFrameDepth;
  int phase = 0;  // 0 idle, 1 primary, 2 shadow, 3 / 4 primary / shadow finished (parked)
  // the raster kernels made this frame: nothing to take (the exit still runs)
  bool exhausted = P.raster && P.rlist[1] == 0u, handed_over = false;
  PixState local;
  PixState& ps = pix_state<kThroughput && (J3DG_COLD_SMEM & 4) != 0, kFrameThreads>(local);
  ps = PixState{0, 0u, 0u, 0.f, 0.f};
  size_t& pix = ps.pix;
  uint32_t& w0 = ps.w0;
  float &su = ps.su, &sv = ps.sv;
  uint32_t visits = 0, tests = 0;
  // a finished ray's finish code (parked: phase 3 / 4, or in-line: 1 / 2);
  // the pixel's stamp follows its last write, one store site for all paths
  auto finish = [&](int ph) {
    bool last;
    if (ph == 1 || ph == 3) {
      phase = primary_finish(P, T, pix, w0, su, sv) ? 2 : 0;
      last = phase == 0;
    } else {
      shadow_finish(P, T, pix, w0, su, sv);
      phase = 0;
      last = true;
    }
    if (last) stamp_pixel(P, pix);
  };
#pragma unroll 1
  for (;;) {
    if (phase >= 3) finish(phase);
    // refill: every idle lane takes the next pixel; one atomic per warp
    const bool need = phase == 0 && !exhausted;
    const uint32_t m = __ballot_sync(0xffffffffu, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(taken, (uint32_t)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const uint32_t my = base + __popc(m & ((1u << lane) - 1u));
        int x, y;
        if (my >= n) {
          exhausted = true;
        } else if (item_pixel(P, my, x, y)) {
          pix = (size_t)y * P.w + x;
          if (P.n_inst == 0) {
            await_pixel(P, pix);
            write_miss(P, pix);
            stamp_pixel(P, pix);
          } else {
            primary_begin(P, T, x, y);
            phase = 1;
          }
        }
      }
    }
    if (!handed_over && __any_sync(0xffffffffu, exhausted) && handover_allowed(P)) {  // items all taken
      handed_over = true;
      asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    }
    if (__all_sync(0xffffffffu, phase == 0 && exhausted)) break;
    // all lanes step together; leave to refill once enough lanes are idle
#pragma unroll 1
    for (;;) {
      if ((phase == 1 || phase == 2) && T.step(P.inst, P.n_inst, P.status, visits, tests, stack)) {
#if J3DG_DEFER_FINISH
        phase += 2;
#else
        finish(phase);
#endif
      }
      if (__all_sync(0xffffffffu, phase != 1 && phase != 2)) break;
      if (__popc(__ballot_sync(0xffffffffu, (phase == 0 && !exhausted) || phase >= 3)) >= J3DG_REFILL_AT) break;
    }
  }
  if (P.counters) {
    atomicAdd(P.counters + 0, (unsigned long long)visits);
    atomicAdd(P.counters + 1, (unsigned long long)tests);
  }
  frame_exit(P, handed_over);
}

// j3dg_ray batches (find_closest / find_any through the C-ABI)
template <bool ANY>
struct BatchSrc {
  static const bool kAny = ANY;
  const j3dg_ray* rays;
  j3dg_hit* hits;
  uint32_t n;
  __device__ __forceinline__ uint32_t count() const { return n; }
  template <class Tracer>
  __device__ __forceinline__ bool begin(Tracer& T, const DevInst* insts, uint32_t n_inst, uint32_t i) {
    const float* f = reinterpret_cast<const float*>(rays + i);  // 40-byte records: 4-byte loads
    if (T.begin(insts, n_inst, f[0], f[1], f[2], f[4], f[5], f[6], f[8], f[9], ANY)) {
      finish(T, i);
      return false;
    }
    return true;
  }
  template <class Tracer>
  __device__ __forceinline__ void finish(Tracer& T, uint32_t i) {
    const float t_far = reinterpret_cast<const float*>(rays + i)[9];
    j3dg_hit h;
    h.found = T.b.found ? 1u : 0u;
    h.distance = T.b.found ? T.b.t : t_far;
    h.u = T.b.u();
    h.v = T.b.v();
    h.object_id = T.b.found ? T.b.tri() : 0xffffffffu;
    h.two_level_index = T.b.found ? T.b.inst() : 0xffffffffu;
    hits[i] = h;
  }
};

template <bool ANY, bool TOP>
__global__ void __launch_bounds__(kTraceThreads) k_rays(const DevInst* __restrict__ inst, uint32_t n_inst,
                                                        const j3dg_ray* __restrict__ rays, uint32_t n,
                                                        j3dg_hit* __restrict__ hits, uint32_t* counter,
                                                        uint32_t* status, unsigned long long* counters) {
  BatchSrc<ANY> src{rays, hits, n};
  persistent_trace<kIters, kTraceThreads, TOP, kWidth>(src, inst, n_inst, counter, status, counters);
}

// Many frames (canvases, scenes, cameras, resolutions of uneven size) in one
// persistent launch: the pixel lists of all frames are concatenated
// (offsets[f] = first work item of frame f, offsets[n] = total) and lanes
// refill from the one list, so small and large frames share the GPU with a
// single tail. Per-frame parameters live in device memory.
// blocks per SM that keep registers at or under ~96 for a block of TPB threads
template <int TPB, bool kThroughput>
struct MinBlocks {  // the same warps per SM as k_frame
  static const int per128 = kThroughput ? J3DG_TRACE_MINBLOCKS : J3DG_LATENCY_MINBLOCKS;
  static const int value = TPB >= 256 ? per128 / 2 : (TPB >= 128 ? per128 : 2 * per128);
};

template <int TPB, bool kThroughput, bool TOP>
__global__ void __launch_bounds__(TPB, (MinBlocks<TPB, kThroughput>::value))
    k_frame_batch(const FrameParams* __restrict__ params, const uint32_t* __restrict__ offsets, uint32_t n_frames,
                  uint32_t* work) {
  TracerT<TPB, TOP, kWidth> T;
  uint2 stack[J3DG_STACK];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t total = offsets[n_frames];
  int phase = 0;
  bool exhausted = false;
  PixState local;
  PixState& ps = pix_state<kThroughput && (J3DG_COLD_SMEM & 4) != 0, TPB>(local);
  ps = PixState{0, 0u, 0u, 0.f, 0.f};
  uint32_t& frame = ps.frame;
  size_t& pix = ps.pix;
  uint32_t& w0 = ps.w0;
  float &su = ps.su, &sv = ps.sv;
  uint32_t visits = 0, tests = 0;
#pragma unroll 1
  for (;;) {
    if (phase >= 3) {
      const FrameParams& P = params[frame];
      if (phase == 3) {
        phase = primary_finish(P, T, pix, w0, su, sv) ? 2 : 0;
      } else {
        shadow_finish(P, T, pix, w0, su, sv);
        phase = 0;
      }
    }
    const bool need = phase == 0 && !exhausted;
    const uint32_t m = __ballot_sync(0xffffffffu, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(work, (uint32_t)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const uint32_t my = base + __popc(m & ((1u << lane) - 1u));
        if (my >= total) {
          exhausted = true;
        } else {
          uint32_t lo = 0, hi = n_frames;  // offsets[lo] <= my < offsets[hi]
          while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(offsets + mid) <= my)
              lo = mid;
            else
              hi = mid;
          }
          frame = lo;
          const FrameParams& P = params[frame];
          int x, y;
          if (item_pixel(P, my - __ldg(offsets + frame), x, y)) {
            pix = (size_t)y * P.w + x;
            if (P.n_inst == 0) {
              write_miss(P, pix);
            } else {
              primary_begin(P, T, x, y);
              phase = 1;
            }
          }
        }
      }
    }
    if (__all_sync(0xffffffffu, phase == 0 && exhausted)) break;
#pragma unroll 1
    for (;;) {
      if (phase == 1 || phase == 2) {
        const FrameParams& P = params[frame];
        if (T.step(P.inst, P.n_inst, P.status, visits, tests, stack)) {
#if J3DG_DEFER_FINISH
          phase += 2;
#else
          if (phase == 1) {
            phase = primary_finish(P, T, pix, w0, su, sv) ? 2 : 0;
          } else {
            shadow_finish(P, T, pix, w0, su, sv);
            phase = 0;
          }
#endif
        }
      }
      if (__all_sync(0xffffffffu, phase != 1 && phase != 2)) break;
      if (__popc(__ballot_sync(0xffffffffu, (phase == 0 && !exhausted) || phase >= 3)) >= J3DG_REFILL_AT) break;
    }
  }
  unsigned long long* counters = params[0].counters;
  if (counters) {
    atomicAdd(counters + 0, (unsigned long long)visits);
    atomicAdd(counters + 1, (unsigned long long)tests);
  }
}

// --------------------------------------- primary hits from outside ----
//
// Frames whose primary hits another traversal found (the learned path):
// k_primary_rays writes the frame's primary rays (row-major over the
// rectangle, the same rays k_frame traces), the caller fills j3dg_hit per
// ray, k_keys_from_hits turns them into the raster keys, and the raster
// path's back half (k_resolve, k_shadow) makes the G-buffer records, the
// shadow rays and the plain shading from there.

__global__ void k_primary_rays(const FrameParams P, j3dg_ray* __restrict__ out) {
  const uint32_t rw = (uint32_t)(P.x1 - P.x0 + 1), rh = (uint32_t)(P.y1 - P.y0 + 1);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rw * rh) return;
  float4 o, d;
  primary_ray(P, P.x0 + (int)(i % rw), P.y0 + (int)(i / rw), o, d);
  float* f = reinterpret_cast<float*>(out + i);
  f[0] = o.x;
  f[1] = o.y;
  f[2] = o.z;
  f[3] = 1.f;
  f[4] = d.x;
  f[5] = d.y;
  f[6] = d.z;
  f[7] = 0.f;
  f[8] = primary_t_near(P);
  f[9] = FLT_MAX;
}

__global__ void k_keys_from_hits(const FrameParams P, const j3dg_hit* __restrict__ hits) {
  const uint32_t rw = (uint32_t)(P.x1 - P.x0 + 1), rh = (uint32_t)(P.y1 - P.y0 + 1);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    P.rlist[1] = 0u;  // no overflow: k_resolve and k_shadow run
    P.work[1] = P.work[2] = 0u;
  }
  if (i >= rw * rh) return;
  const j3dg_hit h = hits[i];
  const size_t pix = (size_t)(P.y0 + (int)(i / rw)) * P.w + (P.x0 + (int)(i % rw));
  const uint32_t low = P.id_bits >= 32u ? h.object_id : ((h.two_level_index << P.id_bits) | h.object_id);
  P.keys[pix] = h.found ? ((unsigned long long)__float_as_uint(h.distance) << 32 | low) : ~0ull;
}

template <class K>
static int persistent_blocks(K* kernel, int threads = kTraceThreads) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
  return sms * (per > 0 ? per : 1);
}

// ----------------------------------------------------------- k_shade ----

__device__ __forceinline__ bool differs(const j3dg_pixel& a, const j3dg_pixel& b) {
  const float th = 0.001f;
  return b.object_id != 0xffffffffu && (fabsf(fs(a.u, b.u)) > th || fabsf(fs(a.v, b.v)) > th);
}

__device__ __forceinline__ float dot4(float4 a, float4 b) {
  return fa(fa(fa(fm(a.x, b.x), fm(a.y, b.y)), fm(a.z, b.z)), fm(a.w, b.w));
}

// canvas.cpp:287-315
__device__ float convex_cos_angle(const FrameParams& P, float x1, float y1, float u1, float v1, float depth1, float x2,
                                  float y2, float u2, float v2, float depth2) {
  float4 d1 = mat_vec(P.pinv, fs(fm(2.f, __fdiv_rn(fa(x1, 0.5f), (float)P.w)), 1.f),
                      fs(fm(2.f, __fdiv_rn(fa(y1, 0.5f), (float)P.h)), 1.f), P.near_plane, 1.f);
  d1.w = 0.f;
  float4 p1 = make_float4(fm(depth1, d1.x), fm(depth1, d1.y), fm(depth1, d1.z), fm(depth1, d1.w));
  float4 d2 = mat_vec(P.pinv, fs(fm(2.f, __fdiv_rn(fa(x2, 0.5f), (float)P.w)), 1.f),
                      fs(fm(2.f, __fdiv_rn(fa(y2, 0.5f), (float)P.h)), 1.f), P.near_plane, 1.f);
  d2.w = 0.f;
  float4 p2 = make_float4(fm(depth2, d2.x), fm(depth2, d2.y), fm(depth2, d2.z), fm(depth2, d2.w));
  float4 n1 = make_float4(u1, v1, __fsqrt_rn(fs(fs(1.f, fm(u1, u1)), fm(v1, v1))), 0.f);
  float4 n2 = make_float4(u2, v2, __fsqrt_rn(fs(fs(1.f, fm(u2, u2)), fm(v2, v2))), 0.f);
  if ((double)fabsf(fs(dot4(n1, n2), 1.f)) > 0.0001) {
    float4 pt = make_float4(fs(p2.x, p1.x), fs(p2.y, p1.y), fs(p2.z, p1.z), fs(p2.w, p1.w));
    float len = __fsqrt_rn(dot4(pt, pt));
    pt = make_float4(__fdiv_rn(pt.x, len), __fdiv_rn(pt.y, len), __fdiv_rn(pt.z, len), __fdiv_rn(pt.w, len));
    return dot4(pt, n1);
  }
  return 0.f;
}

__device__ __forceinline__ uint32_t one_bit_res(uint32_t clr) {
  return ((((clr & 0xff0000u) >> 16) + ((clr & 0xff00u) >> 8) + (clr & 0xffu)) >> 7) + 1u;
}

// canvas_to_image for one pixel. mode: 0 plain, 1 edges, 2 wireframe, 3 one-bit.
__global__ void __launch_bounds__(256) k_shade(const FrameParams P, const j3dg_pixel* __restrict__ G, int mode,
                                               int fill_background) {
  const uint32_t x = blockIdx.x * 32 + (threadIdx.x & 31);
  const uint32_t y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (x >= P.w || y >= P.h) return;
  const size_t pix = (size_t)y * P.w + x;
  const j3dg_pixel p = G[pix];
  if (p.object_id == 0xffffffffu) {
    if (fill_background) P.im[pix] = P.background ? __ldg(P.background + pix) : P.im[pix];
    return;
  }
  const uint32_t mark = p.mark;
  uint32_t out;
  const bool last_col = (x + 1 == P.w);
  const j3dg_pixel* up = G + (size_t)(y == 0 ? 0 : y - 1) * P.w + x;
  if (mode == 3) {
    uint32_t clr = get_color(P.matcap, P.mw, get_U(p.u, P.mw), get_V(p.v, P.mh), mark);
    uint32_t res = one_bit_res(clr);
    if (last_col) {
      out = (((P.w - 1) % res == 0) && (y % res == 0)) ? 0xff000000u : 0xffffffffu;
    } else {
      float angle = 1.f;
      const j3dg_pixel r = G[pix + 1];
      const j3dg_pixel* q = nullptr;
      j3dg_pixel u = *up;
      if (differs(p, r))
        q = &r;
      else if (differs(p, u))
        q = &u;
      if (q) {
        float w1 = __fsqrt_rn(fs(fs(1.f, fm(p.u, p.u)), fm(p.v, p.v)));
        float w2 = __fsqrt_rn(fs(fs(1.f, fm(q->u, q->u)), fm(q->v, q->v)));
        angle = fa(fa(fm(p.u, q->u), fm(p.v, q->v)), fm(w1, w2));
      }
      bool black = ((x % res == 0) && (y % res == 0));
      if (fabsf(angle) < 0.95f) black = (res == 1) ? !black : true;
      out = black ? 0xff000000u : 0xffffffffu;
    }
  } else if (mode == 2 && !last_col) {
    const j3dg_pixel r = G[pix + 1];
    const j3dg_pixel u = *up;
    if ((r.object_id != 0xffffffffu && r.object_id != p.object_id) ||
        (u.object_id != 0xffffffffu && u.object_id != p.object_id)) {
      const float scale = fm(fa(fm(p.u, p.u), fm(p.v, p.v)), 0.5f);
      uint32_t c = (unsigned char)fm(255.f, scale);
      out = 0xff000000u | (c << 16) | (c << 8) | c;
    } else {
      out = pixel_color(P, mark, p.r, p.g, p.b, p.u, p.v);
    }
  } else if (mode == 1 && !last_col) {
    const j3dg_pixel r = G[pix + 1];
    const j3dg_pixel u = *up;
    if (differs(p, r)) {
      float a = convex_cos_angle(P, (float)x, (float)y, p.u, p.v, p.depth, fa((float)x, 1.f), (float)y, r.u, r.v,
                                 r.depth);
      out = get_angle_color(a, P, p.u, p.v, mark);
    } else if (differs(p, u)) {
      float a = convex_cos_angle(P, (float)x, (float)y, p.u, p.v, p.depth, (float)x, fs((float)y, 1.f), u.u, u.v,
                                 u.depth);
      out = get_angle_color(a, P, p.u, p.v, mark);
    } else {
      out = pixel_color(P, mark, p.r, p.g, p.b, p.u, p.v);
    }
  } else {
    out = pixel_color(P, mark, p.r, p.g, p.b, p.u, p.v);
  }
  P.im[pix] = out;
}

__global__ void k_copy_u32(uint32_t* __restrict__ dst, const uint32_t* __restrict__ src, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

__global__ void k_clear_ids(j3dg_pixel* __restrict__ G, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    G[i].db_id = 0u;
    G[i].object_id = 0xffffffffu;
  }
}

__global__ void k_init_pixels(j3dg_pixel* __restrict__ G, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    // pixel() constructor (pixel.h:13) followed by canvas::resize (canvas.cpp:126-130)
    uint4* q = reinterpret_cast<uint4*>(G + i);
    q[0] = make_uint4(0u, 0u, 0u, 0u);
    q[1] = make_uint4(0xffffffffu, 0u, 0u, 0u);
  }
}

// ------------------------------------------------------------ launchers ----

// k_frame, as a programmatic dependent of the previous kernel on the stream
// when the frame overlaps its canvas's previous frame
template <bool kT, bool TOP>
static cudaError_t launch_frame(int blocks, const FrameParams& P, bool overlap, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3((unsigned)kFrameThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = overlap ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k_frame<kT, TOP>, P);
}

cudaError_t launch_render(const FrameParams& P, cudaStream_t st) {
  const int rw = P.x1 - P.x0 + 1, rh = P.y1 - P.y0 + 1;
  if (rw <= 0 || rh <= 0) return cudaSuccess;
  static int blocks_t = 0, blocks_l = 0, blocks_tt = 0, blocks_lt = 0;
  if (!blocks_t) {
    blocks_t = persistent_blocks(k_frame<true, false>, kFrameThreads);
    blocks_l = persistent_blocks(k_frame<false, false>, kFrameThreads);
    blocks_tt = persistent_blocks(k_frame<true, true>, kFrameThreads);
    blocks_lt = persistent_blocks(k_frame<false, true>, kFrameThreads);
  }
  // an overlapped frame finds its counter slot zeroed by the slot's
  // previous user (completed before this frame could start); any other
  // frame zeroes the canvas's slots here
  const bool overlap = P.wait_seq != 0u && !P.raster;
  cudaError_t e = cudaSuccess;
  if (!overlap) e = cudaMemsetAsync(P.work + 4, 0, 2 * kFrameDepth * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (P.raster) {
    static int blocks_s = 0, blocks_t = 0, blocks_r = 0;
    if (!blocks_s) {
      blocks_s = persistent_blocks(k_shadow<false>);
      blocks_t = persistent_blocks(k_raster_test, kRasterThreads);
      blocks_r = persistent_blocks(k_raster<false>, kRasterThreads);
    }
    e = cudaMemsetAsync(P.work, 0, 4 * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(P.keys, 0xff, sizeof(unsigned long long) * (size_t)P.w * P.h, st);
    if (e != cudaSuccess) return e;
    k_raster_setup<<<1, 128, 0, st>>>(P);
    const uint32_t need = (P.raster_total + kRasterThreads - 1) / kRasterThreads;
    if (P.n_inst == 1)
      k_raster<true><<<need < (uint32_t)blocks_r ? need : (uint32_t)blocks_r, kRasterThreads, 0, st>>>(P);
    else
      k_raster<false><<<need < (uint32_t)blocks_r ? need : (uint32_t)blocks_r, kRasterThreads, 0, st>>>(P);
    k_raster_large<<<dim3(16, 64), kRasterThreads, 0, st>>>(P);
    k_raster_test<<<blocks_t, kRasterThreads, 0, st>>>(P);
    k_resolve<<<(unsigned)(((size_t)rw * rh + kResolveThreads - 1) / kResolveThreads), kResolveThreads, 0, st>>>(P);
    if (P.top)
      k_shadow<true><<<blocks_s, kTraceThreads, 0, st>>>(P);
    else
      k_shadow<false><<<blocks_s, kTraceThreads, 0, st>>>(P);
    // k_frame below returns at once unless the large-triangle list overflowed
  }
  const bool thr = primary_items(P) >= J3DG_THROUGHPUT_ITEMS;
  if (P.top) {
    if (thr)
      e = launch_frame<true, true>(blocks_tt, P, overlap, st);
    else
      e = launch_frame<false, true>(blocks_lt, P, overlap, st);
  } else {
    if (thr)
      e = launch_frame<true, false>(blocks_t, P, overlap, st);
    else
      e = launch_frame<false, false>(blocks_l, P, overlap, st);
  }
  return e != cudaSuccess ? e : cudaGetLastError();
}

template <bool kT, bool TOP>
static cudaError_t launch_batch_variant(const FrameParams* d_params, const uint32_t* d_offsets, uint32_t n_frames,
                                        uint32_t* work, int block_threads, cudaStream_t st) {
  static int b64 = 0, b128 = 0, b256 = 0;
  if (!b64) {
    b64 = persistent_blocks(k_frame_batch<64, kT, TOP>, 64);
    b128 = persistent_blocks(k_frame_batch<128, kT, TOP>, 128);
    b256 = persistent_blocks(k_frame_batch<256, kT, TOP>, 256);
  }
  if (block_threads == 64)
    k_frame_batch<64, kT, TOP><<<b64, 64, 0, st>>>(d_params, d_offsets, n_frames, work);
  else if (block_threads == 256)
    k_frame_batch<256, kT, TOP><<<b256, 256, 0, st>>>(d_params, d_offsets, n_frames, work);
  else
    k_frame_batch<128, kT, TOP><<<b128, 128, 0, st>>>(d_params, d_offsets, n_frames, work);
  return cudaGetLastError();
}

cudaError_t launch_render_batch(const FrameParams* d_params, const uint32_t* d_offsets, uint32_t n_frames,
                                uint32_t total_items, uint32_t* work, int block_threads, bool top, int,
                                cudaStream_t st) {
  if (n_frames == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(work, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  const bool thr = total_items >= J3DG_THROUGHPUT_ITEMS;
  if (top)
    return thr ? launch_batch_variant<true, true>(d_params, d_offsets, n_frames, work, block_threads, st)
               : launch_batch_variant<false, true>(d_params, d_offsets, n_frames, work, block_threads, st);
  return thr ? launch_batch_variant<true, false>(d_params, d_offsets, n_frames, work, block_threads, st)
             : launch_batch_variant<false, false>(d_params, d_offsets, n_frames, work, block_threads, st);
}

uint32_t primary_items(const FrameParams& P) {
  const uint32_t rw = (uint32_t)(P.x1 - P.x0 + 1), rh = (uint32_t)(P.y1 - P.y0 + 1);
  return ((rw + 7u) >> 3) * ((rh + 3u) >> 2) * 32u;
}

cudaError_t launch_shade(const FrameParams& P, const j3dg_pixel* G, int mode, int fill_background, cudaStream_t st) {
  dim3 grid((P.w + 31) / 32, (P.h + 7) / 8);
  k_shade<<<grid, 256, 0, st>>>(P, G, mode, fill_background);
  return cudaGetLastError();
}

cudaError_t launch_copy_u32(uint32_t* dst, const uint32_t* src, size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_copy_u32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dst, src, n);
  return cudaGetLastError();
}

cudaError_t launch_clear_ids(j3dg_pixel* G, size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_clear_ids<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(G, n);
  return cudaGetLastError();
}

cudaError_t launch_init_pixels(j3dg_pixel* G, size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_init_pixels<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(G, n);
  return cudaGetLastError();
}

cudaError_t launch_primary_rays(const FrameParams& P, j3dg_ray* out, cudaStream_t st) {
  const uint32_t n = (uint32_t)(P.x1 - P.x0 + 1) * (uint32_t)(P.y1 - P.y0 + 1);
  if (n == 0) return cudaSuccess;
  k_primary_rays<<<(n + 255) / 256, 256, 0, st>>>(P, out);
  return cudaGetLastError();
}

cudaError_t launch_frame_from_hits(const FrameParams& P, const j3dg_hit* hits, cudaStream_t st) {
  const uint32_t rw = (uint32_t)(P.x1 - P.x0 + 1), rh = (uint32_t)(P.y1 - P.y0 + 1);
  if (rw * rh == 0) return cudaSuccess;
  static int blocks_s = 0;
  if (!blocks_s) blocks_s = persistent_blocks(k_shadow<false>);
  k_keys_from_hits<<<(rw * rh + 255) / 256, 256, 0, st>>>(P, hits);
  k_resolve<<<(rw * rh + kResolveThreads - 1) / kResolveThreads, kResolveThreads, 0, st>>>(P);
  if (P.top)
    k_shadow<true><<<blocks_s, kTraceThreads, 0, st>>>(P);
  else
    k_shadow<false><<<blocks_s, kTraceThreads, 0, st>>>(P);
  return cudaGetLastError();
}

cudaError_t launch_rays(const DevInst* inst, uint32_t n_inst, bool top, int, const j3dg_ray* rays, uint32_t n,
                        j3dg_hit* hits, bool any, uint32_t* counter, uint32_t* status, unsigned long long* counters,
                        cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  static int blocks_c = 0, blocks_a = 0;
  if (!blocks_c) {
    blocks_c = persistent_blocks(k_rays<false, false>);
    blocks_a = persistent_blocks(k_rays<true, false>);
  }
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (top) {
    if (any)
      k_rays<true, true><<<blocks_a, kTraceThreads, 0, st>>>(inst, n_inst, rays, n, hits, counter, status, counters);
    else
      k_rays<false, true><<<blocks_c, kTraceThreads, 0, st>>>(inst, n_inst, rays, n, hits, counter, status, counters);
  } else {
    if (any)
      k_rays<true, false><<<blocks_a, kTraceThreads, 0, st>>>(inst, n_inst, rays, n, hits, counter, status, counters);
    else
      k_rays<false, false><<<blocks_c, kTraceThreads, 0, st>>>(inst, n_inst, rays, n, hits, counter, status, counters);
  }
  return cudaGetLastError();
}

}  // namespace J3DG_WNS
}  // namespace j3dg
