// device_common.cuh -- exact fp32 math, ray preparation, slab test,
// Moller-Trumbore with the bounds gate, and wide-BVH traversal.
//
// Every operation that decides a hit or produces a G-buffer value is written
// with round-to-nearest intrinsics (__fmul_rn, __fadd_rn, __fdiv_rn,
// __fsqrt_rn, __fmaf_rn), so it matches the host restatement bit for bit
// regardless of FMA contraction. The fixed operation order:
//   mat x vec   r_i = ((m[i] x + m[4+i] y) + m[8+i] z) + m[12+i] w   (column-major)
//   dot3        (a.x b.x + a.y b.y) + a.z b.z
//   cross       (a.y b.z - a.z b.y, a.z b.x - a.x b.z, a.x b.y - a.y b.x)
//   triangle    Moller-Trumbore (1997), double sided; accept iff det != 0,
//               u >= 0, v >= 0, u + v <= 1, t > t_near, the hit t inside the
//               slab interval of the triangle's own AABB, and (t, object,
//               triangle) smaller than the best so far (strictly t < t_far).
//   slab        d' = d with |d_i| < 1e-12 replaced by copysign(1e-12, d_i),
//               inv = 1/d', pad = (max|o| + mesh scale) 2^-19, near/far
//               origins o -/+ pad by sign(inv), t = fma(plane, inv, -(o') inv),
//               enter = max over axes, exit = min over axes.
// Node boxes hold their triangles' boxes exactly (min/max are exact) and the
// slab formula is monotone in the planes, so no node on the path to an
// accepted triangle is ever culled: results do not depend on the BVH shape.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace j3dg {

struct DevInst {
  const float4* nodes;     // 8 float4 per wide node
  const float4* tris;      // 3 float4 per triangle, leaf order; v0.w = id bits
  const float4* normals;   // per triangle id
  const uint32_t* slot_of; // leaf-order position (tris) of each triangle id
  const uint32_t* index;   // caller's triangle indices (3 per triangle)
  const float* colors;     // per vertex rgb or null
  const float* uv;         // 6 per triangle or null
  const uint32_t* tex;     // RGBA8 or null
  uint32_t tex_w, tex_h;
  uint32_t root_ref;       // inner node 0, or a leaf ref for tiny meshes
  uint32_t n_nodes;
  uint32_t nt;
  uint32_t db_id;
  float scale;
  uint32_t width;          // children per BVH node (2, 4, 8)
  float cs[16];
  float inv[16];
};

// Header of every instance table, just in front of its first DevInst (the
// kernels receive &inst[0]): the per-frame top level over the objects' world
// boxes (the two-level structure of canvas.cpp:762; built on the host,
// toplevel.cpp), whose nodes follow the table. Leaves hold one object:
// ref = J3DG_LEAF_BIT | object << 3.
struct DevTop {
  const float4* nodes;  // BVH4 nodes, or null when the table has no top level
  uint32_t root;        // inner node 0, or the leaf of the only object
  uint32_t n_nodes;
  uint32_t n_inst;
  float pad_scale;      // max |coordinate| of the padded object boxes
  uint32_t reserved[2];
};
static_assert(sizeof(DevTop) % 16 == 0, "the instance table follows the header");
static_assert(sizeof(DevInst) % 16 == 0, "top-level nodes follow the instance table");

__device__ __forceinline__ const DevTop& top_of(const DevInst* insts) {
  return reinterpret_cast<const DevTop*>(insts)[-1];
}

// inst while the walk is in the top level; stack entry that returns the walk
// from an object to the top level (J3DG_LEAF_BIT with a first triangle beyond
// J3DG_MAX_TRIANGLES: never a leaf of a mesh)
static const uint32_t kTopInst = 0xffffffffu;
static const uint32_t kPopTop = 0xfffffffeu;

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }

__device__ __forceinline__ float4 mat_vec(const float* m, float x, float y, float z, float w) {
  float r[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) r[i] = fa(fa(fa(fm(m[i], x), fm(m[4 + i], y)), fm(m[8 + i], z)), fm(m[12 + i], w));
  return make_float4(r[0], r[1], r[2], r[3]);
}

#ifndef J3DG_PREFETCH
#define J3DG_PREFETCH 1
#endif

// three-input min / max (one instruction each on sm_100 and later); min and
// max are exact, so the grouping does not change any value
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
  return fa(fa(fm(ax, bx), fm(ay, by)), fm(az, bz));
}

struct Ray {
  float ox, oy, oz, dx, dy, dz;
  float ix, iy, iz;     // 1 / clamped direction
  float nnx, nny, nnz;  // -(near origin) * inv
  float nfx, nfy, nfz;  // -(far origin) * inv
  uint32_t neg;         // bit a: inv_a < 0
  float t_near;
};

__device__ __forceinline__ void prep_axis(float o, float d, float pad, float& inv, float& nn, float& nf, bool& neg) {
  float dd = (fabsf(d) < 1e-12f) ? copysignf(1e-12f, d) : d;
  inv = __fdiv_rn(1.f, dd);
  neg = inv < 0.f;
  float on = neg ? fs(o, pad) : fa(o, pad);
  float of = neg ? fa(o, pad) : fs(o, pad);
  nn = fm(-on, inv);
  nf = fm(-of, inv);
}

__device__ __forceinline__ Ray make_ray_pad(float ox, float oy, float oz, float dx, float dy, float dz, float t_near,
                                            float pad) {
  Ray r;
  r.ox = ox;
  r.oy = oy;
  r.oz = oz;
  r.dx = dx;
  r.dy = dy;
  r.dz = dz;
  r.t_near = t_near;
  bool nx, ny, nz;
  prep_axis(ox, dx, pad, r.ix, r.nnx, r.nfx, nx);
  prep_axis(oy, dy, pad, r.iy, r.nny, r.nfy, ny);
  prep_axis(oz, dz, pad, r.iz, r.nnz, r.nfz, nz);
  r.neg = (nx ? 1u : 0u) | (ny ? 2u : 0u) | (nz ? 4u : 0u);
  return r;
}

__device__ __forceinline__ Ray make_ray(float ox, float oy, float oz, float dx, float dy, float dz, float t_near,
                                        float scale) {
  Ray r;
  r.ox = ox;
  r.oy = oy;
  r.oz = oz;
  r.dx = dx;
  r.dy = dy;
  r.dz = dz;
  r.t_near = t_near;
  float mo = fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz));
  float pad = fm(fa(mo, scale), 0x1p-19f);
  bool nx, ny, nz;
  prep_axis(ox, dx, pad, r.ix, r.nnx, r.nfx, nx);
  prep_axis(oy, dy, pad, r.iy, r.nny, r.nfy, ny);
  prep_axis(oz, dz, pad, r.iz, r.nnz, r.nfz, nz);
  r.neg = (nx ? 1u : 0u) | (ny ? 2u : 0u) | (nz ? 4u : 0u);
  return r;
}

// Slab interval of [lo, hi]; returns (enter, exit) before clipping.
__device__ __forceinline__ void slab(const Ray& r, float lox, float loy, float loz, float hix, float hiy, float hiz,
                                     float& tn, float& tf) {
  float pnx = (r.neg & 1u) ? hix : lox, pfx = (r.neg & 1u) ? lox : hix;
  float pny = (r.neg & 2u) ? hiy : loy, pfy = (r.neg & 2u) ? loy : hiy;
  float pnz = (r.neg & 4u) ? hiz : loz, pfz = (r.neg & 4u) ? loz : hiz;
  tn = max3f(__fmaf_rn(pnx, r.ix, r.nnx), __fmaf_rn(pny, r.iy, r.nny), __fmaf_rn(pnz, r.iz, r.nnz));
  tf = min3f(__fmaf_rn(pfx, r.ix, r.nfx), __fmaf_rn(pfy, r.iy, r.nfy), __fmaf_rn(pfz, r.iz, r.nfz));
}

// 1: state a traversal step does not read (the world ray, the best hit's
// attributes) lives in shared memory, one slot per thread, so that the
// registers left cover the step's working set and more warps fit an SM.
// The slots are sized by the tracing kernel's block (N threads): every
// tracing kernel's launch bounds equal the N it instantiates.
#ifndef J3DG_COLD_SMEM
#define J3DG_COLD_SMEM 7
#endif
template <int N>
struct ColdSlots {
  static constexpr int S = N;
  // world ray [6][S], best-hit u / v [2][S], best-hit inst / tri / slot [3][S]
  __device__ static __forceinline__ float* ray() {
    __shared__ float a[6 * S];
    return a;
  }
  __device__ static __forceinline__ float* uv() {
    __shared__ float a[2 * S];
    return a;
  }
  __device__ static __forceinline__ uint32_t* key() {
    __shared__ uint32_t a[3 * S];
    return a;
  }
};

// Best hit so far: t and found are read every step; the key (inst, tri) only
// on a t tie, u / v / slot only when the ray finishes.
template <int N>
struct BestT {
  float t;
  bool found;  // found == (t < t_far set by an accept)
#if J3DG_COLD_SMEM & 2
  using C = ColdSlots<N>;
  __device__ __forceinline__ float& u() const { return C::uv()[threadIdx.x]; }
  __device__ __forceinline__ float& v() const { return C::uv()[C::S + threadIdx.x]; }
  __device__ __forceinline__ uint32_t& inst() const { return C::key()[threadIdx.x]; }
  __device__ __forceinline__ uint32_t& tri() const { return C::key()[C::S + threadIdx.x]; }
  __device__ __forceinline__ uint32_t& slot() const { return C::key()[2 * C::S + threadIdx.x]; }
#else
  float u_, v_;
  uint32_t inst_, tri_, slot_;
  __device__ __forceinline__ float& u() { return u_; }
  __device__ __forceinline__ float& v() { return v_; }
  __device__ __forceinline__ uint32_t& inst() { return inst_; }
  __device__ __forceinline__ uint32_t& tri() { return tri_; }
  __device__ __forceinline__ uint32_t& slot() { return slot_; }
  __device__ __forceinline__ float u() const { return u_; }
  __device__ __forceinline__ float v() const { return v_; }
  __device__ __forceinline__ uint32_t inst() const { return inst_; }
  __device__ __forceinline__ uint32_t tri() const { return tri_; }
  __device__ __forceinline__ uint32_t slot() const { return slot_; }
#endif
};

__device__ __forceinline__ bool key_less(uint32_t ia, uint32_t ta, uint32_t ib, uint32_t tb) {
  return ia < ib || (ia == ib && ta < tb);
}

// Moller-Trumbore + gate for triangle `slot`. any: the caller stops at the
// first accept, so the (t, key) comparison only needs t < t_best.
template <class BestHit>
__device__ __forceinline__ bool tri_test(const Ray& r, const float4* __restrict__ tris, uint32_t slot, uint32_t inst,
                                         BestHit& b, bool any) {
  const float4 a = __ldg(tris + 3 * (size_t)slot);
  const float4 c1 = __ldg(tris + 3 * (size_t)slot + 1);
  const float4 c2 = __ldg(tris + 3 * (size_t)slot + 2);
  float e1x = fs(c1.x, a.x), e1y = fs(c1.y, a.y), e1z = fs(c1.z, a.z);
  float e2x = fs(c2.x, a.x), e2y = fs(c2.y, a.y), e2z = fs(c2.z, a.z);
  float px = fs(fm(r.dy, e2z), fm(r.dz, e2y));
  float py = fs(fm(r.dz, e2x), fm(r.dx, e2z));
  float pz = fs(fm(r.dx, e2y), fm(r.dy, e2x));
  float det = dot3(e1x, e1y, e1z, px, py, pz);
  if (det == 0.f) return false;
  float inv = __fdiv_rn(1.f, det);
  float sx = fs(r.ox, a.x), sy = fs(r.oy, a.y), sz = fs(r.oz, a.z);
  float u = fm(dot3(sx, sy, sz, px, py, pz), inv);
  float qx = fs(fm(sy, e1z), fm(sz, e1y));
  float qy = fs(fm(sz, e1x), fm(sx, e1z));
  float qz = fs(fm(sx, e1y), fm(sy, e1x));
  float v = fm(dot3(r.dx, r.dy, r.dz, qx, qy, qz), inv);
  float t = fm(dot3(e2x, e2y, e2z, qx, qy, qz), inv);
  if (!(u >= 0.f && v >= 0.f && fa(u, v) <= 1.f)) return false;
  if (!(t > r.t_near)) return false;
  uint32_t id = __float_as_uint(a.w);
  if (!(t < b.t || (!any && t == b.t && b.found && key_less(inst, id, b.inst(), b.tri())))) return false;
  // bounds gate: t inside the slab interval of the triangle's own box
  float tn, tf;
  slab(r, min3f(a.x, c1.x, c2.x), min3f(a.y, c1.y, c2.y), min3f(a.z, c1.z, c2.z), max3f(a.x, c1.x, c2.x),
       max3f(a.y, c1.y, c2.y), max3f(a.z, c1.z, c2.z), tn, tf);
  if (!(tn <= t && t <= tf)) return false;
  b.t = t;
  b.inst() = inst;
  b.tri() = id;
  b.u() = u;
  b.v() = v;
  b.slot() = slot;
  b.found = true;
  return true;
}

// Resumable traversal of one world ray over all objects of the scene
// (qbvh_two_level_with_transformations::find_closest_triangle): in an
// object the ray is in that object's space (origin as a point, direction as
// a vector) and the object's BVH4 is walked with a per-thread stack. With
// TOP, the walk starts in the table's top level (a BVH4 over the objects'
// world boxes) with the world ray; a top-level leaf pushes a kPopTop entry
// (which carries the top level's remaining visit budget) and enters its
// object; popping that entry takes the world ray back to the top level.
// Without TOP the objects are walked one after the other. run() advances by
// at most `iters` node or leaf steps, so persistent warps can refill lanes
// whose rays have finished. Corrupt trees raise status bits instead of
// trapping.
// Child c's near / far planes of a width-W node for the ray's octant, and
// its ref (the layout of J3DG_NODE_F4; the same values slab() selects).
template <int W>
struct NodeLoad {
  float pnx[W], pfx[W], pny[W], pfy[W], pnz[W], pfz[W];
  uint32_t rc[W];
  __device__ __forceinline__ void load(const float4* __restrict__ nd, uint32_t neg) {
    const uint32_t ox = neg & 1u, oy = (neg >> 1) & 1u, oz = (neg >> 2) & 1u;
    if constexpr (W == 2) {
      // [lo0 lo1 hi0 hi1] per axis, refs in float4 3
      const float4 x = __ldg(nd), y = __ldg(nd + 1), z = __ldg(nd + 2), r = __ldg(nd + 3);
      pnx[0] = ox ? x.z : x.x, pnx[1] = ox ? x.w : x.y, pfx[0] = ox ? x.x : x.z, pfx[1] = ox ? x.y : x.w;
      pny[0] = oy ? y.z : y.x, pny[1] = oy ? y.w : y.y, pfy[0] = oy ? y.x : y.z, pfy[1] = oy ? y.y : y.w;
      pnz[0] = oz ? z.z : z.x, pnz[1] = oz ? z.w : z.y, pfz[0] = oz ? z.x : z.z, pfz[1] = oz ? z.y : z.w;
      rc[0] = __float_as_uint(r.x);
      rc[1] = __float_as_uint(r.y);
    } else {
      // W / 4 float4 per plane; refs after the six planes
      constexpr int Q = W / 4;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const float4 a = __ldg(nd + (0 * 2 + ox) * Q + q), b = __ldg(nd + (0 * 2 + (ox ^ 1u)) * Q + q);
        const float4 c = __ldg(nd + (1 * 2 + oy) * Q + q), d = __ldg(nd + (1 * 2 + (oy ^ 1u)) * Q + q);
        const float4 e = __ldg(nd + (2 * 2 + oz) * Q + q), f = __ldg(nd + (2 * 2 + (oz ^ 1u)) * Q + q);
        const float4 r = __ldg(nd + 6 * Q + q);
        pnx[4 * q] = a.x, pnx[4 * q + 1] = a.y, pnx[4 * q + 2] = a.z, pnx[4 * q + 3] = a.w;
        pfx[4 * q] = b.x, pfx[4 * q + 1] = b.y, pfx[4 * q + 2] = b.z, pfx[4 * q + 3] = b.w;
        pny[4 * q] = c.x, pny[4 * q + 1] = c.y, pny[4 * q + 2] = c.z, pny[4 * q + 3] = c.w;
        pfy[4 * q] = d.x, pfy[4 * q + 1] = d.y, pfy[4 * q + 2] = d.z, pfy[4 * q + 3] = d.w;
        pnz[4 * q] = e.x, pnz[4 * q + 1] = e.y, pnz[4 * q + 2] = e.z, pnz[4 * q + 3] = e.w;
        pfz[4 * q] = f.x, pfz[4 * q + 1] = f.y, pfz[4 * q + 2] = f.z, pfz[4 * q + 3] = f.w;
        rc[4 * q] = __float_as_uint(r.x), rc[4 * q + 1] = __float_as_uint(r.y);
        rc[4 * q + 2] = __float_as_uint(r.z), rc[4 * q + 3] = __float_as_uint(r.w);
      }
    }
  }
};

// ascending (t, ref) by a sorting network: 1, 5 or 19 compare-exchanges
template <int W>
__device__ __forceinline__ void sort_children(float (&tc)[W], uint32_t (&rc)[W]) {
#define J3DG_CX(i, j)    \
  if (tc[j] < tc[i]) {   \
    float tt = tc[i];    \
    tc[i] = tc[j];       \
    tc[j] = tt;          \
    uint32_t rr = rc[i]; \
    rc[i] = rc[j];       \
    rc[j] = rr;          \
  }
  if constexpr (W == 2) {
    J3DG_CX(0, 1)
  } else if constexpr (W == 4) {
    J3DG_CX(0, 1) J3DG_CX(2, 3) J3DG_CX(0, 2) J3DG_CX(1, 3) J3DG_CX(1, 2)
  } else {
    J3DG_CX(0, 2) J3DG_CX(1, 3) J3DG_CX(4, 6) J3DG_CX(5, 7)
    J3DG_CX(0, 4) J3DG_CX(1, 5) J3DG_CX(2, 6) J3DG_CX(3, 7)
    J3DG_CX(0, 1) J3DG_CX(2, 3) J3DG_CX(4, 5) J3DG_CX(6, 7)
    J3DG_CX(2, 4) J3DG_CX(3, 5)
    J3DG_CX(1, 4) J3DG_CX(3, 6)
    J3DG_CX(1, 2) J3DG_CX(3, 4) J3DG_CX(5, 6)
  }
#undef J3DG_CX
}

template <int N, bool TOP = false, int W = 4>
struct TracerT {
#if J3DG_COLD_SMEM & 1
  // world ray: read only when an object's walk starts, kept in shared memory
  __device__ __forceinline__ float& wr(int k) { return ColdSlots<N>::ray()[k * ColdSlots<N>::S + threadIdx.x]; }
#else
  float wr_[6];  // world ray
  __device__ __forceinline__ float& wr(int k) { return wr_[k]; }
#endif
  bool any;                             // stop at the first accepted triangle
  Ray r;                                // object-space ray of object `inst` (world ray in the top level)
  BestT<N> b;
  const float4* nodes;
  const float4* tris;
  uint32_t n_nodes, nt;
  uint32_t cur;
  int sp;
  uint32_t inst;                        // kTopInst while in the top level
  uint32_t budget;

  __device__ __forceinline__ void start_object(const DevInst* __restrict__ insts) {
    const DevInst& I = insts[inst];
    if (I.width != (uint32_t)W) {  // a tree of another width: walk nothing (the host never launches that)
      nodes = nullptr;
      n_nodes = 0;
      cur = J3DG_EMPTY_REF;
      budget = 0;
      return;
    }
    float4 o = mat_vec(I.inv, wr(0), wr(1), wr(2), 1.f);
    float4 d = mat_vec(I.inv, wr(3), wr(4), wr(5), 0.f);
    r = make_ray(o.x, o.y, o.z, d.x, d.y, d.z, r.t_near, I.scale);
    nodes = I.nodes;
    tris = I.tris;
    n_nodes = I.n_nodes;
    nt = I.nt;
    cur = I.root_ref;
    budget = n_nodes + 1;
  }

  // the top level with the world ray; its slab test is padded by
  // (max|origin| + pad_scale) 2^-12 so that it never culls an object that
  // holds an object-space hit (toplevel.cpp)
  __device__ __forceinline__ void start_top(const DevInst* __restrict__ insts, uint32_t bud) {
    const DevTop& H = top_of(insts);
    const float ox = wr(0), oy = wr(1), oz = wr(2);
    const float mo = fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz));
    r = make_ray_pad(ox, oy, oz, wr(3), wr(4), wr(5), r.t_near, fm(fa(mo, H.pad_scale), 0x1p-12f));
    nodes = H.nodes;
    tris = nullptr;
    n_nodes = H.n_nodes;
    nt = H.n_inst;
    inst = kTopInst;
    budget = bud;
  }

  // Returns true if the ray is already finished (no objects).
  __device__ __forceinline__ bool begin(const DevInst* __restrict__ insts, uint32_t n_inst, float ox, float oy,
                                        float oz, float dx, float dy, float dz, float t_near, float t_far,
                                        bool any_hit) {
    any = any_hit;
    wr(0) = ox;
    wr(1) = oy;
    wr(2) = oz;
    wr(3) = dx;
    wr(4) = dy;
    wr(5) = dz;
    r.t_near = t_near;
    b.t = t_far;
    b.found = false;
    b.inst() = b.tri() = 0;
    b.u() = b.v() = 0.f;
    b.slot() = 0;
    sp = 0;
    if (n_inst == 0) return true;
    if (TOP) {
      const DevTop& H = top_of(insts);
      start_top(insts, H.n_nodes + 1);
      cur = H.root;
    } else {
      inst = 0;
      start_object(insts);
    }
    return false;
  }

  // stack: the caller's per-thread traversal stack of (ref, entry t bits)
  // pairs, one 8-byte access per push or pop (kept out of the struct so
  // that its scalar state can stay in registers)
  __device__ __forceinline__ bool run(const DevInst* __restrict__ insts, uint32_t n_inst, int iters,
                                      uint32_t* status, uint32_t& visits, uint32_t& tests,
                                      uint2* __restrict__ stack) {
#pragma unroll 1
    for (int it = 0; it < iters; ++it)
      if (step(insts, n_inst, status, visits, tests, stack)) return true;
    return false;
  }

  // One traversal step: a pop, a leaf (its triangles, or with TOP an
  // object entered) or a node. Returns true when the ray is finished.
  __device__ __forceinline__ bool step(const DevInst* __restrict__ insts, uint32_t n_inst, uint32_t* status,
                                       uint32_t& visits, uint32_t& tests, uint2* __restrict__ stack) {
    {
      if (cur == J3DG_EMPTY_REF) {
        bool got = false;
        while (sp > 0) {
          --sp;
          const uint2 e = stack[sp];
          if (TOP && e.x == kPopTop) {  // the object is done: back to the top level
            start_top(insts, e.y);
            continue;
          }
          if (__uint_as_float(e.y) <= b.t) {
            cur = e.x;
            got = true;
            break;
          }
        }
        if (!got) {
          if (TOP) return true;
          if (++inst >= n_inst) return true;
          start_object(insts);
          return false;
        }
      }
      if (cur & J3DG_LEAF_BIT) {
        const uint32_t first = (cur & 0x7fffffffu) >> 3, cnt = (cur & 7u) + 1u;
        if (first + cnt > nt) {
          atomicOr(status, J3DG_DEV_BAD_INDEX);
          return true;
        }
        if (TOP && inst == kTopInst) {
          // a top-level leaf: walk its object, then come back
          if (cnt != 1u || sp + 1 > J3DG_STACK) {
            atomicOr(status, cnt != 1u ? J3DG_DEV_BAD_INDEX : J3DG_DEV_STACK_OVERFLOW);
            return true;
          }
          stack[sp] = make_uint2(kPopTop, budget);
          ++sp;
          inst = first;
          start_object(insts);
          return false;
        }
#pragma unroll 1
        for (uint32_t k = 0; k < cnt; ++k) {
          ++tests;
          if (tri_test(r, tris, first + k, inst, b, any) && any) return true;
        }
        cur = J3DG_EMPTY_REF;
        return false;
      }
      if (budget-- == 0) {
        atomicOr(status, J3DG_DEV_VISIT_CAP);
        return true;
      }
      if (cur >= n_nodes) {
        atomicOr(status, J3DG_DEV_BAD_INDEX);
        return true;
      }
      ++visits;
      const float4* nd = nodes + J3DG_NODE_F4(W) * (size_t)cur;
      // near / far planes by the ray's octant: the same values slab() selects,
      // picked by the load offsets instead of per-child selects
      NodeLoad<W> L;
      L.load(nd, r.neg);
      float tc[W];
      uint32_t rc[W];
#pragma unroll
      for (int c = 0; c < W; ++c) {
        rc[c] = L.rc[c];
        // enter = max(tx, ty, tz, t_near), exit = min(tx, ty, tz, t_best)
        const float a = max3f(__fmaf_rn(L.pnx[c], r.ix, r.nnx), __fmaf_rn(L.pny[c], r.iy, r.nny),
                              fmaxf(__fmaf_rn(L.pnz[c], r.iz, r.nnz), r.t_near));
        const float e = min3f(__fmaf_rn(L.pfx[c], r.ix, r.nfx), __fmaf_rn(L.pfy[c], r.iy, r.nfy),
                              fminf(__fmaf_rn(L.pfz[c], r.iz, r.nfz), b.t));
        bool hit = (rc[c] != J3DG_EMPTY_REF) && (a <= e);
        tc[c] = hit ? a : __int_as_float(0x7f800000);
        if (!hit) rc[c] = J3DG_EMPTY_REF;
      }
      sort_children<W>(tc, rc);
      if (sp + (W - 1) > J3DG_STACK) {
        atomicOr(status, J3DG_DEV_STACK_OVERFLOW);
        return true;
      }
#pragma unroll
      for (int c = W - 1; c >= 1; --c)
        if (rc[c] != J3DG_EMPTY_REF) {
          stack[sp] = make_uint2(rc[c], __float_as_uint(tc[c]));
          ++sp;
        }
      cur = rc[0];
#if J3DG_PREFETCH
      // the next step starts with this child: its line is requested now, so
      // the fetch runs while the warp finishes the other lanes' branches
      // (not in the top level, whose leaves are objects, not triangles)
      if (cur != J3DG_EMPTY_REF && !(TOP && inst == kTopInst)) {
        const bool leaf = (cur & J3DG_LEAF_BIT) != 0;
        const uint32_t first = (cur & 0x7fffffffu) >> 3;
        if (leaf ? first + (cur & 7u) + 1u <= nt : cur < n_nodes) {  // the checks the next step makes
          const float4* line = leaf ? tris + 3 * (size_t)first : nodes + J3DG_NODE_F4(W) * (size_t)cur;
          asm volatile("prefetch.global.L1 [%0];" ::"l"(line));
        }
      }
#endif
    }
    return false;
  }
};

// Persistent warps with per-lane refill (Aila and Laine 2009, "dynamic
// fetch"): every lane whose ray finished takes the next work item; the warp
// fetches for all such lanes with one atomic. Src supplies count(), begin()
// (returns false when the item needs no tracing and was handled) and
// finish(); ITERS node/leaf steps run between refills.
// N: the kernel's block size.
template <int ITERS, int N, bool TOP, int W, class Src>
__device__ __forceinline__ void persistent_trace(Src& src, const DevInst* __restrict__ insts, uint32_t n_inst,
                                                 uint32_t* counter, uint32_t* status,
                                                 unsigned long long* counters) {
  TracerT<N, TOP, W> T;
  uint2 stack[J3DG_STACK];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t n = src.count();
  int64_t idx = -1;
  bool exhausted = false;
  uint32_t visits = 0, tests = 0;
#pragma unroll 1
  for (;;) {
    const bool need = idx < 0 && !exhausted;
    const uint32_t m = __ballot_sync(0xffffffffu, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      uint32_t base = 0;
      if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const uint32_t my = base + __popc(m & ((1u << lane) - 1u));
        if (my < n) {
          idx = my;
          if (!src.begin(T, insts, n_inst, my)) idx = -1;  // handled without tracing
        } else {
          exhausted = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, idx < 0 && exhausted)) break;
    if (idx >= 0 && T.run(insts, n_inst, ITERS, status, visits, tests, stack)) {
      src.finish(T, (uint32_t)idx);
      idx = -1;
    }
  }
  if (counters) {
    atomicAdd(counters + 0, (unsigned long long)visits);
    atomicAdd(counters + 1, (unsigned long long)tests);
  }
}

}  // namespace j3dg
