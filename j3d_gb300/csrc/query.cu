// query.cu -- all-hits ray queries and the voxel grid built from them.
//
// k_find_all replaces jtk's find_all_triangles (called at vox.cpp:333): every
// accepted triangle along the ray with t < t_far, kept sorted by (t, id) in
// the caller's per-ray buffer (the smallest `cap` when there are more).
// k_voxelize replaces the grid part of write_vox (vox.cpp:284-380): three
// axis-aligned sweeps of rays, each hit's voxel set to its colour index. The
// reference writes from parallel threads; here the order is fixed: sweep,
// then ray (d1 major), then hit (t, id) — the last write of a voxel wins,
// which an atomicMax over (ray order << 8 | colour) reproduces on the GPU.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include <string>

#include "device_common.cuh"
#include "query.cuh"

namespace j3dg {

// block size of the query kernels (their launch bounds; the per-thread
// shared slots of the hit record are sized by it)
static const int kQueryThreads = 128;

// Inserts (t, id, u, v) into the sorted buffer h[0..n) of capacity cap.
// `extra` goes to two_level_index (the object, or a leaf slot internally).
__device__ __forceinline__ void insert_sorted(j3dg_hit* h, uint32_t& n, uint32_t cap, float t, uint32_t id, float u,
                                              float v, uint32_t extra) {
  uint32_t pos = n < cap ? n : cap;
  if (n >= cap) {
    const j3dg_hit& last = h[cap - 1];
    if (!(t < last.distance || (t == last.distance && id < last.object_id))) {
      ++n;
      return;
    }
    pos = cap - 1;
  }
  while (pos > 0 && (t < h[pos - 1].distance || (t == h[pos - 1].distance && id < h[pos - 1].object_id))) {
    if (pos < cap) h[pos] = h[pos - 1];
    --pos;
  }
  j3dg_hit x;
  x.found = 1u;
  x.distance = t;
  x.u = u;
  x.v = v;
  x.object_id = id;
  x.two_level_index = extra;
  h[pos] = x;
  ++n;
}

// Visits every leaf whose slab interval meets [t_near, t_far]; calls
// on_hit(slot, t, u, v) for each accepted triangle. Returns false on a status.
template <class F>
__device__ bool all_hits(const DevInst& I, const Ray& r, float t_far, uint32_t* status, F on_hit) {
  uint32_t stack[J3DG_STACK];
  int sp = 0;
  uint32_t cur = I.root_ref;
  uint32_t budget = I.n_nodes + 1;
  for (;;) {
    if (cur != J3DG_EMPTY_REF) {
      if (cur & J3DG_LEAF_BIT) {
        const uint32_t first = (cur & 0x7fffffffu) >> 3, cnt = (cur & 7u) + 1u;
        if (first + cnt > I.nt) {
          atomicOr(status, J3DG_DEV_BAD_INDEX);
          return false;
        }
        for (uint32_t k = 0; k < cnt; ++k) {
          BestT<kQueryThreads> b;
          b.t = t_far;
          b.found = false;
          if (tri_test(r, I.tris, first + k, 0u, b, true)) on_hit(first + k, b.t, b.u(), b.v());
        }
        cur = J3DG_EMPTY_REF;
      } else {
        if (budget-- == 0) {
          atomicOr(status, J3DG_DEV_VISIT_CAP);
          return false;
        }
        if (cur >= I.n_nodes) {
          atomicOr(status, J3DG_DEV_BAD_INDEX);
          return false;
        }
        const float4* N = I.nodes + 8 * (size_t)cur;
        const float4 lox = __ldg(N + 0), hix = __ldg(N + 1), loy = __ldg(N + 2), hiy = __ldg(N + 3);
        const float4 loz = __ldg(N + 4), hiz = __ldg(N + 5), chf = __ldg(N + 6);
        const uint32_t rc[4] = {__float_as_uint(chf.x), __float_as_uint(chf.y), __float_as_uint(chf.z),
                                __float_as_uint(chf.w)};
        const float lx[4] = {lox.x, lox.y, lox.z, lox.w}, hx[4] = {hix.x, hix.y, hix.z, hix.w};
        const float ly[4] = {loy.x, loy.y, loy.z, loy.w}, hy[4] = {hiy.x, hiy.y, hiy.z, hiy.w};
        const float lz[4] = {loz.x, loz.y, loz.z, loz.w}, hz[4] = {hiz.x, hiz.y, hiz.z, hiz.w};
        cur = J3DG_EMPTY_REF;
        for (int c = 0; c < 4; ++c) {
          if (rc[c] == J3DG_EMPTY_REF) continue;
          float tn, tf;
          slab(r, lx[c], ly[c], lz[c], hx[c], hy[c], hz[c], tn, tf);
          if (!(fmaxf(tn, r.t_near) <= fminf(tf, t_far))) continue;
          if (sp >= J3DG_STACK) {
            atomicOr(status, J3DG_DEV_STACK_OVERFLOW);
            return false;
          }
          stack[sp++] = rc[c];
        }
      }
    }
    if (sp == 0) return true;
    cur = stack[--sp];
  }
}

__global__ void __launch_bounds__(kQueryThreads) k_find_all(const DevInst* __restrict__ inst, const j3dg_ray* __restrict__ rays, uint32_t n,
                           uint32_t cap, j3dg_hit* __restrict__ hits, uint32_t* __restrict__ counts,
                           uint32_t* status) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const DevInst& I = inst[0];
  const float* f = reinterpret_cast<const float*>(rays + i);
  const Ray r = make_ray(f[0], f[1], f[2], f[4], f[5], f[6], f[8], I.scale);
  j3dg_hit* h = hits + (size_t)i * cap;
  uint32_t cnt = 0;
  all_hits(I, r, f[9], status, [&](uint32_t slot, float t, float u, float v) {
    const uint32_t id = __float_as_uint(__ldg(I.tris + 3 * (size_t)slot).w);
    if (cap)
      insert_sorted(h, cnt, cap, t, id, u, v, 0u);
    else
      ++cnt;
  });
  counts[i] = cnt;
}

// vox.cpp:154-173
__device__ __forceinline__ uint32_t color_to_index(uint32_t r, uint32_t g, uint32_t b) {
  r = r < 16 ? 0 : r - 16;
  g = g < 16 ? 0 : g - 16;
  b = b < 32 ? 0 : b - 32;
  const uint32_t ret = ((r >> 5) << 5) | ((g >> 5) << 2) | (b >> 6);
  return ret == 0 ? 1u : ret;
}

__device__ __forceinline__ uint32_t vox_cell(float p, float lo, float hi, uint32_t dim) {
  const float x = __fdiv_rn(fs(p, lo), fs(hi, lo));
  const float f = fm(x, (float)dim);
  uint32_t X = f > 0.f ? (uint32_t)f : 0u;
  return X >= dim ? dim - 1 : X;
}

static const uint32_t kVoxHits = 64;

__global__ void __launch_bounds__(kQueryThreads) k_voxelize(const DevInst* __restrict__ inst, VoxParams V, uint32_t* __restrict__ keys,
                           uint32_t* status) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= V.rays_total) return;
  const DevInst& I = inst[0];
  // which sweep and which ray of it (the rays of sweep dd are d1-major)
  uint32_t dd = 0, local = g;
  while (dd < 2 && local >= V.rays[dd]) {
    local -= V.rays[dd];
    ++dd;
  }
  const uint32_t a1 = (dd + 1) % 3, a2 = (dd + 2) % 3;
  const uint32_t d1 = local / V.dim[a2], d2 = local % V.dim[a2];
  // vox.cpp:309-330
  float st[3];
  st[dd] = V.mn[dd];
  st[a1] = fa(fm(__fdiv_rn(fa((float)d1, 0.5f), (float)V.dim[a1]), fs(V.mx[a1], V.mn[a1])), V.mn[a1]);
  st[a2] = fa(fm(__fdiv_rn(fa((float)d2, 0.5f), (float)V.dim[a2]), fs(V.mx[a2], V.mn[a2])), V.mn[a2]);
  float dir[3] = {0.f, 0.f, 0.f};
  dir[dd] = dd == 2 ? 2.f : 1.f;
  const Ray r = make_ray(st[0], st[1], st[2], dir[0], dir[1], dir[2], 0.f, I.scale);
  j3dg_hit h[kVoxHits];
  uint32_t cnt = 0;
  const bool ok = all_hits(I, r, FLT_MAX, status, [&](uint32_t slot, float t, float u, float v) {
    const uint32_t id = __float_as_uint(__ldg(I.tris + 3 * (size_t)slot).w);
    insert_sorted(h, cnt, kVoxHits, t, id, u, v, slot);
  });
  if (!ok) return;
  if (cnt > kVoxHits) {
    atomicOr(status, J3DG_DEV_HIT_OVERFLOW);
    return;
  }
  const uint32_t order = g + 1;  // sweeps in order, then rays d1-major
  uint32_t cell[kVoxHits], color[kVoxHits];
  for (uint32_t i = 0; i < cnt; ++i) {
    const uint32_t id = h[i].object_id, slot = h[i].two_level_index;
    const uint32_t* T = I.index + 3 * (size_t)id;
    // the triangle's vertices, as stored in leaf order (the caller's values)
    const float4 A4 = __ldg(I.tris + 3 * (size_t)slot), B4 = __ldg(I.tris + 3 * (size_t)slot + 1),
                 C4 = __ldg(I.tris + 3 * (size_t)slot + 2);
    const float A[3] = {A4.x, A4.y, A4.z}, B[3] = {B4.x, B4.y, B4.z}, C[3] = {C4.x, C4.y, C4.z};
    const float u = h[i].u, v = h[i].v, wgt = fs(fs(1.f, u), v);
    float pos[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) pos[k] = fa(fa(fm(A[k], wgt), fm(u, B[k])), fm(v, C[k]));
    float clr[3] = {1.f, 1.f, 1.f};
    if (V.use_texture) {
      const float* uv = I.uv + 6 * (size_t)id;
      float c0 = fa(fa(fm(wgt, uv[0]), fm(u, uv[2])), fm(v, uv[4]));
      float c1 = fa(fa(fm(wgt, uv[1]), fm(u, uv[3])), fm(v, uv[5]));
      c0 = fmaxf(fminf(c0, 1.f), 0.f);
      c1 = fmaxf(fminf(c1, 1.f), 0.f);
      const int x = (int)fm(c0, (float)(I.tex_w - 1)), y = (int)fm(c1, (float)(I.tex_h - 1));
      const uint32_t c = __ldg(I.tex + (size_t)y * I.tex_w + x);
      clr[0] = __fdiv_rn((float)(c & 255u), 255.f);
      clr[1] = __fdiv_rn((float)((c >> 8) & 255u), 255.f);
      clr[2] = __fdiv_rn((float)((c >> 16) & 255u), 255.f);
    } else if (V.use_colors) {
      const float* c0 = I.colors + 3 * (size_t)T[0];
      const float* c1 = I.colors + 3 * (size_t)T[1];
      const float* c2 = I.colors + 3 * (size_t)T[2];
#pragma unroll
      for (int k = 0; k < 3; ++k) clr[k] = fa(fa(fm(c0[k], wgt), fm(u, c1[k])), fm(v, c2[k]));
    }
    const uint32_t X = vox_cell(pos[0], V.mn[0], V.mx[0], V.dim[0]);
    const uint32_t Y = vox_cell(pos[1], V.mn[1], V.mx[1], V.dim[1]);
    const uint32_t Z = vox_cell(pos[2], V.mn[2], V.mx[2], V.dim[2]);
    cell[i] = X + (Y + Z * V.dim[1]) * V.dim[0];  // vox.cpp:123-127
    color[i] = color_to_index((uint8_t)fm(clr[0], 255.f), (uint8_t)fm(clr[1], 255.f), (uint8_t)fm(clr[2], 255.f));
  }
  for (uint32_t i = 0; i < cnt; ++i) {
    bool later = false;  // a later hit of this ray writes the same voxel
    for (uint32_t j = i + 1; j < cnt; ++j) later |= cell[j] == cell[i];
    if (!later) atomicMax(keys + cell[i], (order << 8) | color[i]);
  }
}

__global__ void k_keys_to_voxels(const uint32_t* __restrict__ keys, uint8_t* __restrict__ out, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (uint8_t)(keys[i] & 0xffu);
}

cudaError_t launch_find_all(const DevInst* inst, const j3dg_ray* rays, uint32_t n, uint32_t cap, j3dg_hit* hits,
                            uint32_t* counts, uint32_t* status, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_find_all<<<(n + kQueryThreads - 1) / kQueryThreads, kQueryThreads, 0, st>>>(inst, rays, n, cap, hits, counts, status);
  return cudaGetLastError();
}

cudaError_t launch_voxelize(const DevInst* inst, const VoxParams& V, uint32_t* keys, uint8_t* out,
                            uint32_t* status, cudaStream_t st) {
  const size_t total = (size_t)V.dim[0] * V.dim[1] * V.dim[2];
  cudaError_t e = cudaMemsetAsync(keys, 0, sizeof(uint32_t) * total, st);
  if (e != cudaSuccess) return e;
  if (V.rays_total) k_voxelize<<<(V.rays_total + kQueryThreads - 1) / kQueryThreads, kQueryThreads, 0, st>>>(inst, V, keys, status);
  k_keys_to_voxels<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(keys, out, total);
  return cudaGetLastError();
}

}  // namespace j3dg

namespace j3dg {

// Counts G-buffer records with a hit (object_id != ~0) and with the shadow bit.
__global__ void k_count_hits(const j3dg_pixel* __restrict__ G, size_t n, unsigned long long* out) {
  unsigned long long hits = 0, shadowed = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t id = G[i].object_id;
    hits += id != 0xffffffffu;
    shadowed += id != 0xffffffffu && (G[i].mark & 1u);
  }
  for (int o = 16; o > 0; o >>= 1) {
    hits += __shfl_xor_sync(0xffffffffu, hits, o);
    shadowed += __shfl_xor_sync(0xffffffffu, shadowed, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, hits);
    atomicAdd(out + 1, shadowed);
  }
}

cudaError_t launch_count_hits(const j3dg_pixel* G, size_t n, unsigned long long* out, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), st);
  if (e != cudaSuccess || n == 0) return e;
  k_count_hits<<<256, 256, 0, st>>>(G, n, out);
  return cudaGetLastError();
}

}  // namespace j3dg

// --------------------------------------------- voxel grid without allocation
//
// Scratch for j3dg_voxelize_noalloc, for callers that must not allocate
// device memory once they are running. It lives in this file-scope array,
// which every GPU that loads the library holds until the process exits:
// per voxel a 4-byte key, plus 1 byte of staging used when the caller's
// output is in host memory. Host code cannot use the array's name as a
// device address (it names a host-side stand-in); voxel_scratch() looks the
// real address up with cudaGetSymbolAddress on the current device. Contexts
// call it once, when they are created, and keep the address for their life,
// so the module holding the array is loaded then and a context created after
// a device reset looks the address up again.
namespace j3dg {

static __device__ __align__(256) uint32_t g_voxel_scratch[J3DG_NOALLOC_MAX_VOXELS + J3DG_NOALLOC_MAX_VOXELS / 4];

int voxel_scratch(uint32_t** keys, uint8_t** staging, std::string& err) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_voxel_scratch);
  if (e != cudaSuccess || p == nullptr) {
    cudaGetLastError();
    err = std::string("voxelize_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
    return J3DG_ERR_CUDA;
  }
  *keys = static_cast<uint32_t*>(p);
  *staging = reinterpret_cast<uint8_t*>(static_cast<uint32_t*>(p) + J3DG_NOALLOC_MAX_VOXELS);
  return J3DG_OK;
}

}  // namespace j3dg
