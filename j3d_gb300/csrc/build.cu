// build.cu -- GPU construction of the 4-wide BVH over an indexed triangle mesh.
//
// Replaces, in scene.cpp:20-23 (add_object), compute_triangle_normals,
// compute_bb (mesh.cpp:39-58) and `new jtk::qbvh(triangles, vertices)`.
//
// Pipeline (all on the context stream):
//   1. vertex bbox: two-pass min/max reduction (exact)
//   2. per triangle: normal (fixed fp32 order), AABB centroid -> 48-bit Morton
//      code over the vertex bbox
//   3. LSD radix sort of (Morton, triangle id), 8-bit digits, stable
//   4. leaf-ordered triangle array: 3 float4 per triangle (v0.w = id bits)
//   5. binary tree: by default binned-SAH splits top-down down to ranges of
//      at most J3DG_SAH_TOP triangles (section 5c), then PLOC clustering
//      within each range (section 5b); with J3DG_BUILD_LBVH the LBVH,
//      bottom-up in one pass
//      (Apetrei 2014, "Fast and Simple Agglomerative LBVH Construction"),
//      with a strict total order on the split keys (xor of neighbouring
//      codes, then i ^ (i+1), then i)
//   6. collapse to 4-wide nodes level by level: slots and leaves chosen by
//      the SAH cost programme of section 6b (LBVH: open the largest-area
//      child until four children, subtrees of <= leaf_size triangles become
//      leaves); then the wide nodes are numbered depth-first (section 7).
// Child boxes are exact unions of triangle boxes, which the traversal's
// topology-independence argument requires.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "internal.h"

namespace j3dg {

static const int kMortonBitsPerAxis = 16;
static const int kRadixPasses = (3 * kMortonBitsPerAxis + 7) / 8;

// ------------------------------------------------------------- 1. bbox ----

__global__ void k_bbox_partial(const float* __restrict__ V, uint32_t nv, float* __restrict__ part) {
  float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float x = V[3 * (size_t)i + k];
      mn[k] = fminf(mn[k], x);
      mx[k] = fmaxf(mx[k], x);
    }
  }
  __shared__ float s[6][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
      mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
    }
  }
  if (lane == 0)
    for (int k = 0; k < 3; ++k) {
      s[k][warp] = mn[k];
      s[3 + k][warp] = mx[k];
    }
  __syncthreads();
  if (threadIdx.x < 6) {
    float v = s[threadIdx.x][0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      v = threadIdx.x < 3 ? fminf(v, s[threadIdx.x][w]) : fmaxf(v, s[threadIdx.x][w]);
    part[6 * blockIdx.x + threadIdx.x] = v;
  }
}

__global__ void k_bbox_final(const float* __restrict__ part, int n, float* __restrict__ out) {
  if (threadIdx.x < 6) {
    float v = part[threadIdx.x];
    for (int b = 1; b < n; ++b) v = threadIdx.x < 3 ? fminf(v, part[6 * b + threadIdx.x]) : fmaxf(v, part[6 * b + threadIdx.x]);
    out[threadIdx.x] = v;
  }
}

// ------------------------------------------------ 2. normals and Morton ----

// spreads the low 21 bits of x to every third bit (Morton interleave)
__device__ __forceinline__ uint64_t spread3(uint32_t x) {
  uint64_t v = x & 0x1fffffu;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

__global__ void k_tri_prep(const float* __restrict__ V, uint32_t nv, const uint32_t* __restrict__ T, uint32_t nt,
                           const float* __restrict__ bb, float4* __restrict__ normals, uint64_t* __restrict__ keys,
                           uint32_t* __restrict__ vals, uint32_t* status) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  uint32_t a = T[3 * (size_t)i], b = T[3 * (size_t)i + 1], c = T[3 * (size_t)i + 2];
  if (a >= nv || b >= nv || c >= nv) {
    atomicOr(status, J3DG_DEV_BAD_INDEX);
    a = b = c = 0;
  }
  const float* A = V + 3 * (size_t)a;
  const float* B = V + 3 * (size_t)b;
  const float* C = V + 3 * (size_t)c;
  // jtk compute_triangle_normals: normalize(cross(V1 - V0, V2 - V0))
  float e1x = fs(B[0], A[0]), e1y = fs(B[1], A[1]), e1z = fs(B[2], A[2]);
  float e2x = fs(C[0], A[0]), e2y = fs(C[1], A[1]), e2z = fs(C[2], A[2]);
  float nx = fs(fm(e1y, e2z), fm(e1z, e2y));
  float ny = fs(fm(e1z, e2x), fm(e1x, e2z));
  float nz = fs(fm(e1x, e2y), fm(e1y, e2x));
  float len = __fsqrt_rn(dot3(nx, ny, nz, nx, ny, nz));
  if (len > 0.f) {
    nx = __fdiv_rn(nx, len);
    ny = __fdiv_rn(ny, len);
    nz = __fdiv_rn(nz, len);
  }
  normals[i] = make_float4(nx, ny, nz, 0.f);
  // Morton code of the AABB centroid over the vertex bbox
  const float scale = (float)(1u << kMortonBitsPerAxis);
  uint32_t q[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float lo = fminf(fminf(A[k], B[k]), C[k]), hi = fmaxf(fmaxf(A[k], B[k]), C[k]);
    float cen = (lo + hi) * 0.5f;
    float ext = bb[3 + k] - bb[k];
    float f = ext > 0.f ? (cen - bb[k]) / ext * scale : 0.f;
    f = fminf(fmaxf(f, 0.f), scale - 1.f);
    q[k] = (uint32_t)f;
  }
  keys[i] = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
  vals[i] = i;
}

// ------------------------------------------------------ 3. radix sort ----

static const int kSortThreads = 256;
static const int kSortItems = 8;  // tiles of 2048 keys: the scatter's shared-memory reorder fits 34 KB
static const int kSortTile = kSortThreads * kSortItems;

__global__ void k_radix_hist(const uint64_t* __restrict__ keys, uint32_t n, int shift, uint32_t num_tiles,
                             uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  size_t base = (size_t)blockIdx.x * kSortTile;
#pragma unroll 4
  for (int j = 0; j < kSortItems; ++j) {
    size_t idx = base + (size_t)j * kSortThreads + threadIdx.x;
    if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * num_tiles + blockIdx.x] = h[threadIdx.x];
}

// exclusive scan helpers (three phases over chunks of 1024 elements):
// k_scan_chunks scans each chunk (256 threads x 4 elements: a sequential
// scan of the thread's uint4, a shuffle scan of the warp's totals, the
// eight warp totals through shared memory) and writes the chunk total,
// k_scan_sums scans the chunk totals, k_scan_add adds them back. in and out
// are 16-byte aligned (device allocations); elements past n read as 0 and
// are not written.
__global__ void __launch_bounds__(256) k_scan_chunks(const uint32_t* in, uint32_t* out, uint32_t n,
                                                     uint32_t* __restrict__ sums) {
  __shared__ uint32_t wsum[8];
  const uint32_t base = blockIdx.x * 1024u + threadIdx.x * 4u;
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (base + 3 < n) {
    v = *reinterpret_cast<const uint4*>(in + base);
  } else {
    if (base < n) v.x = in[base];
    if (base + 1 < n) v.y = in[base + 1];
    if (base + 2 < n) v.z = in[base + 2];
  }
  const uint32_t tot = v.x + v.y + v.z + v.w;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t inc = tot;  // inclusive scan of the thread totals within the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= (uint32_t)o) inc += y;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  uint32_t woff = 0, all = 0;
#pragma unroll
  for (uint32_t w = 0; w < 8; ++w) {
    const uint32_t x = wsum[w];
    woff += w < warp ? x : 0u;
    all += x;
  }
  const uint32_t e = woff + inc - tot;  // exclusive prefix of this thread's first element
  const uint4 o4 = make_uint4(e, e + v.x, e + v.x + v.y, e + v.x + v.y + v.z);
  if (base + 3 < n) {
    *reinterpret_cast<uint4*>(out + base) = o4;
  } else {
    if (base < n) out[base] = o4.x;
    if (base + 1 < n) out[base + 1] = o4.y;
    if (base + 2 < n) out[base + 2] = o4.z;
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = all;
}

__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t* __restrict__ sums_a, uint32_t* __restrict__ sums_b,
                                                    uint32_t n, uint32_t* __restrict__ totals,
                                                    const uint32_t* __restrict__ len_p = nullptr) {
  // len_p (if given): the scanned list's length in device memory; the chunk
  // totals to scan are then ceil(len / 1024)
  if (len_p) n = (*len_p + 1023u) / 1024u;
  // single block of 1024 threads, over one array of chunk totals (sums_b
  // null) or two: each thread sums a strip of consecutive chunk totals, the
  // strip sums are scanned by warp shuffles (within each warp, then the 32
  // warp totals by warp 0), and each thread rewrites its strip as exclusive
  // prefixes; totals (if not null) receives each array's grand total
  __shared__ uint32_t wtot[32];
  const uint32_t per = (n + 1023) / 1024;
  const uint32_t b = threadIdx.x * per, e = min(n, b + per);
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (int q = 0; q < 2; ++q) {
    uint32_t* sums = q ? sums_b : sums_a;
    if (!sums) break;  // uniform over the block
    uint32_t acc = 0;
    for (uint32_t i = b; i < e; ++i) acc += sums[i];
    uint32_t inc = acc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= (uint32_t)o) inc += y;
    }
    if (lane == 31) wtot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      const uint32_t x = wtot[lane];
      uint32_t xi = x;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, xi, o);
        if (lane >= (uint32_t)o) xi += y;
      }
      wtot[lane] = xi - x;
      if (lane == 31 && totals) totals[q] = xi;
    }
    __syncthreads();
    uint32_t run = wtot[warp] + inc - acc;
    for (uint32_t i = b; i < e; ++i) {
      const uint32_t x = sums[i];
      sums[i] = run;
      run += x;
    }
    __syncthreads();  // wtot is reused by the second array
  }
}

__global__ void __launch_bounds__(256) k_scan_add(uint32_t* __restrict__ out, uint32_t n,
                                                  const uint32_t* __restrict__ sums) {
  const uint32_t base = blockIdx.x * 1024u + threadIdx.x * 4u, add = sums[blockIdx.x];
  if (base + 3 < n) {
    uint4 v = *reinterpret_cast<const uint4*>(out + base);
    v.x += add;
    v.y += add;
    v.z += add;
    v.w += add;
    *reinterpret_cast<uint4*>(out + base) = v;
  } else {
    for (uint32_t k = base; k < n && k < base + 4u; ++k) out[k] += add;
  }
}

// One tile of kSortTile keys per block: each key's rank among the tile's
// keys of its digit comes from kSortItems rounds of 256 keys (warp
// match_any ranks, per-warp digit counts scanned across the warps, a
// running count per digit); the tile is then reordered by digit in shared
// memory (stable) and written out so that consecutive threads write
// consecutive positions of one digit's run (coalesced, instead of one
// scattered 8-byte write per key).
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const uint64_t* __restrict__ kin,
                                                                const uint32_t* __restrict__ vin,
                                                                uint64_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                                uint32_t n, int shift, uint32_t num_tiles,
                                                                const uint32_t* __restrict__ offsets,
                                                                const uint32_t* __restrict__ chunk_offsets,
                                                                uint32_t* status) {
  __shared__ uint32_t base[256];     // global position of the tile's first key of each digit
  __shared__ uint32_t run[256];      // keys of each digit in the tile's earlier rounds, then the digit's local start
  __shared__ uint32_t wc[kSortThreads / 32][257];
  __shared__ uint64_t sk[kSortTile];
  __shared__ uint32_t sv[kSortTile];
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  {
    // offsets: the digit histogram's scan within chunks of 1024 entries;
    // chunk_offsets: the scanned chunk totals
    const size_t h = (size_t)tid * num_tiles + blockIdx.x;
    base[tid] = offsets[h] + chunk_offsets[h >> 10];
  }
  run[tid] = 0;
  const size_t tile = (size_t)blockIdx.x * kSortTile;
  uint64_t key[kSortItems];
  uint32_t rnk[kSortItems];  // digit (low 9 bits: 256 = no key) and rank within the tile's digit
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    for (int w = 0; w < kSortThreads / 32; ++w) wc[w][tid] = 0;
    if (tid == 0)
      for (int w = 0; w < kSortThreads / 32; ++w) wc[w][256] = 0;
    __syncthreads();
    const size_t idx = tile + (size_t)j * kSortThreads + tid;
    const bool valid = idx < n;
    const uint64_t k = valid ? kin[idx] : 0;
    const uint32_t d = valid ? (uint32_t)((k >> shift) & 255u) : 256u;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    if (rank == 0) wc[warp][d] = __popc(peers);
    __syncthreads();
    uint32_t tot = 0;
    {
      uint32_t acc = 0;
      for (int w = 0; w < kSortThreads / 32; ++w) {
        const uint32_t c = wc[w][tid];
        wc[w][tid] = acc;
        acc += c;
      }
      tot = acc;
    }
    __syncthreads();
    key[j] = k;
    rnk[j] = d | ((valid ? run[d] + wc[warp][d] + rank : 0u) << 9);
    __syncthreads();
    run[tid] += tot;
  }
  __syncthreads();
  // the digits' starts within the tile: exclusive scan of the counts (run)
  {
    const uint32_t c = run[tid];
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) wc[0][warp] = incl;
    __syncthreads();
    uint32_t woff = 0;
    for (uint32_t w = 0; w < warp; ++w) woff += wc[0][w];
    __syncthreads();
    run[tid] = woff + incl - c;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kSortItems; ++j) {
    const uint32_t d = rnk[j] & 511u;
    if (d < 256u) {
      const uint32_t l = run[d] + (rnk[j] >> 9);
      sk[l] = key[j];
      sv[l] = vin[tile + (size_t)j * kSortThreads + tid];
    }
  }
  __syncthreads();
  const uint32_t tile_n = (uint32_t)min((size_t)kSortTile, (size_t)n - tile);
  for (uint32_t i = tid; i < tile_n; i += kSortThreads) {
    const uint64_t k = sk[i];
    const uint32_t d = (uint32_t)((k >> shift) & 255u);
    const uint32_t pos = base[d] + (i - run[d]);
    if (pos < n) {
      kout[pos] = k;
      vout[pos] = sv[i];
    } else {
      atomicOr(status, J3DG_DEV_BAD_INDEX);
    }
  }
}

// ----------------------------------------------- 4. leaf-ordered triangles ----

__global__ void k_soup(const float* __restrict__ V, const uint32_t* __restrict__ T, const uint32_t* __restrict__ order,
                       uint32_t nt, uint32_t nv, float4* __restrict__ tris, uint32_t* status) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  uint32_t id = order[i];
  if (id >= nt) {
    atomicOr(status, J3DG_DEV_BAD_INDEX);
    id = 0;
  }
  uint32_t a = T[3 * (size_t)id], b = T[3 * (size_t)id + 1], c = T[3 * (size_t)id + 2];
  if (a >= nv || b >= nv || c >= nv) a = b = c = 0;
  tris[3 * (size_t)i] = make_float4(V[3 * (size_t)a], V[3 * (size_t)a + 1], V[3 * (size_t)a + 2], __uint_as_float(id));
  tris[3 * (size_t)i + 1] = make_float4(V[3 * (size_t)b], V[3 * (size_t)b + 1], V[3 * (size_t)b + 2], 0.f);
  tris[3 * (size_t)i + 2] = make_float4(V[3 * (size_t)c], V[3 * (size_t)c + 1], V[3 * (size_t)c + 2], 0.f);
}

// ------------------------------------------------------------- 5. LBVH ----

struct BinNode {   // binary node n (split between sorted leaves n and n+1)
  float4 lo, hi;   // box (w unused)
};

__device__ __forceinline__ void leaf_box(const float4* __restrict__ tris, uint32_t i, float4& lo, float4& hi) {
  float4 a = tris[3 * (size_t)i], b = tris[3 * (size_t)i + 1], c = tris[3 * (size_t)i + 2];
  lo = make_float4(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y), fminf(fminf(a.z, b.z), c.z), 0.f);
  hi = make_float4(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y), fmaxf(fmaxf(a.z, b.z), c.z), 0.f);
}

// split order: smaller (xor, i ^ (i+1), i) merges first
__device__ __forceinline__ bool split_less(const uint64_t* __restrict__ k, uint32_t a, uint32_t b) {
  uint64_t xa = k[a] ^ k[a + 1], xb = k[b] ^ k[b + 1];
  if (xa != xb) return xa < xb;
  uint32_t sa = a ^ (a + 1), sb = b ^ (b + 1);
  if (sa != sb) return sa < sb;
  return a < b;
}

// child refs: bit 31 set = sorted leaf index, else binary node index
__global__ void k_lbvh(const uint64_t* __restrict__ keys, const float4* __restrict__ tris, uint32_t n,
                       uint2* __restrict__ child, BinNode* __restrict__ box, uint2* __restrict__ range,
                       uint32_t* __restrict__ other, uint32_t* __restrict__ root) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t l = i, r = i;
  uint32_t cur = 0x80000000u | i;
  float4 lo, hi;
  leaf_box(tris, i, lo, hi);
  for (;;) {
    uint32_t p, prev;
    bool as_left;
    if (l == 0 || (r != n - 1 && split_less(keys, r, l - 1))) {
      p = r;
      as_left = true;
      __stcg(&child[p].x, cur);
      __threadfence();
      prev = atomicExch(&other[p], l);
    } else {
      p = l - 1;
      as_left = false;
      __stcg(&child[p].y, cur);
      __threadfence();
      prev = atomicExch(&other[p], r);
    }
    if (prev == 0xffffffffu) return;  // first to arrive: the sibling finishes p
    __threadfence();
    if (as_left)
      r = prev;
    else
      l = prev;
    uint32_t sib = as_left ? __ldcg(&child[p].y) : __ldcg(&child[p].x);
    float4 slo, shi;
    if (sib & 0x80000000u) {
      leaf_box(tris, sib & 0x7fffffffu, slo, shi);
    } else {
      slo = __ldcg(&box[sib].lo);
      shi = __ldcg(&box[sib].hi);
    }
    lo = make_float4(fminf(lo.x, slo.x), fminf(lo.y, slo.y), fminf(lo.z, slo.z), 0.f);
    hi = make_float4(fmaxf(hi.x, shi.x), fmaxf(hi.y, shi.y), fmaxf(hi.z, shi.z), 0.f);
    __stcg(&box[p].lo, lo);
    __stcg(&box[p].hi, hi);
    __stcg(&range[p], make_uint2(l, r));
    cur = p;
    if (l == 0 && r == n - 1) {
      *root = p;
      return;
    }
  }
}

// --------------------------------------------------------- 6. collapse ----

struct CollapseItem {
  uint32_t bin;    // binary node index
  uint32_t wide;   // wide node index to fill
  uint32_t depth;
};

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
  float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
  return dx * dy + dy * dz + dz * dx;
}
__device__ __forceinline__ float half_area4(float4 lo, float4 hi) { return half_area(lo, hi); }

// One binary node of the LBVH's 4-wide collapse: it becomes wide node
// it.wide, whose slots are its children, the largest-area child opened until
// four slots are filled (or every slot is small enough to be a leaf); the
// slots that stay internal get wide nodes (n_wide) and are queued for the
// next level (n_out). bound: the wide array's and the queue's size; an index
// past it raises J3DG_DEV_BAD_INDEX and is not written.
__device__ __forceinline__ void collapse_one(const uint2* __restrict__ child, const BinNode* __restrict__ box,
                                             const uint2* __restrict__ range, const float4* __restrict__ tris,
                                             const CollapseItem it, CollapseItem* __restrict__ qout,
                                             uint32_t* __restrict__ n_out, uint32_t* __restrict__ n_wide,
                                             float4* __restrict__ wide, uint32_t bound, uint32_t leaf_size,
                                             uint32_t* __restrict__ max_depth, uint32_t* __restrict__ status) {
  if (it.wide >= bound) {
    atomicOr(status, J3DG_DEV_BAD_INDEX);
    return;
  }
  uint32_t ref[4];
  float4 lo[4], hi[4];
  uint32_t cnt[4];
  int m = 0;
  auto load = [&](uint32_t r, int s) {
    ref[s] = r;
    if (r & 0x80000000u) {
      leaf_box(tris, r & 0x7fffffffu, lo[s], hi[s]);
      cnt[s] = 1;
    } else {
      lo[s] = box[r].lo;
      hi[s] = box[r].hi;
      uint2 rg = range[r];
      cnt[s] = rg.y - rg.x + 1;
    }
  };
  uint2 c = child[it.bin];
  load(c.x, 0);
  load(c.y, 1);
  m = 2;
  while (m < 4) {
    int best = -1;
    float ba = -1.f;
    for (int s = 0; s < m; ++s)
      if (cnt[s] > leaf_size) {
        float a = half_area(lo[s], hi[s]);
        if (a > ba) {
          ba = a;
          best = s;
        }
      }
    if (best < 0) break;
    uint2 cc = child[ref[best]];
    load(cc.y, m);
    load(cc.x, best);
    ++m;
  }
  float4* W = wide + 8 * (size_t)it.wide;
  float v[6][4];
  uint32_t out_ref[4];
  for (int s = 0; s < 4; ++s) {
    if (s < m) {
      v[0][s] = lo[s].x;
      v[1][s] = hi[s].x;
      v[2][s] = lo[s].y;
      v[3][s] = hi[s].y;
      v[4][s] = lo[s].z;
      v[5][s] = hi[s].z;
      if (cnt[s] <= leaf_size) {
        uint32_t first = (ref[s] & 0x80000000u) ? (ref[s] & 0x7fffffffu) : range[ref[s]].x;
        out_ref[s] = J3DG_LEAF_BIT | (first << 3) | (cnt[s] - 1u);
      } else {
        const uint32_t w = atomicAdd(n_wide, 1u);
        const uint32_t q = atomicAdd(n_out, 1u);
        if (w < bound && q < bound) {
          qout[q] = CollapseItem{ref[s], w, it.depth + 1};
        } else {
          atomicOr(status, J3DG_DEV_BAD_INDEX);
        }
        out_ref[s] = w;
      }
    } else {
      v[0][s] = v[2][s] = v[4][s] = 3.4e38f;
      v[1][s] = v[3][s] = v[5][s] = -3.4e38f;
      out_ref[s] = J3DG_EMPTY_REF;
    }
  }
  for (int k = 0; k < 6; ++k) W[k] = make_float4(v[k][0], v[k][1], v[k][2], v[k][3]);
  W[6] = make_float4(__uint_as_float(out_ref[0]), __uint_as_float(out_ref[1]), __uint_as_float(out_ref[2]),
                     __uint_as_float(out_ref[3]));
  W[7] = make_float4(0.f, 0.f, 0.f, 0.f);
  atomicMax(max_depth, it.depth);
}

// One level of the collapse: the level's item count is read from the device
// (n_in_p) and the grid strides over it.
__global__ void k_collapse(const uint2* __restrict__ child, const BinNode* __restrict__ box,
                           const uint2* __restrict__ range, const float4* __restrict__ tris,
                           const CollapseItem* __restrict__ qin, const uint32_t* __restrict__ n_in_p,
                           CollapseItem* __restrict__ qout, uint32_t* __restrict__ n_out, uint32_t* __restrict__ n_wide,
                           float4* __restrict__ wide, uint32_t bound, uint32_t leaf_size, uint32_t* __restrict__ max_depth,
                           uint32_t* __restrict__ status) {
  const uint32_t n_in = *n_in_p;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_in; t += gridDim.x * blockDim.x)
    collapse_one(child, box, range, tris, qin[t], qout, n_out, n_wide, wide, bound, leaf_size, max_depth, status);
}

// -------------------------------------------------------- 5b. PLOC ----
//
// Parallel locally-ordered clustering (Meister and Bittner 2018, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction"):
// the Morton-sorted leaves start as clusters; every cluster picks the
// cluster within kPlocRadius list positions whose union box has the smallest
// surface area (equal areas: the smaller position; with the pair order this
// is a total order, so the globally best pair is always mutual and every
// round merges); mutual pairs become a new binary node at the lower
// position; the list is compacted (two exclusive scans) and the rounds
// repeat until one cluster is left. Subtrees are no longer Morton ranges, so
// the collapse below carries each subtree's first position in the new leaf
// order and writes the triangles there.

#ifndef J3DG_PLOC_RADIUS
#define J3DG_PLOC_RADIUS 8  // 2..64 measured on the torus frames: 8 visits the fewest nodes
#endif
static const int kPlocRadius = J3DG_PLOC_RADIUS;
static const int kPlocBlock = 256;

__global__ void k_ploc_init(const float4* __restrict__ tris, uint32_t n, uint32_t* __restrict__ C,
                            float4* __restrict__ lo, float4* __restrict__ hi) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  C[i] = 0x80000000u | i;
  leaf_box(tris, i, lo[i], hi[i]);
}

__device__ __forceinline__ float merged_area(float4 alo, float4 ahi, float4 blo, float4 bhi) {
  const float dx = fmaxf(ahi.x, bhi.x) - fminf(alo.x, blo.x);
  const float dy = fmaxf(ahi.y, bhi.y) - fminf(alo.y, blo.y);
  const float dz = fmaxf(ahi.z, bhi.z) - fminf(alo.z, blo.z);
  const float a = dx * dy + dy * dz + dz * dx;
  return a == a ? a : FLT_MAX;  // boxes with NaN planes still get an order
}

// Clusters are searched within their own segment (seg: the segment of each
// list position, all 0 for one segment); a cluster alone in its segment gets
// no neighbour (0xffffffff) and so never merges.
__global__ void __launch_bounds__(kPlocBlock) k_ploc_nn(const float4* __restrict__ lo, const float4* __restrict__ hi,
                                                       const uint32_t* __restrict__ seg,
                                                       const uint32_t* __restrict__ m_p,
                                                       const uint32_t* __restrict__ n_seg_p, uint32_t* __restrict__ nn) {
  __shared__ float4 slo[kPlocBlock + 2 * kPlocRadius], shi[kPlocBlock + 2 * kPlocRadius];
  __shared__ uint32_t sseg[kPlocBlock + 2 * kPlocRadius];
  const uint32_t m = *m_p;
  if (m <= *n_seg_p) return;  // every segment is one cluster: no round
  for (uint32_t tile = blockIdx.x; tile * kPlocBlock < m; tile += gridDim.x) {  // uniform over the block
    const int base = (int)(tile * kPlocBlock) - kPlocRadius;
    for (int k = threadIdx.x; k < kPlocBlock + 2 * kPlocRadius; k += blockDim.x) {
      const int j = base + k;
      if (j >= 0 && j < (int)m) {
        slo[k] = lo[j];
        shi[k] = hi[j];
        sseg[k] = seg[j];
      }
    }
    __syncthreads();
    const int i = (int)(tile * kPlocBlock + threadIdx.x);
    if (i < (int)m) {
      const int si = threadIdx.x + kPlocRadius;
      const float4 alo = slo[si], ahi = shi[si];
      const uint32_t my = sseg[si];
      float best = INFINITY;
      uint32_t bj = 0xffffffffu;
      for (int o = -kPlocRadius; o <= kPlocRadius; ++o) {
        const int j = i + o;
        if (o == 0 || j < 0 || j >= (int)m || sseg[si + o] != my) continue;
        const float a = merged_area(alo, ahi, slo[si + o], shi[si + o]);
        if (a < best) {  // increasing j: the first of equal areas is the smaller position
          best = a;
          bj = (uint32_t)j;
        }
      }
      nn[i] = bj;
    }
    __syncthreads();  // the tile's shared copies are read before the next tile overwrites them
  }
}

// a PLOC round's two compactions in one pass: position i creates a node if it
// and its nearest neighbour j are mutual with i < j, and survives (keeps a
// list slot) unless it is the j > i side of a mutual pair. Each chunk of 1024
// positions (256 threads x 4) writes the exclusive scans of both flags
// within the chunk (cps, sps) and its two totals (csum, ssum; scanned by
// k_scan_sums, whose grand totals are the round's creates and survivors).
__global__ void __launch_bounds__(256) k_ploc_flag_scan(const uint32_t* __restrict__ nn, const uint32_t* __restrict__ m_p,
                                                        const uint32_t* __restrict__ n_seg_p,
                                                        uint32_t* __restrict__ cps, uint32_t* __restrict__ sps,
                                                        uint32_t* __restrict__ csum, uint32_t* __restrict__ ssum) {
  __shared__ uint32_t wsum[2][8];
  const uint32_t m = *m_p;
  if (m <= *n_seg_p || blockIdx.x * 1024u >= m) return;  // no round, or past the list
  const uint32_t base = blockIdx.x * 1024u + threadIdx.x * 4u;
  uint32_t c[4] = {0u, 0u, 0u, 0u}, v[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t i = base + k;
    if (i < m) {
      const uint32_t j = nn[i];
      const bool mutual = j < m && nn[j] == i;
      c[k] = (mutual && i < j) ? 1u : 0u;
      v[k] = (!mutual || i < j) ? 1u : 0u;
    }
  }
  const uint32_t ct = c[0] + c[1] + c[2] + c[3], vt = v[0] + v[1] + v[2] + v[3];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t ci = ct, vi = vt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t yc = __shfl_up_sync(0xffffffffu, ci, o);
    const uint32_t yv = __shfl_up_sync(0xffffffffu, vi, o);
    if (lane >= (uint32_t)o) {
      ci += yc;
      vi += yv;
    }
  }
  if (lane == 31) {
    wsum[0][warp] = ci;
    wsum[1][warp] = vi;
  }
  __syncthreads();
  uint32_t co = 0, vo = 0, call = 0, vall = 0;
#pragma unroll
  for (uint32_t w = 0; w < 8; ++w) {
    const uint32_t xc = wsum[0][w], xv = wsum[1][w];
    co += w < warp ? xc : 0u;
    vo += w < warp ? xv : 0u;
    call += xc;
    vall += xv;
  }
  const uint32_t ec = co + ci - ct, ev = vo + vi - vt;
  const uint4 oc = make_uint4(ec, ec + c[0], ec + c[0] + c[1], ec + c[0] + c[1] + c[2]);
  const uint4 ov = make_uint4(ev, ev + v[0], ev + v[0] + v[1], ev + v[0] + v[1] + v[2]);
  if (base + 3 < m) {
    *reinterpret_cast<uint4*>(cps + base) = oc;
    *reinterpret_cast<uint4*>(sps + base) = ov;
  } else {
    const uint32_t a4[4] = {oc.x, oc.y, oc.z, oc.w}, b4[4] = {ov.x, ov.y, ov.z, ov.w};
    for (uint32_t k = 0; k < 4 && base + k < m; ++k) {
      cps[base + k] = a4[k];
      sps[base + k] = b4[k];
    }
  }
  if (threadIdx.x == 0) {
    csum[blockIdx.x] = call;
    ssum[blockIdx.x] = vall;
  }
}

__device__ __forceinline__ void ploc_merge_one(const uint32_t* __restrict__ C, const float4* __restrict__ lo,
                                               const float4* __restrict__ hi, const uint32_t* __restrict__ seg,
                                               const uint32_t* __restrict__ nn, const uint32_t* __restrict__ cps,
                                               const uint32_t* __restrict__ sps, const uint32_t* __restrict__ csum,
                                               const uint32_t* __restrict__ ssum, uint32_t i, uint32_t m,
                                               uint32_t node_base, uint32_t* __restrict__ C2,
                                               float4* __restrict__ lo2, float4* __restrict__ hi2,
                                               uint32_t* __restrict__ seg2, uint2* __restrict__ child,
                                               BinNode* __restrict__ box, uint32_t* __restrict__ count) {
  const uint32_t j = nn[i];
  const bool mutual = j < m && nn[j] == i;
  if (mutual && i > j) return;  // merged into the node made at j
  const uint32_t pos = sps[i] + ssum[i >> 10];  // survivors before i
  seg2[pos] = seg[i];
  if (!mutual) {
    C2[pos] = C[i];
    lo2[pos] = lo[i];
    hi2[pos] = hi[i];
    return;
  }
  const uint32_t p = node_base + cps[i] + csum[i >> 10];  // nodes made before i's
  const uint32_t a = C[i], b = C[j];
  const float4 l = make_float4(fminf(lo[i].x, lo[j].x), fminf(lo[i].y, lo[j].y), fminf(lo[i].z, lo[j].z), 0.f);
  const float4 h = make_float4(fmaxf(hi[i].x, hi[j].x), fmaxf(hi[i].y, hi[j].y), fmaxf(hi[i].z, hi[j].z), 0.f);
  child[p] = make_uint2(a, b);
  box[p].lo = l;
  box[p].hi = h;
  count[p] = ((a & 0x80000000u) ? 1u : count[a]) + ((b & 0x80000000u) ? 1u : count[b]);
  C2[pos] = p;
  lo2[pos] = l;
  hi2[pos] = h;
}

__global__ void k_ploc_merge(const uint32_t* __restrict__ C, const float4* __restrict__ lo,
                             const float4* __restrict__ hi, const uint32_t* __restrict__ seg,
                             const uint32_t* __restrict__ nn, const uint32_t* __restrict__ cps,
                             const uint32_t* __restrict__ sps, const uint32_t* __restrict__ csum,
                             const uint32_t* __restrict__ ssum, const uint32_t* __restrict__ m_p,
                             const uint32_t* __restrict__ n_seg_p, const uint32_t* __restrict__ node_base_p,
                             uint32_t* __restrict__ C2, float4* __restrict__ lo2, float4* __restrict__ hi2,
                             uint32_t* __restrict__ seg2, uint2* __restrict__ child, BinNode* __restrict__ box,
                             uint32_t* __restrict__ count) {
  const uint32_t m = *m_p, node_base = *node_base_p;
  if (m <= *n_seg_p) return;  // no round
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    ploc_merge_one(C, lo, hi, seg, nn, cps, sps, csum, ssum, i, m, node_base, C2, lo2, hi2, seg2, child, box, count);
}

// ------------------------------------------- 6b. cost-optimal collapse ----
//
// SAH cost of covering the subtree of binary node n with at most i = 1..4
// slots of a wide node (the dynamic programme of Ylitie, Karras and Laine
// 2017, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide
// BVHs", section 3.1, for 4-wide nodes). A is half the surface area:
//   C(tri, i) = A(tri) c_t
//   C(n, 1)   = min(leaf: A(n) N(n) c_t if N(n) <= leaf_size,
//                   node: A(n) c_n + min_k C(left, k) + C(right, 4 - k))
//   C(n, i)   = min(C(n, i - 1), min_k C(left, k) + C(right, i - k))
// Children are made in earlier PLOC rounds, so one launch per round, in
// round order, sees its children's costs. The decisions steer the collapse:
// dec.x = the k of the node case (bit 7 set: the leaf case is cheaper);
// dec.y, .z, .w for i = 2, 3, 4: 0 = as i - 1, else the k of the best split.

#ifndef J3DG_SAH_COLLAPSE
#define J3DG_SAH_COLLAPSE 1
#endif
#ifndef J3DG_SAH_CTRI
#define J3DG_SAH_CTRI 0.5f  // cost of a triangle test relative to a node visit
#endif

__device__ __forceinline__ float half_area4(float4 lo, float4 hi);

// costs C(r, 1..W) of subtree r (a triangle: its area times c_t for any i)
template <int W>
__device__ __forceinline__ void sub_costs(const float* __restrict__ cost, const float4* __restrict__ tris, uint32_t r,
                                          float (&c)[W + 1]) {
  if (r & 0x80000000u) {
    float4 lo, hi;
    leaf_box(tris, r & 0x7fffffffu, lo, hi);
    const float v = half_area4(lo, hi) * J3DG_SAH_CTRI;
#pragma unroll
    for (int i = 1; i <= W; ++i) c[i] = v;
  } else {
#pragma unroll
    for (int i = 1; i <= W; ++i) c[i] = cost[(size_t)r * W + i - 1];
  }
}

// cost: W floats per binary node (C(n, 1..W)); dec: W bytes per node
// (dec[0] = the k of the node case | 0x80 when the leaf case is cheaper;
// dec[i - 1], i = 2..W: 0 = as i - 1, else the k of the best split)
template <int W>
__device__ __forceinline__ void collapse_cost_one(const uint2* __restrict__ child, const BinNode* __restrict__ box,
                                                  const uint32_t* __restrict__ count, const float4* __restrict__ tris,
                                                  uint32_t n, uint32_t leaf_size, float* __restrict__ cost,
                                                  uint8_t* __restrict__ dec) {
  const uint2 c = child[n];
  float cl[W + 1], cr[W + 1], C[W + 1];
  sub_costs<W>(cost, tris, c.x, cl);
  sub_costs<W>(cost, tris, c.y, cr);
  const float A = half_area4(box[n].lo, box[n].hi);
  float best = FLT_MAX;
  uint32_t bk = 1;
#pragma unroll
  for (uint32_t k = 1; k < (uint32_t)W; ++k)
    if (cl[k] + cr[W - k] < best) {
      best = cl[k] + cr[W - k];
      bk = k;
    }
  const float node = A + best;  // c_n = 1
  const uint32_t N = count[n];
  const float leaf = N <= leaf_size ? A * (float)N * J3DG_SAH_CTRI : FLT_MAX;
  C[1] = fminf(leaf, node);
  uint8_t d[W];
  d[0] = (uint8_t)(bk | (leaf <= node ? 0x80u : 0u));
#pragma unroll
  for (uint32_t i = 2; i <= (uint32_t)W; ++i) {
    float v = C[i - 1];
    uint32_t dk = 0;
    for (uint32_t k = 1; k < i; ++k)
      if (cl[k] + cr[i - k] < v) {
        v = cl[k] + cr[i - k];
        dk = k;
      }
    C[i] = v;
    d[i - 1] = (uint8_t)dk;
  }
#pragma unroll
  for (int i = 1; i <= W; ++i) {
    cost[(size_t)n * W + i - 1] = C[i];
    dec[(size_t)n * W + i - 1] = d[i - 1];
  }
}

template <int W>
__global__ void k_collapse_cost(const uint2* __restrict__ child, const BinNode* __restrict__ box,
                                const uint32_t* __restrict__ count, const float4* __restrict__ tris,
                                const uint32_t* __restrict__ lohi, uint32_t leaf_size, float* __restrict__ cost,
                                uint8_t* __restrict__ dec) {
  // the pass's binary nodes [lohi[0], lohi[1]) (device memory)
  const uint32_t lo = lohi[0], hi = lohi[1];
  for (uint32_t n = lo + blockIdx.x * blockDim.x + threadIdx.x; n < hi; n += gridDim.x * blockDim.x)
    collapse_cost_one<W>(child, box, count, tris, n, leaf_size, cost, dec);
}

struct PlaceItem {
  uint32_t bin;    // binary node index
  uint32_t wide;   // wide node index to fill
  uint32_t depth;
  uint32_t start;  // first leaf-order position of the subtree
};

// The collapse of k_collapse over a tree whose subtrees are not ranges of the
// sorted leaves: each slot carries its subtree's first position; leaves are
// written to tris_out at those positions in depth-first order.
template <int W>
__device__ __forceinline__ void collapse_place_one(const uint2* __restrict__ child, const BinNode* __restrict__ box,
                                                   const uint32_t* __restrict__ count, const float4* __restrict__ tris,
                                                   const PlaceItem* __restrict__ qin, uint32_t t, uint32_t n_in,
                                                   PlaceItem* __restrict__ qout, uint32_t* __restrict__ n_out,
                                                   uint32_t wide_base, float4* __restrict__ wide, uint32_t leaf_size,
                                                   uint32_t* __restrict__ max_depth, float4* __restrict__ tris_out,
                                                   uint32_t nt, uint32_t* status, const uint8_t* __restrict__ dec) {
  // whole warps come here together (the next level's slots are allocated per
  // warp); lanes past n_in place nothing
  const uint32_t lane = threadIdx.x & 31u;
  const bool valid = t < n_in;
  const PlaceItem it = valid ? qin[t] : PlaceItem{0u, 0u, 0u, 0u};
  uint32_t ref[W], cnt[W], start[W];
  float4 lo[W], hi[W];
  auto load = [&](uint32_t r, int s, uint32_t first) {
    ref[s] = r;
    start[s] = first;
    if (r & 0x80000000u) {
      leaf_box(tris, r & 0x7fffffffu, lo[s], hi[s]);
      cnt[s] = 1;
    } else {
      lo[s] = box[r].lo;
      hi[s] = box[r].hi;
      cnt[s] = count[r];
    }
  };
  const uint2 c = valid ? child[it.bin] : make_uint2(0u, 0u);
  int m = 0;
  if (!valid) {
  } else if (dec) {
    // the slots the cost decisions give: expand(left, k) then expand(right, W - k)
    struct Slot {
      uint32_t r, i, start;
    };
    Slot stk[2 * W];
    int sp = 0;
    const uint32_t k = dec[(size_t)it.bin * W] & 0x7fu;
    const uint32_t nl = (c.x & 0x80000000u) ? 1u : count[c.x];
    stk[sp++] = Slot{c.y, (uint32_t)W - k, it.start + nl};
    stk[sp++] = Slot{c.x, k, it.start};
    while (sp > 0 && m < W) {
      const Slot e = stk[--sp];
      if ((e.r & 0x80000000u) || e.i <= 1u) {
        load(e.r, m++, e.start);
        continue;
      }
      const uint32_t d = dec[(size_t)e.r * W + e.i - 1];
      if (d == 0u || sp + 2 > 2 * W) {
        stk[sp++] = Slot{e.r, e.i - 1u, e.start};
        continue;
      }
      const uint2 cc = child[e.r];
      const uint32_t ml = (cc.x & 0x80000000u) ? 1u : count[cc.x];
      stk[sp++] = Slot{cc.y, e.i - d, e.start + ml};
      stk[sp++] = Slot{cc.x, d, e.start};
    }
  } else {
    load(c.x, 0, it.start);
    load(c.y, 1, it.start + cnt[0]);
    m = 2;
  }
  while (valid && !dec && m < W) {
    int best = -1;
    float ba = -1.f;
    for (int s = 0; s < m; ++s)
      if (cnt[s] > leaf_size) {
        const float a = half_area(lo[s], hi[s]);
        if (a > ba) {
          ba = a;
          best = s;
        }
      }
    if (best < 0) break;
    const uint2 cc = child[ref[best]];
    const uint32_t s0 = start[best];
    load(cc.x, best, s0);
    load(cc.y, m, s0 + cnt[best]);
    ++m;
  }
  // slots placed as leaves, and the next level's queue slots for the rest:
  // one atomic per warp (a warp-wide scan of the lanes' internal slots)
  uint32_t leaf_mask = 0u, n_int = 0u;
  for (int s = 0; s < m; ++s) {
    const bool as_leaf = (ref[s] & 0x80000000u) ||
                         (dec ? (dec[(size_t)ref[s] * W] & 0x80u) != 0 : cnt[s] <= leaf_size);
    if (as_leaf && cnt[s] <= J3DG_MAX_LEAF)
      leaf_mask |= 1u << s;
    else
      ++n_int;
  }
  uint32_t incl = n_int;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  uint32_t q_base = 0u;
  if (lane == 31u && incl > 0u) q_base = atomicAdd(n_out, incl);
  uint32_t q = __shfl_sync(0xffffffffu, q_base, 31) + incl - n_int;  // this lane's first queue slot
  const uint32_t dmax = __reduce_max_sync(0xffffffffu, valid ? it.depth : 0u);
  if (lane == 0u && dmax > 0u) atomicMax(max_depth, dmax);
  if (!valid) return;
  // the node in the width-W layout: planes [6][W], refs [W], zero padding
  float F[4 * J3DG_NODE_F4(W)];
#pragma unroll
  for (int k = 0; k < 4 * J3DG_NODE_F4(W); ++k) F[k] = 0.f;
  for (int s = 0; s < W; ++s) {
    uint32_t out_ref = J3DG_EMPTY_REF;
    if (s < m) {
      F[0 * W + s] = lo[s].x;
      F[1 * W + s] = hi[s].x;
      F[2 * W + s] = lo[s].y;
      F[3 * W + s] = hi[s].y;
      F[4 * W + s] = lo[s].z;
      F[5 * W + s] = hi[s].z;
      if (leaf_mask & (1u << s)) {
        out_ref = J3DG_LEAF_BIT | (start[s] << 3) | (cnt[s] - 1u);
        uint32_t stk[J3DG_MAX_LEAF];
        int sp = 0;
        uint32_t k = 0;
        stk[sp++] = ref[s];
        while (sp > 0) {
          const uint32_t r = stk[--sp];
          if (r & 0x80000000u) {
            const uint32_t src = r & 0x7fffffffu, dst = start[s] + k++;
            if (src < nt && dst < nt) {
              tris_out[3 * (size_t)dst] = tris[3 * (size_t)src];
              tris_out[3 * (size_t)dst + 1] = tris[3 * (size_t)src + 1];
              tris_out[3 * (size_t)dst + 2] = tris[3 * (size_t)src + 2];
            } else {
              atomicOr(status, J3DG_DEV_BAD_INDEX);
            }
          } else if (sp + 2 <= (int)J3DG_MAX_LEAF) {
            const uint2 cc = child[r];
            stk[sp++] = cc.y;
            stk[sp++] = cc.x;
          } else {
            atomicOr(status, J3DG_DEV_STACK_OVERFLOW);
            break;
          }
        }
      } else {
        // the next level's wide nodes follow this level's, in queue order
        // (the queue and the node array hold nt entries: a malformed tree
        // is stopped here)
        if (q < nt && wide_base + q < nt) {
          qout[q] = PlaceItem{ref[s], wide_base + q, it.depth + 1, start[s]};
        } else {
          atomicOr(status, J3DG_DEV_BAD_INDEX);
        }
        out_ref = wide_base + q;
        ++q;
      }
    } else {
      F[0 * W + s] = F[2 * W + s] = F[4 * W + s] = 3.4e38f;
      F[1 * W + s] = F[3 * W + s] = F[5 * W + s] = -3.4e38f;
    }
    F[6 * W + s] = __uint_as_float(out_ref);
  }
  if (it.wide >= nt) {
    atomicOr(status, J3DG_DEV_BAD_INDEX);
    return;
  }
  float4* Wn = wide + J3DG_NODE_F4(W) * (size_t)it.wide;
#pragma unroll
  for (int k = 0; k < J3DG_NODE_F4(W); ++k) Wn[k] = make_float4(F[4 * k], F[4 * k + 1], F[4 * k + 2], F[4 * k + 3]);
}

// a level of the placement: the queue's n_in items (device memory) with
// their wide nodes from wide_base on (device memory); warp-uniform strides
template <int W>
__global__ void k_collapse_place(const uint2* __restrict__ child, const BinNode* __restrict__ box,
                                 const uint32_t* __restrict__ count, const float4* __restrict__ tris,
                                 const PlaceItem* __restrict__ qin, const uint32_t* __restrict__ n_in_p,
                                 PlaceItem* __restrict__ qout, uint32_t* __restrict__ n_out,
                                 const uint32_t* __restrict__ wide_base_p, float4* __restrict__ wide,
                                 uint32_t leaf_size, uint32_t* __restrict__ max_depth, float4* __restrict__ tris_out,
                                 uint32_t nt, uint32_t* status, const uint8_t* __restrict__ dec) {
  const uint32_t n_in = *n_in_p, wide_base = *wide_base_p;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t t0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); t0 < n_in; t0 += stride)
    collapse_place_one<W>(child, box, count, tris, qin, t0 + (threadIdx.x & 31u), n_in, qout, n_out, wide_base, wide,
                          leaf_size, max_depth, tris_out, nt, status, dec);
}

// ------------------------------------------------ 7. depth-first order ----
//
// The collapse numbers wide nodes level by level, so the nodes on one ray's
// path from the root to a leaf lie far apart in memory (one per level, each
// level hundreds of MB wide at the bottom). Renumbering in depth-first order
// puts every subtree in one contiguous range: the deep part of a path, and
// the paths of neighbouring rays, then fall in the same few pages. Each
// level is a contiguous index range (a collapse launch allocates exactly the
// next level), so subtree sizes go bottom-up and new positions top-down, one
// launch per level.

template <int W>
__device__ __forceinline__ void child_refs(const float4* __restrict__ wide, uint32_t i, uint32_t (&r)[W]) {
  const float* f = reinterpret_cast<const float*>(wide + J3DG_NODE_F4(W) * (size_t)i) + 6 * W;
#pragma unroll
  for (int c = 0; c < W; ++c) r[c] = __float_as_uint(f[c]);
}

// size[i] = wide nodes in the subtree of i (children of level lo..hi are done)
template <int W>
__global__ void k_dfs_size(const float4* __restrict__ wide, const uint32_t* __restrict__ lohi,
                           uint32_t* __restrict__ size) {
  const uint32_t lo = lohi[0], hi = lohi[1];  // the level's nodes (device memory)
  for (uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += gridDim.x * blockDim.x) {
    uint32_t r[W], s = 1;
    child_refs<W>(wide, i, r);
#pragma unroll
    for (int c = 0; c < W; ++c)
      if (!(r[c] & J3DG_LEAF_BIT)) s += size[r[c]];  // the empty ref has the leaf bit
    size[i] = s;
  }
}

// children of the level's nodes take consecutive ranges after their parent
template <int W>
__global__ void k_dfs_place(const float4* __restrict__ wide, const uint32_t* __restrict__ lohi,
                            const uint32_t* __restrict__ size, uint32_t* __restrict__ pos) {
  const uint32_t lo = lohi[0], hi = lohi[1];  // the level's nodes (device memory)
  for (uint32_t i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += gridDim.x * blockDim.x) {
    uint32_t r[W], next = pos[i] + 1;
    child_refs<W>(wide, i, r);
#pragma unroll
    for (int c = 0; c < W; ++c)
      if (!(r[c] & J3DG_LEAF_BIT)) {
        pos[r[c]] = next;
        next += size[r[c]];
      }
  }
}

template <int W>
__global__ void k_dfs_permute(const float4* __restrict__ wide, const uint32_t* __restrict__ n_p,
                              const uint32_t* __restrict__ pos, float4* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *n_p) return;
  constexpr int F4 = J3DG_NODE_F4(W);
  const float4* src = wide + F4 * (size_t)i;
  float F[4 * F4];
#pragma unroll
  for (int k = 0; k < F4; ++k) {
    const float4 v = src[k];
    F[4 * k] = v.x, F[4 * k + 1] = v.y, F[4 * k + 2] = v.z, F[4 * k + 3] = v.w;
  }
#pragma unroll
  for (int c = 0; c < W; ++c) {
    const uint32_t r = __float_as_uint(F[6 * W + c]);
    if (!(r & J3DG_LEAF_BIT)) F[6 * W + c] = __uint_as_float(pos[r]);
  }
  float4* dst = out + F4 * (size_t)pos[i];
#pragma unroll
  for (int k = 0; k < F4; ++k) dst[k] = make_float4(F[4 * k], F[4 * k + 1], F[4 * k + 2], F[4 * k + 3]);
}

// the device-driven builder's fixed grids (grid-stride kernels)
static const uint32_t kStrideBlocks = 2048;

// one full wave of 128-thread blocks (16 per SM): the collapse kernels are
// chains of dependent loads per item, so every resident thread slot is used
static uint32_t wave_blocks128() {
  static uint32_t blocks = 0;
  if (!blocks) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    blocks = sms > 0 ? 16u * (uint32_t)sms : kStrideBlocks;
  }
  return blocks;
}

static void launch_collapse_cost(uint32_t W, const uint2* child, const BinNode* box, const uint32_t* count,
                                 const float4* tris, const uint32_t* lohi, uint32_t leaf_size, float* cost,
                                 uint8_t* dec, cudaStream_t st) {
  if (W == 2)
    k_collapse_cost<2><<<kStrideBlocks, 256, 0, st>>>(child, box, count, tris, lohi, leaf_size, cost, dec);
  else if (W == 8)
    k_collapse_cost<8><<<kStrideBlocks, 256, 0, st>>>(child, box, count, tris, lohi, leaf_size, cost, dec);
  else
    k_collapse_cost<4><<<kStrideBlocks, 256, 0, st>>>(child, box, count, tris, lohi, leaf_size, cost, dec);
}

static void launch_collapse_place(uint32_t W, const uint2* child, const BinNode* box, const uint32_t* count,
                                  const float4* tris, const PlaceItem* qin, const uint32_t* n_in, PlaceItem* qout,
                                  uint32_t* n_out, const uint32_t* wide_base, float4* wide, uint32_t leaf_size,
                                  uint32_t* max_depth, float4* tris_out, uint32_t nt, uint32_t* status,
                                  const uint8_t* dec, cudaStream_t st) {
  if (W == 2)
    k_collapse_place<2><<<wave_blocks128(), 128, 0, st>>>(child, box, count, tris, qin, n_in, qout, n_out, wide_base, wide,
                                                      leaf_size, max_depth, tris_out, nt, status, dec);
  else if (W == 8)
    k_collapse_place<8><<<wave_blocks128(), 128, 0, st>>>(child, box, count, tris, qin, n_in, qout, n_out, wide_base, wide,
                                                      leaf_size, max_depth, tris_out, nt, status, dec);
  else
    k_collapse_place<4><<<wave_blocks128(), 128, 0, st>>>(child, box, count, tris, qin, n_in, qout, n_out, wide_base, wide,
                                                      leaf_size, max_depth, tris_out, nt, status, dec);
}

// -------------------------------------------------- 5c. SAH top levels ----
//
// Above J3DG_SAH_TOP triangles a node is split top-down by binned SAH (Wald
// 2007, "On fast Construction of SAH-based Bounding Volume Hierarchies"):
// per level, every task (a range of the triangle order `ord`) bins its
// triangles' centroids into kTopBins bins per axis (per-block bins in shared
// memory, then merged into the task's bins; tasks of at most kTopWarpTask
// triangles are binned by one warp each), one warp per task finds the split
// of least A_L N_L + A_R N_R from prefix and suffix unions of the bins
// (shuffles, lanes = bins), and a stable partition
// (flags from the bin codes that binning stored per position, one exclusive
// scan) reorders the range. A stable partition of the
// Morton-sorted order keeps every range in Morton order, so each range of at
// most J3DG_SAH_TOP triangles (a segment) is then clustered by PLOC on its
// own (neighbours searched within the segment only), and the segment roots
// are linked under the top nodes.

// segment size below which PLOC takes over (0: PLOC over the whole mesh).
// Measured on the 28M-triangle torus frames (node visits per ray, ms per
// 1080p frame, build ms): PLOC only 6.955 / 0.881 / 39; 4096: 6.402 / 0.862
// / 67; 256: 6.256 / 0.855 / 76; 64: 6.200 / 0.851 / 87; 16: 6.193 / 0.852
// / 112.
#ifndef J3DG_SAH_TOP
#define J3DG_SAH_TOP 64u
#endif
static const int kTopBins = 16;
static_assert(kTopBins <= 16, "bin codes keep 4 bits per axis");
// per bin: count, box lo / hi xyz (ordered-float encoded). The children's
// centroid ranges (the next level's bin ranges) are their boxes: every
// centroid lies in its triangle's box, and with triangles small against a
// task the two ranges differ by about one triangle
static const int kTopVals = 7;
static const uint32_t kNoTask = 0xffffffffu;
static const uint32_t kPendingRef = 0xfffffffeu;  // child slot filled by a segment root later

struct TopTask {
  uint32_t begin, end, node, pad;
  float4 clo, chi;  // centroid bounds
};

struct TopSplit {
  uint32_t axis;   // 3: split by position (no usable SAH split)
  uint32_t bin;    // bins 0..bin go left
  uint32_t nleft;
  uint32_t pad;
  uint32_t task[2];  // the children's tasks of the next level (kNoTask: a finished range)
  uint32_t pad2[2];
  float4 lclo, lchi, rclo, rchi;  // children's centroid bounds
};

// triangle boxes by triangle, computed once for the top levels
__global__ void k_top_boxes(const float4* __restrict__ tris, uint32_t n, float4* __restrict__ blo,
                            float4* __restrict__ bhi) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) leaf_box(tris, i, blo[i], bhi[i]);
}

struct TopRange {  // a finished range: a segment for PLOC
  uint32_t begin, end, parent, side;
};

// float <-> uint32 with the same order (for atomic min / max)
__device__ __forceinline__ uint32_t f2o(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t o) { return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o); }

__device__ __forceinline__ int top_bin(float c, float lo, float hi) {
  const float ext = hi - lo;
  if (!(ext > 0.f)) return 0;
  const int b = (int)((c - lo) / ext * (float)kTopBins);
  return b < 0 ? 0 : (b >= kTopBins ? kTopBins - 1 : b);
}

static const int kTopChunk = 2048;
// Tasks up to this size are binned by one warp each (k_top_bin_warp): at
// that depth 32 neighbouring triangles span many bins, so grouping lanes by
// bin (match + reductions per group) serialises; plain shared atomics do not.
static const uint32_t kTopWarpTask = 2048;

// global bins of the tasks larger than kTopWarpTask (k_top_bin's); the
// smaller tasks keep their bins in shared memory
// (the level's task count and largest task are read from device memory;
// levels with no task above kTopWarpTask have nothing to do here)
__global__ void k_top_bins_init(uint32_t* __restrict__ bins, const uint32_t* __restrict__ n_tasks_p,
                                const uint32_t* __restrict__ max_task_p, const TopTask* __restrict__ tasks) {
  if (*max_task_p <= kTopWarpTask) return;
  const uint32_t n_words = *n_tasks_p * 3 * kTopBins * kTopVals;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_words; i += gridDim.x * blockDim.x) {
    const TopTask& T = tasks[i / (3 * kTopBins * kTopVals)];
    if (T.end - T.begin <= kTopWarpTask) continue;
    const uint32_t v = i % kTopVals;
    bins[i] = v == 0 ? 0u : (((v - 1) % 6) < 3 ? 0xffffffffu : 0u);  // lo fields: max code, hi fields: 0
  }
}


// bins of every active task: [task][axis][bin][kTopVals]
__global__ void __launch_bounds__(256) k_top_bin(const uint32_t* __restrict__ ord, const float4* __restrict__ blo,
                                                 const float4* __restrict__ bhi, const uint32_t* __restrict__ task_of,
                                                 const TopTask* __restrict__ tasks,
                                                 const uint32_t* __restrict__ n_tasks_p,
                                                 const uint32_t* __restrict__ max_task_p, uint32_t n,
                                                 uint32_t* __restrict__ bins, uint16_t* __restrict__ code) {
  __shared__ uint32_t sb[3 * kTopBins * kTopVals];
  __shared__ uint32_t s_task;
  const uint32_t n_tasks = *n_tasks_p;
  if (n_tasks == 0 || *max_task_p <= kTopWarpTask) return;  // k_top_bin_warp's level, or no level
  const uint32_t c0 = blockIdx.x * kTopChunk, c1 = min(n, c0 + kTopChunk);
  if (c0 >= n) return;
  if (threadIdx.x == 0) {
    const uint32_t a = task_of[c0], b = task_of[c1 - 1];
    s_task = (a == b && a < n_tasks && tasks[a].end - tasks[a].begin > kTopWarpTask) ? a : kNoTask;
  }
  for (uint32_t k = threadIdx.x; k < 3 * kTopBins * kTopVals; k += blockDim.x) {
    const uint32_t v = k % kTopVals;
    sb[k] = v == 0 ? 0u : (((v - 1) % 6) < 3 ? 0xffffffffu : 0u);
  }
  __syncthreads();
  const uint32_t st = s_task;
  const uint32_t lane = threadIdx.x & 31u;
  for (uint32_t base = c0; base < c1; base += blockDim.x) {  // uniform trip count: whole warps
    const uint32_t p = base + threadIdx.x;
    uint32_t t = p < c1 ? (st != kNoTask ? st : task_of[p]) : kNoTask;
    if (st == kNoTask && t < n_tasks && tasks[t].end - tasks[t].begin <= kTopWarpTask) t = kNoTask;  // k_top_bin_warp's
    const bool valid = t < n_tasks;
    float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo, c = lo;
    int bx = 0, by = 0, bz = 0;
    if (valid) {
      const uint32_t tri = ord[p];
      lo = blo[tri];
      hi = bhi[tri];
      c = make_float4(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z), 0.f);
      const TopTask T = tasks[t];
      bx = top_bin(c.x, T.clo.x, T.chi.x);
      by = top_bin(c.y, T.clo.y, T.chi.y);
      bz = top_bin(c.z, T.clo.z, T.chi.z);
      code[p] = (uint16_t)(bx | (by << 4) | (bz << 8));
    }
    // neighbouring triangles (Morton order) mostly share a task and bins:
    // lanes of one (task, bin) reduce in registers and one lane updates the
    // bin -- in shared memory when the whole chunk is one task, else in the
    // task's global bins
    const uint32_t vm = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      const uint32_t v[6] = {f2o(lo.x), f2o(lo.y), f2o(lo.z), f2o(hi.x), f2o(hi.y), f2o(hi.z)};
      const int bins3[3] = {bx, by, bz};
      uint32_t* dst = st != kNoTask ? sb : bins + (size_t)t * 3 * kTopBins * kTopVals;
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        const uint32_t g = __match_any_sync(vm, t * (uint32_t)kTopBins + (uint32_t)bins3[ax]);
        const uint32_t n_g = (uint32_t)__popc(g);
        uint32_t r[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) r[k] = k < 3 ? __reduce_min_sync(g, v[k]) : __reduce_max_sync(g, v[k]);
        if (lane == (uint32_t)(__ffs(g) - 1)) {
          uint32_t* b = dst + (ax * kTopBins + bins3[ax]) * kTopVals;
          atomicAdd(b, n_g);
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            if (k < 3)
              atomicMin(b + 1 + k, r[k]);
            else
              atomicMax(b + 1 + k, r[k]);
          }
        }
      }
    }
  }
  if (st == kNoTask) return;
  __syncthreads();
  uint32_t* g = bins + (size_t)st * 3 * kTopBins * kTopVals;
  for (uint32_t k = threadIdx.x; k < 3 * kTopBins * kTopVals; k += blockDim.x) {
    const uint32_t v = k % kTopVals;
    if (v == 0) {
      if (sb[k]) atomicAdd(g + k, sb[k]);
    } else if (((v - 1) % 6) < 3) {
      atomicMin(g + k, sb[k]);
    } else {
      atomicMax(g + k, sb[k]);
    }
  }
}

__device__ __forceinline__ float box_half_area(float lx, float ly, float lz, float hx, float hy, float hz) {
  const float dx = hx - lx, dy = hy - ly, dz = hz - lz;
  return dx * dy + dy * dz + dz * dx;
}

// One warp: the split of least SAH cost A_L N_L + A_R N_R over the task's
// bins B ([axis][bin][kTopVals], shared or global memory); writes the split,
// the node's box and its triangle count. Lanes b and b + 16 hold bin b of
// the axis in hand; prefix and suffix unions of the bins come from shuffles
// within the 16 lanes. Among equal costs the lowest (axis, bin) wins, the
// split a sweep over the axes and bins in order with a strict comparison
// takes. Bins with no triangle carry no box (their encoded fields would
// decode to NaN).
__device__ void warp_top_split(const uint32_t* B, const TopTask& T, TopSplit* __restrict__ split,
                               BinNode* __restrict__ box, uint32_t* __restrict__ count) {
  const uint32_t lane = threadIdx.x & 31u, b = lane & 15u;
  const uint32_t n = T.end - T.begin;
  float best = FLT_MAX;
  uint32_t best_idx = 0xffffffffu, best_lc = 0;
  float bl[3], bh[3], rl_best[3], rh_best[3];
  float nlo[3], nhi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) bl[k] = bh[k] = rl_best[k] = rh_best[k] = nlo[k] = nhi[k] = 0.f;
  for (int ax = 0; ax < 3; ++ax) {
    const uint32_t* V = B + (ax * kTopBins + b) * kTopVals;
    const uint32_t c = V[0];
    float pl[3], ph[3], sl[3], sh[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      pl[k] = sl[k] = c ? o2f(V[1 + k]) : FLT_MAX;
      ph[k] = sh[k] = c ? o2f(V[4 + k]) : -FLT_MAX;
    }
    uint32_t pc = c, sc = c;
#pragma unroll
    for (int o = 1; o < kTopBins; o <<= 1) {  // inclusive prefix (bins 0..b) and suffix (bins b..15)
      const uint32_t yp = __shfl_up_sync(0xffffffffu, pc, o, kTopBins);
      const uint32_t ys = __shfl_down_sync(0xffffffffu, sc, o, kTopBins);
      float ypl[3], yph[3], ysl[3], ysh[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        ypl[k] = __shfl_up_sync(0xffffffffu, pl[k], o, kTopBins);
        yph[k] = __shfl_up_sync(0xffffffffu, ph[k], o, kTopBins);
        ysl[k] = __shfl_down_sync(0xffffffffu, sl[k], o, kTopBins);
        ysh[k] = __shfl_down_sync(0xffffffffu, sh[k], o, kTopBins);
      }
      if (b >= (uint32_t)o) {
        pc += yp;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          pl[k] = fminf(pl[k], ypl[k]);
          ph[k] = fmaxf(ph[k], yph[k]);
        }
      }
      if (b + (uint32_t)o < (uint32_t)kTopBins) {
        sc += ys;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          sl[k] = fminf(sl[k], ysl[k]);
          sh[k] = fmaxf(sh[k], ysh[k]);
        }
      }
    }
    // the right side of a split after bin b: the suffix from bin b + 1
    const uint32_t rc = __shfl_down_sync(0xffffffffu, sc, 1, kTopBins);
    float rl[3], rh[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      rl[k] = __shfl_down_sync(0xffffffffu, sl[k], 1, kTopBins);
      rh[k] = __shfl_down_sync(0xffffffffu, sh[k], 1, kTopBins);
    }
    if (ax == 0) {  // the node's box: the union of all bins of one axis
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        nlo[k] = __shfl_sync(0xffffffffu, sl[k], 0, kTopBins);
        nhi[k] = __shfl_sync(0xffffffffu, sh[k], 0, kTopBins);
      }
    }
    if (b + 1 < (uint32_t)kTopBins && pc != 0 && rc != 0) {
      const float cost = box_half_area(pl[0], pl[1], pl[2], ph[0], ph[1], ph[2]) * (float)pc +
                         box_half_area(rl[0], rl[1], rl[2], rh[0], rh[1], rh[2]) * (float)rc;
      if (cost < best) {
        best = cost;
        best_idx = (uint32_t)ax * kTopBins + b;
        best_lc = pc;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          bl[k] = pl[k];
          bh[k] = ph[k];
          rl_best[k] = rl[k];
          rh_best[k] = rh[k];
        }
      }
    }
  }
  // lowest (cost, axis, bin) over the warp
  float wc = best;
  uint32_t wi = best_idx;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oc = __shfl_xor_sync(0xffffffffu, wc, o);
    const uint32_t oi = __shfl_xor_sync(0xffffffffu, wi, o);
    if (oc < wc || (oc == wc && oi < wi)) {
      wc = oc;
      wi = oi;
    }
  }
  if (wi == 0xffffffffu) {  // no usable SAH split: split by position
    if (lane == 0) {
      TopSplit S;
      S.axis = 3;
      S.bin = 0;
      S.nleft = n / 2;
      S.pad = 0;
      S.task[0] = S.task[1] = 0;
      S.pad2[0] = S.pad2[1] = 0;
      S.lclo = S.rclo = T.clo;
      S.lchi = S.rchi = T.chi;
      *split = S;
    }
  } else if (lane < (uint32_t)kTopBins && best_idx == wi) {
    TopSplit S;
    S.axis = wi / kTopBins;
    S.bin = wi % kTopBins;
    S.nleft = best_lc;
    S.pad = 0;
    S.task[0] = S.task[1] = 0;
    S.pad2[0] = S.pad2[1] = 0;
    S.lclo = make_float4(bl[0], bl[1], bl[2], 0.f);
    S.lchi = make_float4(bh[0], bh[1], bh[2], 0.f);
    S.rclo = make_float4(rl_best[0], rl_best[1], rl_best[2], 0.f);
    S.rchi = make_float4(rh_best[0], rh_best[1], rh_best[2], 0.f);
    *split = S;
  }
  if (lane == 0) {
    box[T.node].lo = make_float4(nlo[0], nlo[1], nlo[2], 0.f);
    box[T.node].hi = make_float4(nhi[0], nhi[1], nhi[2], 0.f);
    count[T.node] = n;
  }
}

// one warp bins task T (index t) into its shared bins `my` and splits it
__device__ __forceinline__ void top_bin_warp_task(const uint32_t* __restrict__ ord, const float4* __restrict__ blo,
                                                       const float4* __restrict__ bhi, const TopTask& T, uint32_t t,
                                                       uint32_t* my, uint32_t lane, TopSplit* __restrict__ splits,
                                                       BinNode* __restrict__ box, uint32_t* __restrict__ count,
                                                       uint16_t* __restrict__ code) {
  for (uint32_t k = lane; k < 3 * kTopBins * kTopVals; k += 32) {
    const uint32_t v = k % kTopVals;
    my[k] = v == 0 ? 0u : (((v - 1) % 6) < 3 ? 0xffffffffu : 0u);
  }
  __syncwarp();
  for (uint32_t p = T.begin + lane; p < T.end; p += 32) {
    const uint32_t tri = ord[p];
    const float4 lo = blo[tri], hi = bhi[tri];
    const float4 c = make_float4(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z), 0.f);
    const int bins3[3] = {top_bin(c.x, T.clo.x, T.chi.x), top_bin(c.y, T.clo.y, T.chi.y),
                          top_bin(c.z, T.clo.z, T.chi.z)};
    code[p] = (uint16_t)(bins3[0] | (bins3[1] << 4) | (bins3[2] << 8));
    const uint32_t v[6] = {f2o(lo.x), f2o(lo.y), f2o(lo.z), f2o(hi.x), f2o(hi.y), f2o(hi.z)};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      uint32_t* b = my + (ax * kTopBins + bins3[ax]) * kTopVals;
      atomicAdd(b, 1u);
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        if (k < 3)
          atomicMin(b + 1 + k, v[k]);
        else
          atomicMax(b + 1 + k, v[k]);
      }
    }
  }
  __syncwarp();
  warp_top_split(my, T, splits + t, box, count);
  __syncwarp();  // the split has read the bins before the warp's next task resets them
}

// tasks of at most kTopWarpTask triangles: one warp bins a whole task into
// its own shared-memory bins with per-lane shared atomics, then splits it
// from those bins (its bins never go to global memory)
__global__ void __launch_bounds__(256) k_top_bin_warp(const uint32_t* __restrict__ ord, const float4* __restrict__ blo,
                                                      const float4* __restrict__ bhi, const TopTask* __restrict__ tasks,
                                                      const uint32_t* __restrict__ n_tasks_p,
                                                      TopSplit* __restrict__ splits, BinNode* __restrict__ box,
                                                      uint32_t* __restrict__ count, uint16_t* __restrict__ code) {
  __shared__ uint32_t sb[8][3 * kTopBins * kTopVals];
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  const uint32_t n_tasks = *n_tasks_p;
  // whole warps take tasks together (a warp-stride loop over the level's tasks)
  for (uint32_t t = blockIdx.x * 8u + warp; t < n_tasks; t += gridDim.x * 8u) {
    const TopTask T = tasks[t];
    if (T.end - T.begin > kTopWarpTask) continue;
    top_bin_warp_task(ord, blo, bhi, T, t, sb[warp], lane, splits, box, count, code);
  }
}

// one warp per task larger than kTopWarpTask (the smaller ones were split
// by k_top_bin_warp from their shared-memory bins)
__global__ void __launch_bounds__(128) k_top_split(const TopTask* __restrict__ tasks,
                                                   const uint32_t* __restrict__ n_tasks_p,
                                                   const uint32_t* __restrict__ max_task_p,
                                                   const uint32_t* __restrict__ bins, TopSplit* __restrict__ splits,
                                                   BinNode* __restrict__ box, uint32_t* __restrict__ count) {
  if (*max_task_p <= kTopWarpTask) return;
  const uint32_t n_tasks = *n_tasks_p;
  for (uint32_t t = blockIdx.x * 4u + (threadIdx.x >> 5); t < n_tasks; t += gridDim.x * 4u) {  // whole warps
    const TopTask T = tasks[t];
    if (T.end - T.begin <= kTopWarpTask) continue;
    warp_top_split(bins + (size_t)t * 3 * kTopBins * kTopVals, T, splits + t, box, count);
  }
}

// 1 if position p (of task t) goes left: its bin on the split axis (the
// bin codes that binning wrote: 4 bits per axis) is at most the split bin,
// or, for a split by position, it lies in the first nleft positions
__device__ __forceinline__ uint32_t top_goes_left(uint32_t p, uint32_t code, const TopTask& T, const TopSplit& S) {
  if (S.axis < 3) return ((code >> (4 * S.axis)) & 15u) <= S.bin ? 1u : 0u;
  return (p - T.begin) < S.nleft ? 1u : 0u;
}

// the flags of the stable partition and the first phase of their exclusive
// scan in one pass: each chunk of 1024 positions (256 threads x 4) scans its
// flags into pscan and writes its total to sums (scanned by k_scan_sums;
// k_top_scatter adds a chunk's offset itself)
__global__ void __launch_bounds__(256) k_top_flag_scan(const uint32_t* __restrict__ task_of,
                                                       const uint16_t* __restrict__ code,
                                                       const TopTask* __restrict__ tasks,
                                                       const TopSplit* __restrict__ splits,
                                                       const uint32_t* __restrict__ n_tasks_p, uint32_t n,
                                                       uint32_t* __restrict__ pscan, uint32_t* __restrict__ sums) {
  __shared__ uint32_t wsum[8];
  const uint32_t n_tasks = *n_tasks_p;
  if (n_tasks == 0) return;  // no level
  const uint32_t base = blockIdx.x * 1024u + threadIdx.x * 4u;
  uint32_t f[4] = {0u, 0u, 0u, 0u}, tk[4] = {kNoTask, kNoTask, kNoTask, kNoTask}, cd[4] = {0u, 0u, 0u, 0u};
  if (base + 3 < n) {  // task_of, code: 16- and 8-byte aligned groups of 4
    const uint4 t4 = *reinterpret_cast<const uint4*>(task_of + base);
    const uint2 c4 = *reinterpret_cast<const uint2*>(code + base);
    tk[0] = t4.x, tk[1] = t4.y, tk[2] = t4.z, tk[3] = t4.w;
    cd[0] = c4.x & 0xffffu, cd[1] = c4.x >> 16, cd[2] = c4.y & 0xffffu, cd[3] = c4.y >> 16;
  } else {
    for (uint32_t k = 0; k < 4 && base + k < n; ++k) {
      tk[k] = task_of[base + k];
      cd[k] = code[base + k];
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (tk[k] < n_tasks) f[k] = top_goes_left(base + k, cd[k], tasks[tk[k]], splits[tk[k]]);
  const uint32_t tot = f[0] + f[1] + f[2] + f[3];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t inc = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= (uint32_t)o) inc += y;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  uint32_t woff = 0, all = 0;
#pragma unroll
  for (uint32_t w = 0; w < 8; ++w) {
    const uint32_t x = wsum[w];
    woff += w < warp ? x : 0u;
    all += x;
  }
  const uint32_t e = woff + inc - tot;
  const uint4 o4 = make_uint4(e, e + f[0], e + f[0] + f[1], e + f[0] + f[1] + f[2]);
  if (base + 3 < n) {
    *reinterpret_cast<uint4*>(pscan + base) = o4;
  } else {
    if (base < n) pscan[base] = o4.x;
    if (base + 1 < n) pscan[base + 1] = o4.y;
    if (base + 2 < n) pscan[base + 2] = o4.z;
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = all;
}

// stable partition of every active task's range: the lefts before p within
// its task are the exclusive scan (chunk scan + chunk offset) at p minus that
// at the task's first position; task_of2 gets each position's task of the
// next level
__global__ void __launch_bounds__(256) k_top_scatter(const uint32_t* __restrict__ ord, uint32_t* __restrict__ ord2,
                                                     const uint32_t* __restrict__ task_of,
                                                     uint32_t* __restrict__ task_of2, const uint16_t* __restrict__ code,
                                                     const TopTask* __restrict__ tasks,
                                                     const TopSplit* __restrict__ splits,
                                                     const uint32_t* __restrict__ n_tasks_p,
                                                     const uint32_t* __restrict__ pscan,
                                                     const uint32_t* __restrict__ sums, uint32_t n, uint32_t* status) {
  const uint32_t n_tasks = *n_tasks_p;
  if (n_tasks == 0) return;  // no level: the order stays where it is
  // 4 consecutive positions per thread (one chunk of the scan: base is a multiple of 4)
  const uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) * 4u;
  if (base >= n) return;
  uint32_t tk[4] = {kNoTask, kNoTask, kNoTask, kNoTask}, cd[4] = {0u, 0u, 0u, 0u}, ps[4] = {0u, 0u, 0u, 0u},
           od[4] = {0u, 0u, 0u, 0u};
  const uint32_t m = min(4u, n - base);
  if (m == 4) {
    const uint4 t4 = *reinterpret_cast<const uint4*>(task_of + base);
    const uint2 c4 = *reinterpret_cast<const uint2*>(code + base);
    const uint4 p4 = *reinterpret_cast<const uint4*>(pscan + base);
    const uint4 o4 = *reinterpret_cast<const uint4*>(ord + base);
    tk[0] = t4.x, tk[1] = t4.y, tk[2] = t4.z, tk[3] = t4.w;
    cd[0] = c4.x & 0xffffu, cd[1] = c4.x >> 16, cd[2] = c4.y & 0xffffu, cd[3] = c4.y >> 16;
    ps[0] = p4.x, ps[1] = p4.y, ps[2] = p4.z, ps[3] = p4.w;
    od[0] = o4.x, od[1] = o4.y, od[2] = o4.z, od[3] = o4.w;
  } else {
    for (uint32_t k = 0; k < m; ++k) {
      tk[k] = task_of[base + k];
      cd[k] = code[base + k];
      ps[k] = pscan[base + k];
      od[k] = ord[base + k];
    }
  }
  const uint32_t chunk_off = sums[base >> 10];
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k) {
    if (k >= m) break;
    const uint32_t p = base + k, t = tk[k];
    uint32_t d = p, next = kNoTask;
    if (t < n_tasks) {
      const TopTask T = tasks[t];
      const TopSplit S = splits[t];
      const uint32_t f = top_goes_left(p, cd[k], T, S);
      // lefts before p within its task: the exclusive scan at p minus that at the task's first position
      const uint32_t l = (ps[k] + chunk_off) - (pscan[T.begin] + sums[T.begin >> 10]);
      d = f ? T.begin + l : T.begin + S.nleft + (p - T.begin - l);
      next = S.task[f ? 0 : 1];
      if (d < T.begin || d >= T.end) {
        atomicOr(status, J3DG_DEV_BAD_INDEX);
        continue;
      }
    }
    ord2[d] = od[k];
    task_of2[d] = next;
  }
}

// children of every task: a new task above J3DG_SAH_TOP triangles, else a
// finished range (segment) whose root PLOC supplies later
__device__ __forceinline__ void top_children_of(const TopTask* __restrict__ tasks, TopSplit* __restrict__ splits,
                                                uint32_t t, uint32_t seg_max, uint32_t* __restrict__ counters,
                                                TopTask* __restrict__ next, TopRange* __restrict__ ranges,
                                                uint2* __restrict__ child, uint32_t cap_tasks, uint32_t cap_ranges,
                                                uint32_t max_nodes, uint32_t* status) {
  const TopTask T = tasks[t];
  TopSplit S = splits[t];
  const uint32_t n = T.end - T.begin;
  uint32_t nl = S.nleft;
  if (nl == 0 || nl >= n) {  // cannot happen (both sides of a split are non-empty); kept safe
    atomicOr(status, J3DG_DEV_BAD_INDEX);
    nl = n / 2;
    S.axis = 3;
    S.nleft = nl;
  }
  const uint32_t mid = T.begin + nl;
  uint32_t ref[2];
  S.task[0] = S.task[1] = kNoTask;
  for (int side = 0; side < 2; ++side) {
    const uint32_t b = side ? mid : T.begin, e = side ? T.end : mid;
    if (e - b > seg_max) {
      const uint32_t q = atomicAdd(counters + 1, 1u);
      const uint32_t node = atomicAdd(counters + 0, 1u);
      if (q >= cap_tasks || node >= max_nodes) {
        atomicOr(status, J3DG_DEV_BAD_INDEX);
        ref[side] = kPendingRef;
        continue;
      }
      atomicMax(counters + 3, e - b);  // the next level's largest task
      TopTask C;
      C.begin = b;
      C.end = e;
      C.node = node;
      C.pad = 0;
      C.clo = side ? S.rclo : S.lclo;
      C.chi = side ? S.rchi : S.lchi;
      next[q] = C;
      ref[side] = node;
      S.task[side] = q;
    } else {
      const uint32_t q = atomicAdd(counters + 2, 1u);
      if (q < cap_ranges)
        ranges[q] = TopRange{b, e, T.node, (uint32_t)side};
      else
        atomicOr(status, J3DG_DEV_BAD_INDEX);
      ref[side] = kPendingRef;
    }
  }
  child[T.node] = make_uint2(ref[0], ref[1]);
  splits[t] = S;
}

__global__ void k_top_children(const TopTask* __restrict__ tasks, TopSplit* __restrict__ splits,
                               const uint32_t* __restrict__ n_tasks_p, uint32_t seg_max,
                               uint32_t* __restrict__ counters, TopTask* __restrict__ next,
                               TopRange* __restrict__ ranges, uint2* __restrict__ child, uint32_t cap_tasks,
                               uint32_t cap_ranges, uint32_t max_nodes, uint32_t* status) {
  // counters: [0] nodes allocated, [1] next tasks, [2] ranges, [3] largest next task
  const uint32_t n_tasks = *n_tasks_p;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_tasks; t += gridDim.x * blockDim.x)
    top_children_of(tasks, splits, t, seg_max, counters, next, ranges, child, cap_tasks, cap_ranges, max_nodes,
                    status);
}

__global__ void k_iota(uint32_t* __restrict__ a, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = i;
}

// segment starts: flags[begin] = 1 for every finished range
__global__ void k_top_seg_starts(const TopRange* __restrict__ ranges, const uint32_t* __restrict__ n_ranges_p,
                                 uint32_t n, uint32_t* __restrict__ flags) {
  const uint32_t n_ranges = *n_ranges_p;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n_ranges; r += gridDim.x * blockDim.x)
    if (ranges[r].begin < n) flags[ranges[r].begin] = 1u;
}

// PLOC's initial clusters in the order `ord`, with the segment of each position
// (seg = inclusive scan of the starts - 1)
__global__ void k_ploc_init_seg(const float4* __restrict__ tris, const uint32_t* __restrict__ ord_a,
                                const uint32_t* __restrict__ ord_b, const uint32_t* __restrict__ parity, uint32_t n,
                                const uint32_t* __restrict__ starts, const uint32_t* __restrict__ scan,
                                uint32_t* __restrict__ C, float4* __restrict__ lo, float4* __restrict__ hi,
                                uint32_t* __restrict__ seg) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t t = (*parity ? ord_b : ord_a)[i];  // the final order is where the last level put it
  C[i] = 0x80000000u | t;
  leaf_box(tris, t, lo[i], hi[i]);
  seg[i] = scan[i] + starts[i] - 1u;
}

// the root of segment s (its one cluster left, at list position s) fills the
// child slot of the top node that made the segment
// (the clusters are in C0 or C1, by the parity of the PLOC rounds run)
__global__ void k_top_link(const TopRange* __restrict__ ranges, const uint32_t* __restrict__ n_ranges_p,
                           const uint32_t* __restrict__ starts, const uint32_t* __restrict__ scan,
                           const uint32_t* __restrict__ C0, const uint32_t* __restrict__ C1,
                           const uint32_t* __restrict__ parity, const uint32_t* __restrict__ n_seg_p,
                           uint2* __restrict__ child, uint32_t* status) {
  const uint32_t n_ranges = *n_ranges_p, n_seg = *n_seg_p;
  const uint32_t* C = *parity ? C1 : C0;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n_ranges; r += gridDim.x * blockDim.x) {
    const TopRange R = ranges[r];
    const uint32_t s = scan[R.begin] + starts[R.begin] - 1u;
    if (s >= n_seg) {
      atomicOr(status, J3DG_DEV_BAD_INDEX);
      continue;
    }
    if (R.side)
      child[R.parent].y = C[s];
    else
      child[R.parent].x = C[s];
  }
}

// ------------------------------------------------------------- driver ----

#define J3DG_CK(x)                                             \
  do {                                                         \
    cudaError_t e_ = (x);                                      \
    if (e_ != cudaSuccess) {                                   \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);   \
      rc = J3DG_ERR_CUDA;                                      \
      goto cleanup;                                            \
    }                                                          \
  } while (0)

// slot_of[id] = leaf position of triangle id (ids are a permutation of 0..nt)
__global__ void k_slot_of(const float4* __restrict__ tris, uint32_t nt, uint32_t* __restrict__ slot_of,
                          uint32_t* status) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  const uint32_t id = __float_as_uint(tris[3 * (size_t)i].w);
  if (id >= nt) {
    atomicOr(status, J3DG_DEV_BAD_INDEX);
    return;
  }
  slot_of[id] = i;
}

// stream-ordered free of a scratch buffer as soon as it is dead (keeps the
// build's peak device memory down); the pointer is cleared for the cleanup
#define J3DG_DROP(p)             \
  do {                           \
    if (p) cudaFreeAsync(p, st); \
    p = nullptr;                 \
  } while (0)

// ------------------------------------------------ device-driven build ----
//
// A build (the default: binned-SAH top levels, PLOC below them, the
// cost-optimal collapse; or the LBVH: the one-pass tree and its collapse;
// then the depth-first numbering) runs as one CUDA graph with no host round
// trip: every level loop is a conditional while node whose
// body ends in a one-thread step kernel, which advances the loop state kept
// in device memory (BuildCtl) and sets the loop's condition. Kernels read
// their sizes from BuildCtl and stride over them with fixed grids, so one
// captured sequence serves every level. Loops whose levels alternate two
// buffers run two levels per body (the second is a no-op when the first
// ends the loop). enqueue_build only enqueues (it runs under a stream
// capture): j3dg_mesh_build captures and launches it for one mesh, and a
// batch captures it for all its meshes ahead of its frames.

static const uint32_t kMaxTopLevels = 1024, kMaxRounds = 1024, kMaxPlaceLevels = 128;

struct BuildCtl {
  uint32_t top_ctr[4];  // k_top_children: [0] top nodes, [1] next level's tasks, [2] ranges, [3] largest next task
                        // (LBVH: [0] the root that k_lbvh found)
  uint32_t n_tasks, max_task, ord_parity, top_levels;
  uint32_t mcount, n_seg, node_base, c_parity, rounds, tot[2];
  uint32_t lohi[2];  // the running pass's node range (collapse costs, depth-first levels)
  uint32_t pass, n_pass;
  uint32_t n_in, n_out, n_wide, place_levels, max_depth;
  int32_t dfs_level;
  uint32_t error;  // a loop overran its bound: 1 SAH levels, 2 PLOC, 4 placement / collapse
  uint32_t top_end[kMaxTopLevels];     // top nodes of level L end at top_end[L]
  uint32_t round_end[kMaxRounds];      // binary nodes of PLOC round r end at round_end[r]
  uint32_t level_end[kMaxPlaceLevels]; // wide nodes of level L end at level_end[L]
};

__global__ void k_ctl_init(BuildCtl* __restrict__ c, TopTask* __restrict__ tasks, const float* __restrict__ bb,
                           uint32_t nt, uint32_t top) {
  if (top) {
    TopTask r0;
    r0.begin = 0;
    r0.end = nt;
    r0.node = 0;
    r0.pad = 0;
    r0.clo = make_float4(bb[0], bb[1], bb[2], 0.f);  // the vertex bbox holds every centroid
    r0.chi = make_float4(bb[3], bb[4], bb[5], 0.f);
    tasks[0] = r0;
    c->top_ctr[0] = 1;  // the root node
    c->n_tasks = 1;
    c->max_task = nt;
    c->top_levels = 1;
    c->top_end[0] = 1;
  }
  c->mcount = nt;
  c->n_seg = 1;
  c->n_in = 1;  // the placement's root item
  c->n_wide = 1;
  c->place_levels = 1;
  c->level_end[0] = 1;
}

__global__ void k_top_step(BuildCtl* __restrict__ c, uint32_t cap_tasks, uint32_t nt, cudaGraphConditionalHandle h,
                           uint32_t set) {
  if (c->n_tasks) {  // the level ran
    uint32_t next = c->top_ctr[1];
    if (next > cap_tasks || c->top_ctr[2] > nt || c->top_ctr[0] > nt - 1 || c->top_levels >= kMaxTopLevels) {
      c->error |= 1u;
      next = 0;
    } else if (c->top_ctr[0] > c->top_end[c->top_levels - 1]) {
      c->top_end[c->top_levels++] = c->top_ctr[0];
    }
    c->n_tasks = next;
    c->max_task = c->top_ctr[3];
    c->top_ctr[1] = 0;
    c->top_ctr[3] = 0;
    c->ord_parity ^= 1u;
  }
  if (set) cudaGraphSetConditional(h, c->n_tasks > 0 ? 1u : 0u);
}

__global__ void k_ploc_setup(BuildCtl* __restrict__ c) {  // after the SAH levels: one segment per range
  c->n_seg = c->top_ctr[2];
  c->node_base = c->top_ctr[0];
}

__global__ void k_ploc_step(BuildCtl* __restrict__ c, uint32_t nt, cudaGraphConditionalHandle h, uint32_t set) {
  if (c->mcount > c->n_seg) {  // the round ran
    const uint32_t creates = c->tot[0], surv = c->tot[1];
    if (creates == 0 || surv >= c->mcount || c->node_base + creates > nt - 1 || c->rounds >= kMaxRounds) {
      c->error |= 2u;  // no progress or past the node bound
      c->mcount = c->n_seg;
    } else {
      c->node_base += creates;
      c->round_end[c->rounds++] = c->node_base;
      c->mcount = surv;
      c->c_parity ^= 1u;
    }
  }
  if (set) cudaGraphSetConditional(h, c->mcount > c->n_seg ? 1u : 0u);
}

// pass p of the cost programme: the PLOC rounds in order, then the top levels
// deepest first (children before parents)
__device__ __forceinline__ void cost_range(BuildCtl* c, uint32_t p, uint32_t top) {
  uint32_t lo = 0, hi = 0;
  if (p < c->rounds) {
    lo = p ? c->round_end[p - 1] : (top ? c->top_ctr[0] : 0u);
    hi = c->round_end[p];
  } else if (p < c->n_pass) {
    const uint32_t k = c->top_levels - 1 - (p - c->rounds);
    lo = k ? c->top_end[k - 1] : 0u;
    hi = c->top_end[k];
  }
  c->lohi[0] = lo;
  c->lohi[1] = hi;
}

__global__ void k_ploc_done(BuildCtl* __restrict__ c, uint32_t nt, uint32_t top, const uint32_t* __restrict__ C0,
                            const uint32_t* __restrict__ C1, PlaceItem* __restrict__ qa) {
  const uint32_t root = top ? 0u : (c->c_parity ? C1 : C0)[0];
  if (c->node_base != nt - 1 || (root & 0x80000000u)) c->error |= 2u;  // a malformed tree
  qa[0] = PlaceItem{root, 0u, 1u, 0u};
  c->n_pass = c->rounds + (top ? c->top_levels : 0u);
  c->pass = 0;
  cost_range(c, 0, top);
}

__global__ void k_cost_step(BuildCtl* __restrict__ c, uint32_t top, cudaGraphConditionalHandle h, uint32_t set) {
  ++c->pass;
  cost_range(c, c->pass, top);  // past the last pass: an empty range
  if (set) cudaGraphSetConditional(h, c->pass < c->n_pass ? 1u : 0u);
}

__global__ void k_place_step(BuildCtl* __restrict__ c, uint32_t nt, cudaGraphConditionalHandle h, uint32_t set) {
  if (c->n_in) {  // the level ran
    const uint32_t n_out = c->n_out;
    c->n_wide += n_out;
    if (c->n_wide > nt || c->place_levels >= kMaxPlaceLevels) {
      c->error |= 4u;
      c->n_in = 0;
    } else {
      if (n_out) c->level_end[c->place_levels++] = c->n_wide;
      c->n_in = n_out;
    }
    c->n_out = 0;
  }
  if (set) cudaGraphSetConditional(h, c->n_in > 0 ? 1u : 0u);
}

__device__ __forceinline__ void level_range(BuildCtl* c, int32_t l) {
  const bool ok = l >= 0 && l < (int32_t)c->place_levels;
  c->lohi[0] = ok && l > 0 ? c->level_end[l - 1] : 0u;
  c->lohi[1] = ok ? c->level_end[l] : 0u;
}

__global__ void k_dfs_setup(BuildCtl* __restrict__ c, uint32_t* __restrict__ pos, uint32_t up) {
  if (!up) {  // subtree sizes, deepest level first
    c->dfs_level = (int32_t)c->place_levels - 1;
  } else {  // positions, root level first
    c->dfs_level = 0;
    pos[0] = 0;
  }
  level_range(c, c->dfs_level);
}

__global__ void k_dfs_step(BuildCtl* __restrict__ c, uint32_t up, cudaGraphConditionalHandle h, uint32_t set) {
  c->dfs_level += up ? 1 : -1;
  level_range(c, c->dfs_level);  // past the last level: an empty range
  if (set) cudaGraphSetConditional(h, (c->dfs_level >= 0 && c->dfs_level < (int32_t)c->place_levels) ? 1u : 0u);
}

// the LBVH's collapse starts at the root that k_lbvh left in top_ctr[0]
__global__ void k_lbvh_root(BuildCtl* __restrict__ c, CollapseItem* __restrict__ qa) {
  qa[0] = CollapseItem{c->top_ctr[0], 0u, 1u};
}

// after an LBVH collapse level: k_collapse allocated its wide nodes itself
__global__ void k_lbvh_step(BuildCtl* __restrict__ c, uint32_t nt, cudaGraphConditionalHandle h, uint32_t set) {
  if (c->n_in) {  // the level ran
    if (c->n_wide > nt || c->n_out > nt || c->place_levels >= kMaxPlaceLevels) {
      c->error |= 4u;
      c->n_in = 0;
    } else {
      if (c->n_wide > c->level_end[c->place_levels - 1]) c->level_end[c->place_levels++] = c->n_wide;
      c->n_in = c->n_out;
    }
    c->n_out = 0;
  }
  if (set) cudaGraphSetConditional(h, c->n_in > 0 ? 1u : 0u);
}

// Appends a while node (condition initially 1) to the graph that `st` is
// capturing; `body(side, handle)` enqueues the loop body on `side`, which
// captures it into the node's body graph.
template <class Body>
static cudaError_t capture_while(cudaStream_t st, cudaStream_t side, Body&& body) {
  cudaStreamCaptureStatus cs;
  unsigned long long id = 0;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, &id, &g, &deps, nullptr, &nd);
  if (e != cudaSuccess) return e;
  if (cs != cudaStreamCaptureStatusActive) return cudaErrorStreamCaptureUnsupported;
  cudaGraphConditionalHandle h;
  if ((e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if ((e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &p)) != cudaSuccess) return e;
  if ((e = cudaStreamBeginCaptureToGraph(side, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return e;
  body(side, h);
  const cudaError_t eb = cudaGetLastError();
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(side, &captured);
  if (eb != cudaSuccess) return eb;
  if (e != cudaSuccess) return e;
  return cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

// Every buffer of one build, sized by the triangle count alone (upper bounds
// where the tree decides: the wide nodes, the queues).
struct BuildPlan {
  uint32_t nv = 0, nt = 0, W = 4, leaf = 2;
  bool top = false;   // binned-SAH top levels (the default builder, large meshes)
  bool lbvh = false;  // this build is an LBVH (J3DG_BUILD_LBVH)
  // the builders the scratch serves: PLOC (the default) and / or LBVH (a
  // batch's rebuild lane may serve both)
  bool need_ploc = true, need_lbvh = false;
  // scratch
  float* part = nullptr;
  float* bb = nullptr;
  uint64_t *k0 = nullptr, *k1 = nullptr;
  uint32_t *v0 = nullptr, *v1 = nullptr, *hist = nullptr, *sums = nullptr;
  uint32_t *ord_a = nullptr, *ord_b = nullptr, *task_of = nullptr, *task_of2 = nullptr, *seg_starts = nullptr,
           *seg_scan = nullptr, *top_bins = nullptr;
  float4 *tbox_lo = nullptr, *tbox_hi = nullptr;
  uint16_t* codes = nullptr;
  TopTask *tasks_a = nullptr, *tasks_b = nullptr;
  TopSplit* splits = nullptr;
  TopRange* ranges = nullptr;
  uint2* child = nullptr;
  BinNode* box = nullptr;
  uint32_t *count = nullptr, *C0 = nullptr, *C1 = nullptr, *nn = nullptr, *cscan = nullptr, *sscan = nullptr,
           *pl_sums = nullptr, *pl_sums2 = nullptr, *seg0 = nullptr, *seg1 = nullptr;
  float4 *lo0 = nullptr, *hi0 = nullptr, *lo1 = nullptr, *hi1 = nullptr;
  float* dp_cost = nullptr;
  uint8_t* dp_dec = nullptr;
  float4* wide = nullptr;
  PlaceItem *pa = nullptr, *pb = nullptr;
  uint2* range = nullptr;  // LBVH: each binary node's leaf range
  CollapseItem *qa = nullptr, *qb = nullptr;
  uint32_t *dfs_size = nullptr, *dfs_pos = nullptr;
  BuildCtl* ctl = nullptr;
  // outputs (the mesh keeps them)
  float4 *normals = nullptr, *soup = nullptr, *tris_out = nullptr, *nodes = nullptr;
  uint32_t* slot_of = nullptr;
  uint32_t cap_tasks() const { return nt / J3DG_SAH_TOP + 1; }  // tasks of one level are disjoint, each > J3DG_SAH_TOP
  uint32_t n_tiles() const { return (nt + kSortTile - 1) / kSortTile; }
  uint32_t hist_n() const { return 256 * n_tiles(); }
  uint32_t scan_blocks() const { return (hist_n() + 1023) / 1024; }
  uint32_t sblocks() const { return (nt + 1023) / 1024; }
};

static const int kBBoxBlocks = 1024;

// outputs: the mesh's arrays too (else the mesh's own: a rebuild in place);
// node_bound: with them, a node array at the size bound (rebuildable meshes;
// other builds write the nodes into an array of the tree's size at the end)
static cudaError_t plan_alloc(BuildPlan& P, cudaStream_t st, bool outputs = true, bool node_bound = true) {
  const size_t nt = P.nt, F4 = J3DG_NODE_F4(P.W);
  cudaError_t e = cudaSuccess;
  auto A = [&](auto*& p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&p, bytes, st);
  };
  A(P.part, sizeof(float) * 6 * kBBoxBlocks);
  A(P.bb, sizeof(float) * 6);
  A(P.k0, sizeof(uint64_t) * nt);
  A(P.k1, sizeof(uint64_t) * nt);
  A(P.v0, sizeof(uint32_t) * nt);
  A(P.v1, sizeof(uint32_t) * nt);
  A(P.hist, sizeof(uint32_t) * P.hist_n());
  A(P.sums, sizeof(uint32_t) * (P.scan_blocks() + 1));
  if (P.top) {
    A(P.ord_a, sizeof(uint32_t) * nt);
    A(P.ord_b, sizeof(uint32_t) * nt);
    A(P.task_of, sizeof(uint32_t) * nt);
    A(P.task_of2, sizeof(uint32_t) * nt);
    A(P.tbox_lo, sizeof(float4) * nt);
    A(P.tbox_hi, sizeof(float4) * nt);
    A(P.codes, sizeof(uint16_t) * nt);
    A(P.seg_starts, sizeof(uint32_t) * nt);
    A(P.seg_scan, sizeof(uint32_t) * nt);
    A(P.top_bins, sizeof(uint32_t) * (size_t)P.cap_tasks() * 3 * kTopBins * kTopVals);
    A(P.tasks_a, sizeof(TopTask) * P.cap_tasks());
    A(P.tasks_b, sizeof(TopTask) * P.cap_tasks());
    A(P.splits, sizeof(TopSplit) * P.cap_tasks());
    A(P.ranges, sizeof(TopRange) * nt);  // at most one range per triangle
  }
  A(P.child, sizeof(uint2) * (nt - 1));
  A(P.box, sizeof(BinNode) * (nt - 1));
  A(P.count, sizeof(uint32_t) * (nt - 1));  // LBVH: the sibling handshake of k_lbvh
  if (P.need_ploc) {
    A(P.C0, sizeof(uint32_t) * nt);
    A(P.C1, sizeof(uint32_t) * nt);
    A(P.nn, sizeof(uint32_t) * nt);
    A(P.cscan, sizeof(uint32_t) * nt);
    A(P.sscan, sizeof(uint32_t) * nt);
    A(P.pl_sums, sizeof(uint32_t) * (P.sblocks() + 1));
    A(P.pl_sums2, sizeof(uint32_t) * (P.sblocks() + 1));
    A(P.seg0, sizeof(uint32_t) * nt);
    A(P.seg1, sizeof(uint32_t) * nt);
    A(P.lo0, sizeof(float4) * nt);
    A(P.hi0, sizeof(float4) * nt);
    A(P.lo1, sizeof(float4) * nt);
    A(P.hi1, sizeof(float4) * nt);
    A(P.dp_cost, sizeof(float) * P.W * (nt - 1));
    A(P.dp_dec, sizeof(uint8_t) * P.W * (nt - 1));
    A(P.pa, sizeof(PlaceItem) * nt);
    A(P.pb, sizeof(PlaceItem) * nt);
    A(P.soup, sizeof(float4) * 3 * nt);  // the LBVH gathers straight into the leaf order
  }
  if (P.need_lbvh) {
    A(P.range, sizeof(uint2) * (nt - 1));
    A(P.qa, sizeof(CollapseItem) * nt);
    A(P.qb, sizeof(CollapseItem) * nt);
  }
  A(P.wide, sizeof(float4) * F4 * nt);
  A(P.dfs_size, sizeof(uint32_t) * nt);
  A(P.dfs_pos, sizeof(uint32_t) * nt);
  A(P.ctl, sizeof(BuildCtl));
  if (outputs) {  // else the mesh's own arrays (a rebuild in place)
    A(P.normals, sizeof(float4) * nt);
    A(P.tris_out, sizeof(float4) * 3 * nt);
    if (node_bound) A(P.nodes, sizeof(float4) * F4 * nt);  // the wide nodes are at most nt - 1
    A(P.slot_of, sizeof(uint32_t) * nt);
  }
  return e;
}

// frees the scratch (outputs the caller took over are null)
static void plan_free(BuildPlan& P, cudaStream_t st) {
  void* ps[] = {P.part, P.bb, P.k0, P.k1, P.v0, P.v1, P.hist, P.sums, P.ord_a, P.ord_b, P.task_of, P.task_of2,
                P.seg_starts, P.seg_scan, P.top_bins, P.tbox_lo, P.tbox_hi, P.codes, P.tasks_a, P.tasks_b, P.splits,
                P.ranges, P.child, P.box, P.count, P.C0, P.C1, P.nn, P.cscan, P.sscan, P.pl_sums, P.pl_sums2, P.seg0,
                P.seg1, P.lo0, P.hi0, P.lo1, P.hi1, P.dp_cost, P.dp_dec, P.wide, P.pa, P.pb, P.range, P.qa, P.qb,
                P.dfs_size, P.dfs_pos, P.ctl, P.normals, P.soup, P.tris_out, P.nodes, P.slot_of};
  for (void* p : ps)
    if (p) cudaFreeAsync(p, st);
  P = BuildPlan{};
}

#define J3DG_EQ(x)                                \
  do {                                            \
    if (e == cudaSuccess) e = (x);                \
    if (e == cudaSuccess) e = cudaGetLastError(); \
  } while (0)

// the default builder's binary tree and wide nodes (P.wide, level ranges in
// c->level_end): binned-SAH top levels over PLOC ranges (or PLOC alone), the
// cost programme, the placement; the leaf-ordered triangles go to P.tris_out
static cudaError_t enqueue_tree_ploc(BuildPlan& P, cudaStream_t st, cudaStream_t side, uint32_t* d_status) {
  const uint32_t nt = P.nt, W = P.W;
  BuildCtl* c = P.ctl;
  cudaError_t e = cudaSuccess;
  const float4* soup = P.soup;
  if (P.top) {
    k_top_boxes<<<(nt + 255) / 256, 256, 0, st>>>(soup, nt, P.tbox_lo, P.tbox_hi);
    k_iota<<<(nt + 255) / 256, 256, 0, st>>>(P.ord_a, nt);
    J3DG_EQ(cudaMemsetAsync(P.task_of, 0, sizeof(uint32_t) * nt, st));
    // one SAH level: tasks ti, order oi, task of each position si -> the next level's
    auto level = [&](cudaStream_t s, TopTask* ti, TopTask* to, uint32_t* oi, uint32_t* oo, uint32_t* si,
                     uint32_t* so) {
      k_top_bins_init<<<kStrideBlocks, 256, 0, s>>>(P.top_bins, &c->n_tasks, &c->max_task, ti);
      k_top_bin<<<(nt + kTopChunk - 1) / kTopChunk, 256, 0, s>>>(oi, P.tbox_lo, P.tbox_hi, si, ti, &c->n_tasks,
                                                                 &c->max_task, nt, P.top_bins, P.codes);
      k_top_bin_warp<<<kStrideBlocks, 256, 0, s>>>(oi, P.tbox_lo, P.tbox_hi, ti, &c->n_tasks, P.splits, P.box,
                                                   P.count, P.codes);
      k_top_split<<<kStrideBlocks, 128, 0, s>>>(ti, &c->n_tasks, &c->max_task, P.top_bins, P.splits, P.box, P.count);
      k_top_children<<<kStrideBlocks, 128, 0, s>>>(ti, P.splits, &c->n_tasks, J3DG_SAH_TOP, c->top_ctr, to, P.ranges,
                                                   P.child, P.cap_tasks(), nt, nt - 1, d_status);
      k_top_flag_scan<<<P.sblocks(), 256, 0, s>>>(si, P.codes, ti, P.splits, &c->n_tasks, nt, P.cscan, P.pl_sums);
      k_scan_sums<<<1, 1024, 0, s>>>(P.pl_sums, nullptr, P.sblocks(), nullptr);
      k_top_scatter<<<(nt + 1023) / 1024, 256, 0, s>>>(oi, oo, si, so, P.codes, ti, P.splits, &c->n_tasks, P.cscan,
                                                       P.pl_sums, nt, d_status);
    };
    J3DG_EQ(capture_while(st, side, [&](cudaStream_t s, cudaGraphConditionalHandle h) {
      level(s, P.tasks_a, P.tasks_b, P.ord_a, P.ord_b, P.task_of, P.task_of2);
      k_top_step<<<1, 1, 0, s>>>(c, P.cap_tasks(), nt, h, 0u);
      level(s, P.tasks_b, P.tasks_a, P.ord_b, P.ord_a, P.task_of2, P.task_of);
      k_top_step<<<1, 1, 0, s>>>(c, P.cap_tasks(), nt, h, 1u);
    }));
    k_ploc_setup<<<1, 1, 0, st>>>(c);
    // segments numbered in position order: a flag at each range's start, one scan
    J3DG_EQ(cudaMemsetAsync(P.seg_starts, 0, sizeof(uint32_t) * nt, st));
    k_top_seg_starts<<<kStrideBlocks, 256, 0, st>>>(P.ranges, &c->top_ctr[2], nt, P.seg_starts);
    k_scan_chunks<<<P.sblocks(), 256, 0, st>>>(P.seg_starts, P.seg_scan, nt, P.pl_sums);
    k_scan_sums<<<1, 1024, 0, st>>>(P.pl_sums, nullptr, P.sblocks(), nullptr);
    k_scan_add<<<P.sblocks(), 256, 0, st>>>(P.seg_scan, nt, P.pl_sums);
    k_ploc_init_seg<<<(nt + 255) / 256, 256, 0, st>>>(soup, P.ord_a, P.ord_b, &c->ord_parity, nt, P.seg_starts,
                                                      P.seg_scan, P.C0, P.lo0, P.hi0, P.seg0);
  } else {
    k_ploc_init<<<(nt + 255) / 256, 256, 0, st>>>(soup, nt, P.C0, P.lo0, P.hi0);
    J3DG_EQ(cudaMemsetAsync(P.seg0, 0, sizeof(uint32_t) * nt, st));
  }
  J3DG_EQ(cudaSuccess);
  // PLOC rounds: clusters (C, lo, hi, seg) in -> out
  auto round = [&](cudaStream_t s, const uint32_t* Ci, const float4* li, const float4* hi_, const uint32_t* si,
                   uint32_t* Co, float4* lo_, float4* ho, uint32_t* so) {
    k_ploc_nn<<<kStrideBlocks, kPlocBlock, 0, s>>>(li, hi_, si, &c->mcount, &c->n_seg, P.nn);
    k_ploc_flag_scan<<<P.sblocks(), 256, 0, s>>>(P.nn, &c->mcount, &c->n_seg, P.cscan, P.sscan, P.pl_sums,
                                                 P.pl_sums2);
    k_scan_sums<<<1, 1024, 0, s>>>(P.pl_sums, P.pl_sums2, 0u, c->tot, &c->mcount);
    k_ploc_merge<<<kStrideBlocks, 256, 0, s>>>(Ci, li, hi_, si, P.nn, P.cscan, P.sscan, P.pl_sums, P.pl_sums2,
                                               &c->mcount, &c->n_seg, &c->node_base, Co, lo_, ho, so, P.child, P.box,
                                               P.count);
  };
  J3DG_EQ(capture_while(st, side, [&](cudaStream_t s, cudaGraphConditionalHandle h) {
    round(s, P.C0, P.lo0, P.hi0, P.seg0, P.C1, P.lo1, P.hi1, P.seg1);
    k_ploc_step<<<1, 1, 0, s>>>(c, nt, h, 0u);
    round(s, P.C1, P.lo1, P.hi1, P.seg1, P.C0, P.lo0, P.hi0, P.seg0);
    k_ploc_step<<<1, 1, 0, s>>>(c, nt, h, 1u);
  }));
  if (P.top)
    k_top_link<<<kStrideBlocks, 256, 0, st>>>(P.ranges, &c->top_ctr[2], P.seg_starts, P.seg_scan, P.C0, P.C1,
                                              &c->c_parity, &c->n_seg, P.child, d_status);
  k_ploc_done<<<1, 1, 0, st>>>(c, nt, P.top ? 1u : 0u, P.C0, P.C1, P.pa);
  J3DG_EQ(cudaSuccess);
  // cost programme, children before parents
  J3DG_EQ(capture_while(st, side, [&](cudaStream_t s, cudaGraphConditionalHandle h) {
    launch_collapse_cost(W, P.child, P.box, P.count, soup, c->lohi, P.leaf, P.dp_cost, P.dp_dec, s);
    k_cost_step<<<1, 1, 0, s>>>(c, P.top ? 1u : 0u, h, 0u);
    launch_collapse_cost(W, P.child, P.box, P.count, soup, c->lohi, P.leaf, P.dp_cost, P.dp_dec, s);
    k_cost_step<<<1, 1, 0, s>>>(c, P.top ? 1u : 0u, h, 1u);
  }));
  // placement, level by level
  J3DG_EQ(capture_while(st, side, [&](cudaStream_t s, cudaGraphConditionalHandle h) {
    launch_collapse_place(W, P.child, P.box, P.count, soup, P.pa, &c->n_in, P.pb, &c->n_out, &c->n_wide, P.wide,
                          P.leaf, &c->max_depth, P.tris_out, nt, d_status, P.dp_dec, s);
    k_place_step<<<1, 1, 0, s>>>(c, nt, h, 0u);
    launch_collapse_place(W, P.child, P.box, P.count, soup, P.pb, &c->n_in, P.pa, &c->n_out, &c->n_wide, P.wide,
                          P.leaf, &c->max_depth, P.tris_out, nt, d_status, P.dp_dec, s);
    k_place_step<<<1, 1, 0, s>>>(c, nt, h, 1u);
  }));
  return e;
}

// the LBVH (J3DG_BUILD_LBVH): Apetrei's one-pass binary tree over the sorted
// Morton codes, then the 4-wide collapse level by level; the triangles are
// already in leaf order (P.tris_out)
static cudaError_t enqueue_tree_lbvh(BuildPlan& P, const uint64_t* keys, cudaStream_t st, cudaStream_t side,
                                     uint32_t* d_status) {
  const uint32_t nt = P.nt;
  BuildCtl* c = P.ctl;
  cudaError_t e = cudaSuccess;
  J3DG_EQ(cudaMemsetAsync(P.count, 0xff, sizeof(uint32_t) * (nt - 1), st));
  k_lbvh<<<(nt + 255) / 256, 256, 0, st>>>(keys, P.tris_out, nt, P.child, P.box, P.range, P.count, &c->top_ctr[0]);
  k_lbvh_root<<<1, 1, 0, st>>>(c, P.qa);
  J3DG_EQ(cudaSuccess);
  J3DG_EQ(capture_while(st, side, [&](cudaStream_t s, cudaGraphConditionalHandle h) {
    k_collapse<<<wave_blocks128(), 128, 0, s>>>(P.child, P.box, P.range, P.tris_out, P.qa, &c->n_in, P.qb, &c->n_out,
                                             &c->n_wide, P.wide, nt, P.leaf, &c->max_depth, d_status);
    k_lbvh_step<<<1, 1, 0, s>>>(c, nt, h, 0u);
    k_collapse<<<wave_blocks128(), 128, 0, s>>>(P.child, P.box, P.range, P.tris_out, P.qb, &c->n_in, P.qa, &c->n_out,
                                             &c->n_wide, P.wide, nt, P.leaf, &c->max_depth, d_status);
    k_lbvh_step<<<1, 1, 0, s>>>(c, nt, h, 1u);
  }));
  return e;
}

// the sorted Morton codes after the radix passes (they alternate k0 / k1)
static const uint64_t* sorted_keys(const BuildPlan& P) { return (kRadixPasses & 1) ? P.k1 : P.k0; }

// A build's first part, whose launches do not depend on the tree: the loop
// state reset, the bounding box, normals and Morton codes, the radix sort
// and the gather into Morton order. No host synchronisation.
static cudaError_t enqueue_prefix(BuildPlan& P, const float* dV, const uint32_t* dT, cudaStream_t st,
                                  uint32_t* d_status) {
  const uint32_t nt = P.nt, nv = P.nv;
  BuildCtl* c = P.ctl;
  cudaError_t e = cudaSuccess;
  J3DG_EQ(cudaMemsetAsync(c, 0, sizeof(BuildCtl), st));
  k_bbox_partial<<<kBBoxBlocks, 256, 0, st>>>(dV, nv, P.part);
  k_bbox_final<<<1, 32, 0, st>>>(P.part, kBBoxBlocks, P.bb);
  k_ctl_init<<<1, 1, 0, st>>>(c, P.tasks_a, P.bb, nt, P.top ? 1u : 0u);
  k_tri_prep<<<(nt + 255) / 256, 256, 0, st>>>(dV, nv, dT, nt, P.bb, P.normals, P.k0, P.v0, d_status);
  J3DG_EQ(cudaSuccess);
  {
    uint64_t *ka = P.k0, *kb = P.k1;
    uint32_t *va = P.v0, *vb = P.v1;
    for (int pass = 0; pass < kRadixPasses; ++pass) {
      const int shift = 8 * pass;
      k_radix_hist<<<P.n_tiles(), kSortThreads, 0, st>>>(ka, nt, shift, P.n_tiles(), P.hist);
      k_scan_chunks<<<P.scan_blocks(), 256, 0, st>>>(P.hist, P.hist, P.hist_n(), P.sums);
      k_scan_sums<<<1, 1024, 0, st>>>(P.sums, nullptr, P.scan_blocks(), nullptr);
      k_radix_scatter<<<P.n_tiles(), kSortThreads, 0, st>>>(ka, va, kb, vb, nt, shift, P.n_tiles(), P.hist, P.sums,
                                                           d_status);
      std::swap(ka, kb);
      std::swap(va, vb);
    }
    k_soup<<<(nt + 255) / 256, 256, 0, st>>>(dV, dT, va, nt, nv, P.lbvh ? P.tris_out : P.soup, d_status);
  }
  J3DG_EQ(cudaSuccess);
  return e;
}

// The rest: the tree, its wide nodes, the depth-first numbering (and, with
// `permute`, the nodes written in that order into P.nodes) and the
// triangles' slots; its level loops are conditional while nodes, so `st`
// must be capturing.
static cudaError_t enqueue_tree(BuildPlan& P, cudaStream_t st, cudaStream_t side, uint32_t* d_status,
                                bool permute = true) {
  const uint32_t nt = P.nt, W = P.W;
  BuildCtl* c = P.ctl;
  cudaError_t e = cudaSuccess;
  J3DG_EQ(P.lbvh ? enqueue_tree_lbvh(P, sorted_keys(P), st, side, d_status)
                 : enqueue_tree_ploc(P, st, side, d_status));
  // depth-first numbering: subtree sizes bottom-up, positions top-down, permute
  auto dfs = [&](auto Wc) {
    constexpr int WW = decltype(Wc)::value;
    k_dfs_setup<<<1, 1, 0, st>>>(c, P.dfs_pos, 0u);
    J3DG_EQ(capture_while(st, side, [&](cudaStream_t s, cudaGraphConditionalHandle h) {
      k_dfs_size<WW><<<kStrideBlocks, 256, 0, s>>>(P.wide, c->lohi, P.dfs_size);
      k_dfs_step<<<1, 1, 0, s>>>(c, 0u, h, 0u);
      k_dfs_size<WW><<<kStrideBlocks, 256, 0, s>>>(P.wide, c->lohi, P.dfs_size);
      k_dfs_step<<<1, 1, 0, s>>>(c, 0u, h, 1u);
    }));
    k_dfs_setup<<<1, 1, 0, st>>>(c, P.dfs_pos, 1u);
    J3DG_EQ(capture_while(st, side, [&](cudaStream_t s, cudaGraphConditionalHandle h) {
      k_dfs_place<WW><<<kStrideBlocks, 256, 0, s>>>(P.wide, c->lohi, P.dfs_size, P.dfs_pos);
      k_dfs_step<<<1, 1, 0, s>>>(c, 1u, h, 0u);
      k_dfs_place<WW><<<kStrideBlocks, 256, 0, s>>>(P.wide, c->lohi, P.dfs_size, P.dfs_pos);
      k_dfs_step<<<1, 1, 0, s>>>(c, 1u, h, 1u);
    }));
    if (permute) k_dfs_permute<WW><<<(nt + 255) / 256, 256, 0, st>>>(P.wide, &c->n_wide, P.dfs_pos, P.nodes);
  };
  if (W == 2)
    dfs(std::integral_constant<int, 2>());
  else if (W == 8)
    dfs(std::integral_constant<int, 8>());
  else
    dfs(std::integral_constant<int, 4>());
  k_slot_of<<<(nt + 255) / 256, 256, 0, st>>>(P.tris_out, nt, P.slot_of, d_status);
  J3DG_EQ(cudaSuccess);
  return e;
}

// all of a build's work on `st` (capturing)
static cudaError_t enqueue_build(BuildPlan& P, const float* dV, const uint32_t* dT, cudaStream_t st,
                                 cudaStream_t side, uint32_t* d_status) {
  cudaError_t e = cudaSuccess;
  J3DG_EQ(enqueue_prefix(P, dV, dT, st, d_status));
  J3DG_EQ(enqueue_tree(P, st, side, d_status));
  return e;
}
#undef J3DG_EQ

// A build through the device-driven graph: allocate, enqueue the prefix
// (the GPU sorts while the host captures and instantiates the rest), capture
// the tree's part, launch it, then take the tree's size from the device and
// keep an exactly sized copy of the nodes.
static int build_bvh_graph(j3dg_mesh* m, const float* dV, const uint32_t* dT, cudaStream_t st, uint32_t* d_status,
                           cudaEvent_t done, std::string& err) {
  BuildPlan P;
  P.nv = m->nv;
  P.nt = m->nt;
  P.W = m->width;
  P.leaf = m->leaf_size;
  P.lbvh = (m->build_flags & J3DG_BUILD_LBVH) != 0;
  P.need_ploc = !P.lbvh;
  P.need_lbvh = P.lbvh;
  P.top = !P.lbvh && J3DG_SAH_TOP > 0 && m->nt > J3DG_SAH_TOP;
  cudaStream_t side = nullptr;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ex = nullptr;
  BuildCtl h;
  float hbb[6];
  int rc = J3DG_OK;
  cudaError_t e = plan_alloc(P, st, true, (m->build_flags & J3DG_BUILD_REBUILDABLE) != 0);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = enqueue_prefix(P, dV, dT, st, d_status);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    const cudaError_t eq = enqueue_tree(P, st, side, d_status, false);
    e = cudaStreamEndCapture(st, &g);
    if (eq != cudaSuccess) e = eq;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(ex, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, P.ctl, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hbb, P.bb, sizeof(hbb), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    err = std::string("build: ") + cudaGetErrorString(e);
    rc = e == cudaErrorMemoryAllocation ? J3DG_ERR_OUT_OF_MEMORY : J3DG_ERR_CUDA;
  } else if (h.error) {
    err = (h.error & 1u) ? "SAH top levels overran their bounds"
                         : ((h.error & 2u) ? "PLOC clustering ended with a malformed tree"
                                           : "BVH collapse overran its node bound");
    rc = J3DG_ERR_CUDA;
  }
  if (rc == J3DG_OK) {
    m->scale = 0.f;
    for (int k = 0; k < 3; ++k) {
      m->min_bb[k] = hbb[k];
      m->max_bb[k] = hbb[3 + k];
    }
    for (int k = 0; k < 6; ++k) m->scale = std::max(m->scale, std::fabs(hbb[k]));
    m->n_nodes = h.n_wide;
    m->max_depth = h.max_depth;
    m->root_ref = 0;
    // the nodes in depth-first order into an array of the tree's size (a
    // rebuildable mesh keeps the array at the size bound: rebuilds write in
    // place)
    const size_t bytes = sizeof(float4) * J3DG_NODE_F4(P.W) * (size_t)m->n_nodes;
    if (m->build_flags & J3DG_BUILD_REBUILDABLE) {
      m->d_nodes = P.nodes;
      P.nodes = nullptr;
    } else {
      e = cudaMallocAsync(&m->d_nodes, bytes ? bytes : sizeof(float4) * J3DG_NODE_F4(P.W), st);
    }
    if (e == cudaSuccess) {
      float4* out = (float4*)m->d_nodes;
      const uint32_t grid = (m->n_nodes + 255) / 256;
      if (grid) {
        if (P.W == 2)
          k_dfs_permute<2><<<grid, 256, 0, st>>>(P.wide, &P.ctl->n_wide, P.dfs_pos, out);
        else if (P.W == 8)
          k_dfs_permute<8><<<grid, 256, 0, st>>>(P.wide, &P.ctl->n_wide, P.dfs_pos, out);
        else
          k_dfs_permute<4><<<grid, 256, 0, st>>>(P.wide, &P.ctl->n_wide, P.dfs_pos, out);
        e = cudaGetLastError();
      }
    }
    if (e == cudaSuccess && done) e = cudaEventRecord(done, st);  // the BVH is ready; the rest is clean-up
    if (e == cudaSuccess) {
      m->d_normals = P.normals;
      m->d_tris = P.tris_out;
      m->d_slot_of = P.slot_of;
      P.normals = nullptr;
      P.tris_out = nullptr;
      P.slot_of = nullptr;
    } else {
      err = std::string("build: ") + cudaGetErrorString(e);
      rc = e == cudaErrorMemoryAllocation ? J3DG_ERR_OUT_OF_MEMORY : J3DG_ERR_CUDA;
    }
  }
  plan_free(P, st);
  if (ex) cudaGraphExecDestroy(ex);
  if (g) cudaGraphDestroy(g);
  if (side) cudaStreamDestroy(side);
  {
    const cudaError_t es = cudaStreamSynchronize(st);
    if (rc == J3DG_OK && es != cudaSuccess) {
      err = std::string("build: ") + cudaGetErrorString(es);
      rc = J3DG_ERR_CUDA;
    }
  }
  if (rc != J3DG_OK) return rc;
  const uint32_t W = m->width;
  if (m->max_depth > J3DG_MAX_DEPTH_W(W)) {
    err = "BVH depth " + std::to_string(m->max_depth) + " exceeds the traversal stack at width " + std::to_string(W);
    return J3DG_ERR_UNSUPPORTED;
  }
  m->device_bytes = sizeof(float4) * J3DG_NODE_F4(W) *
                        (uint64_t)((m->build_flags & J3DG_BUILD_REBUILDABLE) ? m->nt : (m->n_nodes ? m->n_nodes : 1)) +
                    sizeof(float4) * 4 * (uint64_t)m->nt + sizeof(uint32_t) * 4 * (uint64_t)m->nt;
  return J3DG_OK;
}

// ---------------------------------------------------- batch rebuilds ----
//
// A batch's graph rebuilds its meshes in place: each lane (a forked capture
// stream) owns one build's scratch, sized for its largest mesh, and builds
// its meshes one after another into their own arrays.

struct RebuildLane {
  BuildPlan P;  // scratch only; nt = the lane's largest mesh
};

int rebuild_lane_alloc(uint32_t nt_max, uint32_t nv_max, uint32_t W, bool ploc, bool lbvh, cudaStream_t st,
                       RebuildLane** out, std::string& err) {
  RebuildLane* L = new (std::nothrow) RebuildLane();
  if (!L) return J3DG_ERR_OUT_OF_MEMORY;
  L->P.nt = nt_max;
  L->P.nv = nv_max;
  L->P.W = W;
  L->P.need_ploc = ploc;
  L->P.need_lbvh = lbvh;
  L->P.top = ploc && J3DG_SAH_TOP > 0 && nt_max > J3DG_SAH_TOP;
  const cudaError_t e = plan_alloc(L->P, st, false);
  if (e != cudaSuccess) {
    plan_free(L->P, st);
    delete L;
    err = std::string("batch rebuild scratch: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? J3DG_ERR_OUT_OF_MEMORY : J3DG_ERR_CUDA;
  }
  *out = L;
  return J3DG_OK;
}

void rebuild_lane_free(RebuildLane* L, cudaStream_t st) {
  if (!L) return;
  plan_free(L->P, st);
  delete L;
}

// enqueues (under a capture) the rebuild of mesh m into its own arrays
cudaError_t rebuild_enqueue(RebuildLane* L, const j3dg_mesh* m, cudaStream_t st, cudaStream_t side, uint32_t* d_status) {
  if (m->nt <= m->leaf_size) return cudaSuccess;  // one leaf: nothing to rebuild
  BuildPlan Pm = L->P;  // the lane's scratch, this mesh's sizes and arrays
  Pm.nt = m->nt;
  Pm.nv = m->nv;
  Pm.leaf = m->leaf_size;
  Pm.lbvh = (m->build_flags & J3DG_BUILD_LBVH) != 0;
  Pm.top = !Pm.lbvh && J3DG_SAH_TOP > 0 && m->nt > J3DG_SAH_TOP;
  if (Pm.lbvh ? !Pm.need_lbvh : !Pm.need_ploc) return cudaErrorInvalidValue;  // the lane has no scratch for it
  Pm.normals = (float4*)m->d_normals;
  Pm.tris_out = (float4*)m->d_tris;
  Pm.nodes = (float4*)m->d_nodes;
  Pm.slot_of = (uint32_t*)m->d_slot_of;
  return enqueue_build(Pm, (const float*)m->d_verts, (const uint32_t*)m->d_index, st, side, d_status);
}

// Builds the device BVH. dV and dT are device arrays. On success fills the
// mesh fields (bbox, scale, nodes, leaf-ordered triangles, normals); `done`
// (may be null) is recorded on st once the BVH is ready, before the host's
// clean-up (the build time is taken up to it). Both builders go through
// build_bvh_graph; a mesh of at most one leaf is built here.
int build_bvh(j3dg_mesh* m, const float* dV, const uint32_t* dT, cudaStream_t st, uint32_t* d_status,
              cudaEvent_t done, std::string& err) {
  if (m->nt > m->leaf_size) return build_bvh_graph(m, dV, dT, st, d_status, done, err);
  int rc = J3DG_OK;
  const uint32_t nv = m->nv, nt = m->nt;
  float* d_part = nullptr;
  float* d_bb = nullptr;
  uint64_t* k0 = nullptr;
  uint32_t* v0 = nullptr;
  const int bbox_blocks = 1024;
  float hbb[6];
  const uint32_t W = m->width;
  const size_t F4 = J3DG_NODE_F4(W);

  J3DG_CK(cudaMallocAsync((void**)&d_part, sizeof(float) * 6 * bbox_blocks, st));
  J3DG_CK(cudaMallocAsync((void**)&d_bb, sizeof(float) * 6, st));
  k_bbox_partial<<<bbox_blocks, 256, 0, st>>>(dV, nv, d_part);
  k_bbox_final<<<1, 32, 0, st>>>(d_part, bbox_blocks, d_bb);
  J3DG_CK(cudaGetLastError());
  J3DG_CK(cudaMemcpyAsync(hbb, d_bb, sizeof(hbb), cudaMemcpyDeviceToHost, st));
  J3DG_CK(cudaStreamSynchronize(st));
  m->scale = 0.f;
  for (int k = 0; k < 3; ++k) {
    m->min_bb[k] = hbb[k];
    m->max_bb[k] = hbb[3 + k];
  }
  for (int k = 0; k < 6; ++k) m->scale = std::max(m->scale, std::fabs(hbb[k]));

  // the triangles in input order (a single leaf), their normals; the root
  // is the leaf and the node array one empty node
  J3DG_CK(cudaMallocAsync(&m->d_normals, sizeof(float4) * (size_t)nt, st));
  J3DG_CK(cudaMallocAsync(&m->d_tris, sizeof(float4) * 3 * (size_t)nt, st));
  J3DG_CK(cudaMallocAsync((void**)&k0, sizeof(uint64_t) * nt, st));
  J3DG_CK(cudaMallocAsync((void**)&v0, sizeof(uint32_t) * nt, st));
  k_tri_prep<<<1, 256, 0, st>>>(dV, nv, dT, nt, d_bb, (float4*)m->d_normals, k0, v0, d_status);  // v0[i] = i
  k_soup<<<1, 256, 0, st>>>(dV, dT, v0, nt, nv, (float4*)m->d_tris, d_status);
  J3DG_CK(cudaGetLastError());
  m->root_ref = J3DG_LEAF_BIT | (nt - 1u);
  m->n_nodes = 0;
  m->max_depth = 0;
  J3DG_CK(cudaMallocAsync(&m->d_nodes, sizeof(float4) * F4, st));
  J3DG_CK(cudaMemsetAsync(m->d_nodes, 0, sizeof(float4) * F4, st));
  J3DG_CK(cudaMallocAsync(&m->d_slot_of, sizeof(uint32_t) * (size_t)nt, st));
  k_slot_of<<<1, 256, 0, st>>>((const float4*)m->d_tris, nt, (uint32_t*)m->d_slot_of, d_status);
  J3DG_CK(cudaGetLastError());
  if (done) J3DG_CK(cudaEventRecord(done, st));

cleanup:
  if (d_part) cudaFreeAsync(d_part, st);
  if (d_bb) cudaFreeAsync(d_bb, st);
  if (k0) cudaFreeAsync(k0, st);
  if (v0) cudaFreeAsync(v0, st);
  {
    cudaError_t e = cudaStreamSynchronize(st);
    if (rc == J3DG_OK && e != cudaSuccess) {
      err = std::string("build: ") + cudaGetErrorString(e);
      rc = J3DG_ERR_CUDA;
    }
  }
  if (rc != J3DG_OK) return rc;
  m->device_bytes = sizeof(float4) * F4 + sizeof(float4) * 4 * (uint64_t)nt + sizeof(uint32_t) * 4 * (uint64_t)nt;
  return J3DG_OK;
}

}  // namespace j3dg
