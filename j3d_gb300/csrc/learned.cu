// learned.cu -- learned tmax for closest-hit traversal.
//
// A small network maps a ray (origin, direction) to a cluster of the mesh:
// 16-band Fourier features of the 6 ray coordinates (192 values, padded to
// 256), four 128-wide GELU layers, 4096 cluster logits; bf16 weights, fp32
// accumulation on the tcgen05 tensor cores (the GEMMs with fused epilogues
// of umma_gemm.cu for training, one fused kernel for inference), trained
// with softmax cross-entropy and Adam on rays traced by the plain method.
// Clusters are the BVH4 subtrees at a fixed depth (depth 6: at most 4096),
// which are Morton-ordered ranges of the mesh because the tree is an LBVH.
//
// A learned query traverses the two most likely clusters first; their
// closest accepted hit seeds the exact traversal of the whole tree as its
// best (t, triangle) so far, which only prunes: the final hit is the same
// (bit for bit) as the plain traversal's.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <new>
#include <string>
#include <vector>

#include "../../include/j3dg.h"
#include "device_common.cuh"
#include "internal.h"
#include "mlp.cuh"
#include "umma.cuh"

namespace j3dg {
int ray_query_device(j3dg_ctx* c, const j3dg_mesh* mesh, const j3dg_ray* d_rays, uint32_t n, j3dg_hit* d_hits);
int mesh_devinst(j3dg_ctx* c, const j3dg_mesh* mesh, const DevInst** out);
int ctx_fail(j3dg_ctx* c, int code, const std::string& msg);
unsigned long long* ctx_counters(j3dg_ctx* c);
}

namespace j3dg {

static const int kIn = 256;        // 192 Fourier features + zero padding
static const int kHid = 128;
static const int kOut = 4096;
static const int kBands = 16;

// parameter offsets in the flat vectors (W row-major [in][out])
struct Layout {
  size_t w[5], b[5], total;
  int in[5], out[5];
  Layout() {
    const int ins[5] = {kIn, kHid, kHid, kHid, kHid}, outs[5] = {kHid, kHid, kHid, kHid, kOut};
    size_t o = 0;
    for (int l = 0; l < 5; ++l) {
      in[l] = ins[l];
      out[l] = outs[l];
      w[l] = o;
      o += (size_t)ins[l] * outs[l];
      b[l] = o;
      o += outs[l];
    }
    total = o;
  }
};

// ------------------------------------------------------------------ kernels

// Fourier features of (origin, direction): x_i = ((o - c) / s, d / |d|),
// sin / cos of pi 2^(k/4) x_i for k = 0..15; features [i][k][sin, cos].
__device__ __forceinline__ void ray_inputs(const j3dg_ray* ray, float cx, float cy, float cz, float inv_s,
                                           float (&in6)[6]) {
  const float* f = reinterpret_cast<const float*>(ray);
  const float dl = rsqrtf(f[4] * f[4] + f[5] * f[5] + f[6] * f[6] + 1e-30f);
  in6[0] = (f[0] - cx) * inv_s;
  in6[1] = (f[1] - cy) * inv_s;
  in6[2] = (f[2] - cz) * inv_s;
  in6[3] = f[4] * dl;
  in6[4] = f[5] * dl;
  in6[5] = f[6] * dl;
}

__device__ __forceinline__ uint32_t bits2(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t*>(&v); }

// Frequencies pi 2^(q/4), q = 0..3, of the first octave of bands; band
// k = 4 o + q has frequency 2^o times band q's, so its sine and cosine come
// from band q's by o angle doublings (sin 2a = 2 sin a cos a, cos 2a =
// (cos a - sin a)(cos a + sin a)). The first octave uses the hardware sine /
// cosine (__sincosf: absolute error ~1e-5 at the arguments here), and the
// doublings keep the error far below the bf16 rounding the features get.
// Training and inference compute the features with these same functions.
__device__ __forceinline__ void base_octave(float x, float (&s)[4], float (&c)[4]) {
  const float fr[4] = {0x1.921fb6p+1f, 0x1.de3564p+1f, 0x1.1c5832p+2f, 0x1.5225p+2f};
#pragma unroll
  for (int q = 0; q < 4; ++q) __sincosf(fr[q] * x, &s[q], &c[q]);
}
__device__ __forceinline__ void next_octave(float (&s)[4], float (&c)[4]) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float s2 = 2.f * s[q] * c[q], c2 = (c[q] - s[q]) * (c[q] + s[q]);
    s[q] = s2;
    c[q] = c2;
  }
}
// the 4 feature pairs (sin, cos as bf16) of one octave: 16 bytes of a row
__device__ __forceinline__ uint4 octave_pairs(const float (&s)[4], const float (&c)[4]) {
  return make_uint4(bits2(__floats2bfloat162_rn(s[0], c[0])), bits2(__floats2bfloat162_rn(s[1], c[1])),
                    bits2(__floats2bfloat162_rn(s[2], c[2])), bits2(__floats2bfloat162_rn(s[3], c[3])));
}

// features of ray r: coordinate i, band k at pair i * 16 + k (columns: sin,
// cos); zeros from column 192 to 255
__global__ void k_features(const j3dg_ray* __restrict__ rays, uint32_t n, uint32_t n_pad, float cx, float cy,
                           float cz, float inv_s, __nv_bfloat16* __restrict__ X) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_pad) return;
  uint4* x = reinterpret_cast<uint4*>(X + (size_t)r * kIn);
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  if (r >= n) {
    for (int j = 0; j < kIn / 8; ++j) x[j] = zero;
    return;
  }
  float in6[6];
  ray_inputs(rays + r, cx, cy, cz, inv_s, in6);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    float sn[4], cn[4];
    base_octave(in6[i], sn, cn);
#pragma unroll
    for (int o = 0; o < 4; ++o) {
      x[i * 4 + o] = octave_pairs(sn, cn);
      if (o < 3) next_octave(sn, cn);
    }
  }
  for (int j = 24; j < kIn / 8; ++j) x[j] = zero;
}

// Softmax cross-entropy over the first K logits of each row; rows with
// label < 0 contribute nothing. dlogits = (softmax - onehot) / n_valid.
__global__ void k_softmax_ce(const float* __restrict__ logits, const int32_t* __restrict__ labels, uint32_t rows,
                             uint32_t K, float inv_valid, __nv_bfloat16* __restrict__ dlogits,
                             float* __restrict__ loss, uint32_t* __restrict__ correct) {
  const uint32_t row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const uint32_t lane = threadIdx.x & 31;
  if (row >= rows) return;
  const float* z = logits + (size_t)row * kOut;
  __nv_bfloat16* dz = dlogits + (size_t)row * kOut;
  const int32_t lab = labels[row];
  if (lab < 0) {
    for (uint32_t j = lane; j < kOut; j += 32) dz[j] = __float2bfloat16(0.f);
    return;
  }
  float mx = -FLT_MAX;
  uint32_t arg = 0;
  for (uint32_t j = lane; j < K; j += 32)
    if (z[j] > mx) {
      mx = z[j];
      arg = j;
    }
  for (int o = 16; o > 0; o >>= 1) {
    const float om = __shfl_xor_sync(0xffffffffu, mx, o);
    const uint32_t oa = __shfl_xor_sync(0xffffffffu, arg, o);
    if (om > mx || (om == mx && oa < arg)) {
      mx = om;
      arg = oa;
    }
  }
  float sum = 0.f;
  for (uint32_t j = lane; j < K; j += 32) sum += __expf(z[j] - mx);
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  const float inv = 1.f / sum;
  for (uint32_t j = lane; j < kOut; j += 32) {
    float g = 0.f;
    if (j < K) g = __expf(z[j] - mx) * inv - (j == (uint32_t)lab ? 1.f : 0.f);
    dz[j] = __float2bfloat16(g * inv_valid);
  }
  if (lane == 0) {
    atomicAdd(loss, logf(sum) - (z[lab] - mx));
    if (arg == (uint32_t)lab) atomicAdd(correct, 1u);
  }
}

// column sums of a bf16 [rows x cols] matrix into fp32 `out` (zeroed by the
// caller): blockIdx.y takes a chunk of 128 rows, atomics combine the chunks
__global__ void k_colsum(const __nv_bfloat16* __restrict__ M, uint32_t rows, uint32_t cols, float* __restrict__ out) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const uint32_t r0 = blockIdx.y * 128u, r1 = min(rows, r0 + 128u);
  float s = 0.f;
  for (uint32_t r = r0; r < r1; ++r) s += __bfloat162float(M[(size_t)r * cols + c]);
  atomicAdd(out + c, s);
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       __nv_bfloat16* __restrict__ pb, size_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  p[i] = pi;
  pb[i] = __float2bfloat16(pi);
}

// dst[c * ldd + r] = src[r * lds + c] for r < rows, c < cols (32 x 32 tiles
// through shared memory, so both sides are read and written along rows)
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ src, int rows, int cols, int lds,
                                 __nv_bfloat16* __restrict__ dst, int ldd) {
  __shared__ __nv_bfloat16 t[32][34];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[i][threadIdx.x] = src[(size_t)r * lds + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[(size_t)c * ldd + r] = t[threadIdx.x][i];
  }
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ pb, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pb[i] = __float2bfloat16(p[i]);
}

// top-2 of the first K logits per row (ties to the smaller index)
__global__ void k_top2(const float* __restrict__ logits, uint32_t rows, uint32_t K, uint32_t* __restrict__ out) {
  const uint32_t row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const uint32_t lane = threadIdx.x & 31;
  if (row >= rows) return;
  const float* z = logits + (size_t)row * kOut;
  float v1 = -FLT_MAX, v2 = -FLT_MAX;
  uint32_t i1 = 0xffffffffu, i2 = 0xffffffffu;
  for (uint32_t j = lane; j < K; j += 32) {
    const float x = z[j];
    if (x > v1) {
      v2 = v1;
      i2 = i1;
      v1 = x;
      i1 = j;
    } else if (x > v2) {
      v2 = x;
      i2 = j;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float a1 = __shfl_xor_sync(0xffffffffu, v1, o), a2 = __shfl_xor_sync(0xffffffffu, v2, o);
    const uint32_t j1 = __shfl_xor_sync(0xffffffffu, i1, o), j2 = __shfl_xor_sync(0xffffffffu, i2, o);
    // merge (v1,i1),(v2,i2) with (a1,j1),(a2,j2)
    float c[4] = {v1, v2, a1, a2};
    uint32_t ci[4] = {i1, i2, j1, j2};
    float b1 = -FLT_MAX, b2 = -FLT_MAX;
    uint32_t k1 = 0xffffffffu, k2 = 0xffffffffu;
    for (int q = 0; q < 4; ++q) {
      if (ci[q] == 0xffffffffu || ci[q] == k1) continue;
      if (c[q] > b1 || (c[q] == b1 && ci[q] < k1)) {
        b2 = b1;
        k2 = k1;
        b1 = c[q];
        k1 = ci[q];
      } else if (ci[q] != k2 && (c[q] > b2 || (c[q] == b2 && ci[q] < k2))) {
        b2 = c[q];
        k2 = ci[q];
      }
    }
    v1 = b1;
    v2 = b2;
    i1 = k1;
    i2 = k2;
  }
  if (lane == 0) {
    out[2 * row] = i1;
    out[2 * row + 1] = i2;
  }
}

// ------------------------------------------- fused inference on tcgen05 ----
//
// One CTA runs the whole network on chip for 256 rays, as two tiles of 128
// rows (A, B) that take turns on the tensor core: while the MMAs of one
// tile's stage run, the other tile's epilogue runs on the CUDA cores, and
// every weight chunk brought into shared memory serves both tiles.
//
// Warps 0-3 serve tile A and warps 4-7 tile B (thread = row = TMEM lane of
// the tile's accumulator); warp 8 (one lane) is the producer: it streams
// the weights with cp.async.bulk into two shared-memory buffers and issues
// every MMA (tcgen05, M = 128, fp32 accumulators in TMEM: tile A columns
// 0-255, tile B 256-511). Per tile the network is 21 stages: layer 1 in two
// K parts (K = 208: 192 Fourier features, two bias columns, zeros; the
// second part's operand columns are written once the first part's MMAs have
// read theirs, so a tile's operand rows fit in 36 KB), layers 2-4 (K = 144,
// N = 128) and 16 chunks of 256 logits (K = 144, N = 256). Stage j of a tile
// needs the tile's epilogue of stage j - 1 (its operand rows and its TMEM
// columns); handshakes are mbarriers: MMAs of a tile done (tcgen05.commit),
// epilogue of a tile done (128 arrivals), weights landed and weights
// consumed per buffer. Hidden epilogues: bf16, GELU, bf16 (as the
// layer-by-layer path rounds) back into the tile's operand rows; logit
// epilogues: a per-row running top-2. No activation or logit leaves the SM.
// Every wait is bounded; a CTA that times out raises the status word, lets
// its copies and MMAs drain, frees its TMEM and ends.
//
// The biases ride in the MMAs: every operand row carries two columns of
// ones (layer 1: columns 192, 193; layers 2-5: columns 128, 129 of a
// 16-column block after the 128 activations), and the packed weights carry
// each bias split into two bf16 parts (hi = bf16(b), lo = bf16(b - hi)) in
// those rows, so the fp32 accumulator holds W x + b to ~16 bits of b.
static const int kIn1 = 6 * kBands * 2 + 16;           // 208: K of layer 1
static const int kIn1a = 112;                           // layer 1's first K part (columns 0..111)
static const int kHidB = kHid + 16;                     // 144: K of layers 2..5
static const int kBiasIn = 2 * 6 * kBands;              // layer 1's bias columns: 192, 193
static const int kChunkN = 256;                         // logits per stage
static const int kChunks = kOut / kChunkN;              // 16
static const int kStages = 5 + kChunks;                 // 21
static const int kWeights = 4 + kChunks;                // 20 weight loads (W1 serves stages 0 and 1)
static const uint32_t kTileBytes = 128 * kHidB * 2;     // 36 KB: a tile's operand rows
static const uint32_t kWBytes = kChunkN * kHidB * 2;    // 72 KB: a logit chunk (the largest weight block)
static const uint32_t kFusedSmem = 2 * kTileBytes + 2 * kWBytes + 1024;
static const int kFusedThreads = 9 * 32;
static const int kLoadPieces = 8;  // bulk copies per weight block (every block's size is a multiple of 8 x 16 bytes)
static const long long kFusedWait = 500000000ll;  // ~0.25 s at 2 GHz per wait

// W (fp32 row-major [K][N]) and bias b -> the fused kernel's bf16 K-major
// operand [N][Kp] (canonical layout): rows k < kb are W's, row kb the bias's
// bf16 high part, row kb + 1 its low part, the rest zero; columns n >=
// n_valid get a -inf bias (no cluster there)
__global__ void k_pack_fused(const float* __restrict__ W, const float* __restrict__ b, int Kp, int kb, int N,
                             uint32_t n_valid, __nv_bfloat16* __restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)Kp * N) return;
  const int n = (int)(i / Kp), k = (int)(i % Kp);
  __nv_bfloat16 v = __float2bfloat16(0.f);
  if (k < kb) {
    v = __float2bfloat16(W[(size_t)k * N + n]);
  } else if (k == kb || k == kb + 1) {
    if ((uint32_t)n >= n_valid) {
      v = __float2bfloat16(k == kb ? -INFINITY : 0.f);
    } else {
      const __nv_bfloat16 hi = __float2bfloat16(b[n]);
      v = k == kb ? hi : __float2bfloat16(b[n] - __bfloat162float(hi));
    }
  }
  out[umma::tile_offset(n, k, Kp / 8) / 2] = v;
}

struct FusedArgs {
  const j3dg_ray* rays;
  uint32_t n;
  float cx, cy, cz, inv_s;
  const __nv_bfloat16* w[5];  // packed layers, biases included (k_pack_fused)
  uint32_t n_clusters;
  uint32_t hint_back;  // rays between a CTA's first ray and the ray whose result picks its first chunk
  uint32_t* top2;
  uint32_t* status;
};

__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// bf16, GELU (tanh form), bf16 of 64 accumulator columns (the accumulator
// holds W x + b; the layer-by-layer path rounds the pre-activation to bf16
// as well) into columns c0.. of this thread's operand row (K = 144)
__device__ __forceinline__ void hidden_cols(uint32_t taddr, uint8_t* X, int row, int c0) {
  const float k = 0.7978845608028654f;  // sqrt(2 / pi)
  float v[64];
  umma::ld64(taddr, v);
#pragma unroll
  for (int g = 0; g < 8; ++g) {
    uint32_t pk[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = g * 8 + 2 * q;
      const float z0 = __bfloat162float(__float2bfloat16(v[i]));
      const float z1 = __bfloat162float(__float2bfloat16(v[i + 1]));
      // the hardware tanh (relative error ~2^-11, below the bf16 rounding of the result)
      const float t0 = tanh_hw(z0 * fmaf(k * 0.044715f, z0 * z0, k)), t1 = tanh_hw(z1 * fmaf(k * 0.044715f, z1 * z1, k));
      const float h0 = 0.5f * z0, h1 = 0.5f * z1;
      pk[q] = bits2(__floats2bfloat162_rn(fmaf(h0, t0, h0), fmaf(h1, t1, h1)));
    }
    *reinterpret_cast<uint4*>(X + umma::tile_offset(row, c0 + g * 8, kHidB / 8)) =
        make_uint4(pk[0], pk[1], pk[2], pk[3]);
  }
}

// KS MMAs of one stage of one tile: D[tmem] (+)= A[128 x 16 KS] . B^T with
// A the tile's operand rows and B the weight rows (both canonical K-major
// layouts, kgA / kgB core matrices along K). Descriptors are built once; a
// K step advances both start addresses by 256 bytes (16 in the descriptors'
// address field).
template <int KS>
__device__ __forceinline__ void issue_mmas(uint32_t d_tmem, uint32_t xa, int kgA, uint32_t wb, int kgB, uint32_t idesc,
                                           bool acc) {
  const uint64_t da = umma::desc(xa, 128, (uint32_t)kgA * 128u), db = umma::desc(wb, 128, (uint32_t)kgB * 128u);
#pragma unroll
  for (int s = 0; s < KS; ++s)
    umma::mma_bf16(d_tmem, da + 16u * (uint32_t)s, db + 16u * (uint32_t)s, idesc, (s > 0 || acc) ? 1u : 0u);
}

// stage j of one tile: layer 1's two K parts, layers 2-4 (N = 128), logit chunks (N = 256)
__device__ __forceinline__ void issue_stage(int j, uint32_t d_tmem, uint32_t x0, uint32_t w0) {
  if (j == 0)
    issue_mmas<kIn1a / 16>(d_tmem, x0, kIn1a / 8, w0, kIn1 / 8, umma::idesc_bf16_f32(128, kHid), false);
  else if (j == 1)
    issue_mmas<(kIn1 - kIn1a) / 16>(d_tmem, x0, (kIn1 - kIn1a) / 8, w0 + (kIn1a / 16) * 256, kIn1 / 8,
                                    umma::idesc_bf16_f32(128, kHid), true);
  else if (j < 5)
    issue_mmas<kHidB / 16>(d_tmem, x0, kHidB / 8, w0, kHidB / 8, umma::idesc_bf16_f32(128, kHid), false);
  else
    issue_mmas<kHidB / 16>(d_tmem, x0, kHidB / 8, w0, kHidB / 8, umma::idesc_bf16_f32(128, kChunkN), false);
}

__global__ void __launch_bounds__(kFusedThreads, 1) k_learned_fused(const FusedArgs a) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t bar_md[2];  // a tile's stage MMAs done
  __shared__ __align__(8) uint64_t bar_cf[2];  // a tile's epilogue done (128 arrivals)
  __shared__ __align__(8) uint64_t bar_wl[2];  // weights landed in buffer
  __shared__ __align__(8) uint64_t bar_wf[2];  // MMAs reading buffer done
  __shared__ __align__(8) uint64_t bar_dr;     // all issued MMAs done (the error path's drain)
  __shared__ uint32_t taddr_s, cs_s, stop_s;
  uint8_t* base = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* wbuf = base + 2 * kTileBytes;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) stop_s = *reinterpret_cast<volatile uint32_t*>(a.status) & J3DG_DEV_VISIT_CAP;
  if (warp == 0) {
    umma::tmem_alloc(umma::smem_u32(&taddr_s), 512);
    umma::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      umma::mbar_init(umma::smem_u32(&bar_md[i]), 1);
      umma::mbar_init(umma::smem_u32(&bar_cf[i]), 128);
      umma::mbar_init(umma::smem_u32(&bar_wl[i]), 1);
      umma::mbar_init(umma::smem_u32(&bar_wf[i]), 1);
    }
    umma::mbar_init(umma::smem_u32(&bar_dr), 1);
    // The logit chunks are scanned starting from the chunk of the best
    // cluster of a ray one wave of CTAs earlier (hint_back rays back; most
    // likely written already, and a neighbour of these rays in the image),
    // so that most rows meet their best clusters first and skip the other
    // chunks' groups. Any value read here (even one still being written, or
    // a previous call's) only picks the order: the top-2 does not depend on
    // it.
    uint32_t hint = 0;
    if (blockIdx.x * 256u >= a.hint_back) hint = a.top2[2 * (size_t)(blockIdx.x * 256u - a.hint_back)];
    cs_s = hint < a.n_clusters ? hint / kChunkN : 0u;
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t taddr = taddr_s;
  const int cs = (int)cs_s;
  bool ok = stop_s == 0;  // a CTA that timed out raised the status word: the rest of the grid stops

  if (warp == 8) {
    // ------------------------------------------------------------ producer
    if (lane == 0 && ok) {
      // weight block w (W1, W2, W3, W4, then the logit chunks in scan order)
      // goes to buffer w % 2; stage j uses block j - 1 (stages 0, 1: W1)
      int loads = 0, landed = 0;  // weight blocks requested / landed
      bool any_mma = false;
      auto load = [&](int w) {
        const __nv_bfloat16* src;
        uint32_t bytes;
        if (w == 0) {
          src = a.w[0];
          bytes = 128 * kIn1 * 2;
        } else if (w < 4) {
          src = a.w[w];
          bytes = 128 * kHidB * 2;
        } else {
          src = a.w[4] + (size_t)((cs + w - 4) & (kChunks - 1)) * kChunkN * kHidB;
          bytes = kWBytes;
        }
        const uint32_t b = umma::smem_u32(&bar_wl[w & 1]), dst = umma::smem_u32(wbuf + (w & 1) * kWBytes);
        umma::mbar_arrive_expect_tx(b, bytes);
        // in kLoadPieces copies (each a multiple of 16 bytes): several bulk
        // copies in flight land a block sooner than one
        for (int q = 0; q < kLoadPieces; ++q)
          umma::bulk_copy(dst + q * (bytes / kLoadPieces), reinterpret_cast<const uint8_t*>(src) + q * (bytes / kLoadPieces),
                          bytes / kLoadPieces, b);
        loads = w + 1;
      };
      load(0);
      load(1);
      for (int j = 0; j < kStages && ok; ++j) {
        const int w = j < 2 ? 0 : j - 1, b = w & 1;
        if (j != 1) {
          ok = umma::mbar_wait_sleep(umma::smem_u32(&bar_wl[b]), (uint32_t)(w >> 1) & 1u, kFusedWait);
          if (ok) landed = w + 1;
        }
        // each tile's epilogue of stage j - 1 (epilogue count j: the first
        // feature part counts as epilogue 0)
        for (int t = 0; t < 2 && ok; ++t) {
          ok = umma::mbar_wait_sleep(umma::smem_u32(&bar_cf[t]), (uint32_t)j & 1u, kFusedWait);
          if (!ok) break;
          umma::fence_after_sync();
          issue_stage(j, taddr + (uint32_t)(t * 256), umma::smem_u32(base + t * kTileBytes),
                      umma::smem_u32(wbuf + b * kWBytes));
          umma::commit(umma::smem_u32(&bar_md[t]));
          any_mma = true;
          if (t == 0 && j >= 2 && w + 1 < kWeights) {
            // block w - 1's MMAs ran before these: its buffer takes block w + 1
            // now, while the tensor core works through this stage
            ok = umma::mbar_wait_sleep(umma::smem_u32(&bar_wf[(w - 1) & 1]), (uint32_t)((w - 1) >> 1) & 1u,
                                       kFusedWait);
            if (ok) load(w + 1);
          }
        }
        if (!ok) break;
        if (j == 0) continue;      // W1 serves stage 1 too
        umma::commit(umma::smem_u32(&bar_wf[b]));  // block w is consumed once these MMAs are done
      }
      if (!ok) {
        atomicOr(a.status, J3DG_DEV_VISIT_CAP);
        // drain: the copies requested and the MMAs issued end before the
        // CTA frees its TMEM and shared memory (bounded as well)
        // (at most one block per buffer is still in flight)
        for (int w = landed; w < loads; ++w)
          umma::mbar_wait_sleep(umma::smem_u32(&bar_wl[w & 1]), (uint32_t)(w >> 1) & 1u, kFusedWait);
        if (any_mma) {
          umma::commit(umma::smem_u32(&bar_dr));
          umma::mbar_wait_sleep(umma::smem_u32(&bar_dr), 0u, kFusedWait);
        }
      }
    }
  } else if (ok) {
    // ------------------------------------------------------------ consumers
    const int t = warp >> 2, row = (warp & 3) * 32 + lane;
    uint8_t* X = base + t * kTileBytes;
    const uint32_t r = blockIdx.x * 256u + (uint32_t)(t * 128 + row);
    const uint32_t tcol = taddr + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(t * 256);
    const uint32_t bar_m = umma::smem_u32(&bar_md[t]), bar_c = umma::smem_u32(&bar_cf[t]);
    float v1 = -FLT_MAX, v2 = -FLT_MAX;
    uint32_t i1 = 0xffffffffu, i2 = 0xffffffffu;
    // features of ray r (zeros past n; columns 192, 193 hold the ones of the
    // bias rows), in two K parts: coordinates 0-2 and the first half of
    // coordinate 3 (columns 0..111), then the rest (112..207)
    float in6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const bool live = r < a.n;
    if (live) ray_inputs(a.rays + r, a.cx, a.cy, a.cz, a.inv_s, in6);
    const uint4 zero4 = make_uint4(0u, 0u, 0u, 0u);
    {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        float sn[4], cn[4];
        base_octave(in6[i], sn, cn);
#pragma unroll
        for (int o = 0; o < (i < 3 ? 4 : 2); ++o) {
          *reinterpret_cast<uint4*>(X + umma::tile_offset(row, (i * 4 + o) * 8, kIn1a / 8)) =
              live ? octave_pairs(sn, cn) : zero4;
          next_octave(sn, cn);
        }
      }
    }
    uint4 fb[12];  // columns 112..207: coordinate 3's last two octaves, coordinates 4, 5, the ones, zeros
    {
      float sn[4], cn[4];
      base_octave(in6[3], sn, cn);
      next_octave(sn, cn);
      next_octave(sn, cn);
      fb[0] = octave_pairs(sn, cn);
      next_octave(sn, cn);
      fb[1] = octave_pairs(sn, cn);
#pragma unroll
      for (int i = 4; i < 6; ++i) {
        base_octave(in6[i], sn, cn);
#pragma unroll
        for (int o = 0; o < 4; ++o) {
          fb[2 + (i - 4) * 4 + o] = octave_pairs(sn, cn);
          if (o < 3) next_octave(sn, cn);
        }
      }
      if (!live)
        for (int g = 0; g < 10; ++g) fb[g] = zero4;
      fb[10] = make_uint4(bits2(__floats2bfloat162_rn(1.f, 1.f)), 0u, 0u, 0u);
      fb[11] = zero4;
    }
    umma::fence_async_smem();
    umma::mbar_arrive(bar_c);  // epilogue 0: the first feature part
#pragma unroll 1
    for (int j = 0; j < kStages; ++j) {
      ok = umma::mbar_wait_sleep(bar_m, (uint32_t)j & 1u, kFusedWait);
      if (!ok) break;
      umma::fence_after_sync();
      if (j == 0) {  // the first part's MMAs have read their columns: the second part
#pragma unroll
        for (int g = 0; g < 12; ++g)
          *reinterpret_cast<uint4*>(X + umma::tile_offset(row, g * 8, (kIn1 - kIn1a) / 8)) = fb[g];
        umma::fence_async_smem();
      } else if (j < 5) {
        hidden_cols(tcol, X, row, 0);
        hidden_cols(tcol + 64, X, row, 64);
        if (j == 1) {  // the bias block of layers 2..5: ones in columns 128, 129, zeros to 143
          *reinterpret_cast<uint4*>(X + umma::tile_offset(row, kHid, kHidB / 8)) = fb[10];
          *reinterpret_cast<uint4*>(X + umma::tile_offset(row, kHid + 8, kHidB / 8)) = zero4;
        }
        umma::fence_async_smem();
      } else {
        const int c = (cs + j - 5) & (kChunks - 1);
#pragma unroll 1
        for (int h = 0; h < kChunkN / 64; ++h) {
          float v[64];
          umma::ld64(tcol + (uint32_t)(h * 64), v);  // the logits, biases included
          float m = -FLT_MAX;
#pragma unroll
          for (int q = 0; q < 64; q += 2) m = max3f(m, v[q], v[q + 1]);
          if (m >= v2) {  // rare once the row's top-2 is established
#pragma unroll
            for (int q = 0; q < 64; ++q) {
              // chunks come in a rotated order, so ties are broken by the
              // index itself: (value desc, index asc)
              const float x = v[q];
              const uint32_t col = (uint32_t)(c * kChunkN + h * 64 + q);
              if (x > v2 || (x == v2 && col < i2)) {
                if (x > v1 || (x == v1 && col < i1)) {
                  v2 = v1;
                  i2 = i1;
                  v1 = x;
                  i1 = col;
                } else {
                  v2 = x;
                  i2 = col;
                }
              }
            }
          }
        }
      }
      umma::fence_before_sync();
      umma::mbar_arrive(bar_c);  // epilogue j + 1
    }
    if (!ok) {
      atomicOr(a.status, J3DG_DEV_VISIT_CAP);
    } else if (r < a.n) {
      a.top2[2 * (size_t)r] = i1;
      a.top2[2 * (size_t)r + 1] = i2;
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    umma::fence_after_sync();
    umma::tmem_dealloc(taddr, 512);
  }
}

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
__device__ __forceinline__ float u01(uint32_t seed, uint32_t i, uint32_t k) {
  return (float)(hash32(seed ^ hash32(i * 8u + k)) >> 8) * (1.f / 16777216.f);
}

// Training rays: a camera on a sphere of radius U(r0, r1) around the mesh
// centre looking at it, a uniform image point of a 60-degree (vertical),
// 16:9 frustum; rays are j3d primary rays (t_near = diagonal / 100).
__global__ void k_train_rays(uint32_t seed, uint32_t first, uint32_t n, float cx, float cy, float cz, float r0,
                             float r1, float t_near, j3dg_ray* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t id = first + i;
  const float z = 2.f * u01(seed, id, 0) - 1.f, ph = 6.2831853f * u01(seed, id, 1);
  const float sr = sqrtf(fmaxf(0.f, 1.f - z * z));
  const float bx = sr * cosf(ph), by = sr * sinf(ph), bz = z;  // back axis
  const float rad = r0 + (r1 - r0) * u01(seed, id, 2);
  const float ex = cx + rad * bx, ey = cy + rad * by, ez = cz + rad * bz;
  float ux = 0.f, uy = 1.f, uz = 0.f;
  if (fabsf(by) > 0.99f) {
    uy = 0.f;
    uz = 1.f;
  }
  float rx = uy * bz - uz * by, ry = uz * bx - ux * bz, rz = ux * by - uy * bx;
  const float rl = rsqrtf(rx * rx + ry * ry + rz * rz);
  rx *= rl;
  ry *= rl;
  rz *= rl;
  const float vx = by * rz - bz * ry, vy = bz * rx - bx * rz, vz = bx * ry - by * rx;
  const float th = 0.57735027f;  // tan 30 deg
  const float sx = (2.f * u01(seed, id, 3) - 1.f) * th * (16.f / 9.f), sy = (2.f * u01(seed, id, 4) - 1.f) * th;
  j3dg_ray r;
  r.orig[0] = ex;
  r.orig[1] = ey;
  r.orig[2] = ez;
  r.orig[3] = 1.f;
  r.dir[0] = sx * rx + sy * vx - bx;
  r.dir[1] = sx * ry + sy * vy - by;
  r.dir[2] = sx * rz + sy * vz - bz;
  r.dir[3] = 0.f;
  r.t_near = t_near;
  r.t_far = FLT_MAX;
  out[i] = r;
}

__global__ void k_labels(const j3dg_hit* __restrict__ hits, uint32_t n, uint32_t n_pad,
                         const uint16_t* __restrict__ cluster_of_tri, int32_t* __restrict__ labels) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  labels[i] = (i < n && hits[i].found) ? (int32_t)cluster_of_tri[hits[i].object_id] : -1;
}

// cluster_of_tri for every triangle under cluster root `roots[c]`
__global__ void k_cluster_map(const DevInst* __restrict__ inst, const uint32_t* __restrict__ roots, uint32_t n_roots,
                              uint16_t* __restrict__ cluster_of_tri, uint32_t* status) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_roots) return;
  const DevInst& I = inst[0];
  uint32_t stack[J3DG_STACK];
  int sp = 0;
  stack[sp++] = roots[c];
  uint32_t budget = I.n_nodes + 1;
  while (sp > 0) {
    const uint32_t ref = stack[--sp];
    if (ref == J3DG_EMPTY_REF) continue;
    if (ref & J3DG_LEAF_BIT) {
      const uint32_t first = (ref & 0x7fffffffu) >> 3, cnt = (ref & 7u) + 1u;
      if (first + cnt > I.nt) {
        atomicOr(status, J3DG_DEV_BAD_INDEX);
        return;
      }
      for (uint32_t k = 0; k < cnt; ++k) cluster_of_tri[__float_as_uint(I.tris[3 * (size_t)(first + k)].w)] = (uint16_t)c;
      continue;
    }
    if (budget-- == 0 || ref >= I.n_nodes || sp + 4 > J3DG_STACK) {
      atomicOr(status, J3DG_DEV_BAD_INDEX);
      return;
    }
    const float4 ch = I.nodes[8 * (size_t)ref + 6];
    stack[sp++] = __float_as_uint(ch.x);
    stack[sp++] = __float_as_uint(ch.y);
    stack[sp++] = __float_as_uint(ch.z);
    stack[sp++] = __float_as_uint(ch.w);
  }
}

// Learned closest hit: the two predicted clusters first, then the whole
// tree with their best hit as the starting best (exact).
__global__ void __launch_bounds__(128) k_rays_learned(const DevInst* __restrict__ inst, const j3dg_ray* __restrict__ rays,
                                                      uint32_t n, const uint32_t* __restrict__ top2,
                                                      const uint32_t* __restrict__ roots, uint32_t n_roots,
                                                      j3dg_hit* __restrict__ hits, uint32_t* status,
                                                      unsigned long long* counters,
                                                      unsigned long long* phase_counters) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t visits = 0, tests = 0, exact_visits = 0, exact_tests = 0;
  if (i < n) {
  const float* f = reinterpret_cast<const float*>(rays + i);
  TracerT<128> T;
  uint2 stack[J3DG_STACK];
  T.begin(inst, 1, f[0], f[1], f[2], f[4], f[5], f[6], f[8], f[9], false);
  const uint32_t c0 = top2[2 * i], c1 = top2[2 * i + 1];
  for (int phase = 0; phase < 3; ++phase) {
    uint32_t ref;
    if (phase < 2) {
      const uint32_t c = phase == 0 ? c0 : c1;
      if (c >= n_roots) continue;
      ref = roots[c];
    } else {
      ref = inst[0].root_ref;
    }
    T.cur = ref;
    T.sp = 0;
    T.inst = 0;
    T.budget = T.n_nodes + 1;
    uint32_t& pv = phase < 2 ? visits : exact_visits;
    uint32_t& pt = phase < 2 ? tests : exact_tests;
    while (!T.step(inst, 1, status, pv, pt, stack)) {
    }
  }
  j3dg_hit h;
  h.found = T.b.found ? 1u : 0u;
  h.distance = T.b.found ? T.b.t : f[9];
  h.u = T.b.u();
  h.v = T.b.v();
  h.object_id = T.b.found ? T.b.tri() : 0xffffffffu;
  h.two_level_index = T.b.found ? 0u : 0xffffffffu;
  hits[i] = h;
  }
  if (counters && i < n) {
    atomicAdd(counters + 0, (unsigned long long)(visits + exact_visits));
    atomicAdd(counters + 1, (unsigned long long)(tests + exact_tests));
  }
  if (phase_counters) {  // [cluster visits, cluster tests, exact visits, exact tests]
    const uint32_t v[4] = {__reduce_add_sync(0xffffffffu, visits), __reduce_add_sync(0xffffffffu, tests),
                           __reduce_add_sync(0xffffffffu, exact_visits), __reduce_add_sync(0xffffffffu, exact_tests)};
    if ((threadIdx.x & 31u) == 0)
      for (int k = 0; k < 4; ++k) atomicAdd(phase_counters + k, (unsigned long long)v[k]);
  }
}

}  // namespace j3dg

// ------------------------------------------------------------------ host

using j3dg::DevInst;

struct j3dg_learned {
  j3dg_ctx* ctx = nullptr;
  CtxHold hold;
  const j3dg_mesh* mesh = nullptr;
  j3dg_learned_opts opts;
  j3dg::Layout L;
  uint32_t n_clusters = 0;
  std::vector<uint32_t> h_roots;
  uint32_t* d_roots = nullptr;
  uint16_t* d_cluster_of_tri = nullptr;
  float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
  __nv_bfloat16* d_pb = nullptr;
  uint32_t adam_t = 0;
  // per-batch workspace (batch rows)
  uint32_t B = 0;
  __nv_bfloat16 *X = nullptr, *H[4] = {nullptr, nullptr, nullptr, nullptr}, *Z[4] = {nullptr, nullptr, nullptr, nullptr};
  __nv_bfloat16 *dZ5 = nullptr, *dA = nullptr, *dB = nullptr;
  // transposed copies the tcgen05 GEMMs read K-major: of the features, the
  // hidden activations and the gradients (weight gradients reduce over the
  // batch), and of the bf16 weights (the forward pass)
  __nv_bfloat16 *Xt = nullptr, *Ht[4] = {nullptr, nullptr, nullptr, nullptr};
  __nv_bfloat16 *dZ5t = nullptr, *dAt = nullptr, *dBt = nullptr;
  __nv_bfloat16* d_pbt = nullptr;
  float* logits = nullptr;
  int32_t* labels = nullptr;
  float* d_loss = nullptr;
  uint32_t* d_correct = nullptr;
  j3dg_ray* rays = nullptr;
  j3dg_hit* hits = nullptr;
  uint32_t* top2 = nullptr;
  __nv_bfloat16* d_wpack = nullptr;  // weights in the tcgen05 operand layout (fused inference)
  float center[3] = {0, 0, 0}, inv_scale = 1.f, t_near = 0.f;
};

namespace {

cudaStream_t LS(j3dg_learned* l) {
  ++l->ctx->stream_ops;
  return (cudaStream_t)l->ctx->stream;
}

#define LCK(x, where)                                                                              \
  do {                                                                                             \
    cudaError_t e_ = (x);                                                                          \
    if (e_ != cudaSuccess) return j3dg::ctx_fail(l->ctx, J3DG_ERR_CUDA, std::string(where) + ": " + \
                                                     cudaGetErrorString(e_));                      \
  } while (0)

int alloc_workspace(j3dg_learned* l, uint32_t B) {
  if (l->B >= B) return J3DG_OK;
  cudaFree(l->X);
  for (int k = 0; k < 4; ++k) {
    cudaFree(l->H[k]);
    cudaFree(l->Z[k]);
  }
  cudaFree(l->dZ5);
  cudaFree(l->dA);
  cudaFree(l->dB);
  cudaFree(l->Xt);
  for (int k = 0; k < 4; ++k) cudaFree(l->Ht[k]);
  cudaFree(l->dZ5t);
  cudaFree(l->dAt);
  cudaFree(l->dBt);
  cudaFree(l->logits);
  cudaFree(l->labels);
  cudaFree(l->rays);
  cudaFree(l->hits);
  cudaFree(l->top2);
  l->B = B;
  LCK(cudaMalloc(&l->X, sizeof(__nv_bfloat16) * B * j3dg::kIn), "learned workspace");
  for (int k = 0; k < 4; ++k) {
    LCK(cudaMalloc(&l->H[k], sizeof(__nv_bfloat16) * B * j3dg::kHid), "learned workspace");
    LCK(cudaMalloc(&l->Z[k], sizeof(__nv_bfloat16) * B * j3dg::kHid), "learned workspace");
  }
  LCK(cudaMalloc(&l->dZ5, sizeof(__nv_bfloat16) * B * j3dg::kOut), "learned workspace");
  LCK(cudaMalloc(&l->dA, sizeof(__nv_bfloat16) * B * j3dg::kHid), "learned workspace");
  LCK(cudaMalloc(&l->dB, sizeof(__nv_bfloat16) * B * j3dg::kHid), "learned workspace");
  LCK(cudaMalloc(&l->Xt, sizeof(__nv_bfloat16) * B * j3dg::kIn), "learned workspace");
  for (int k = 0; k < 4; ++k) LCK(cudaMalloc(&l->Ht[k], sizeof(__nv_bfloat16) * B * j3dg::kHid), "learned workspace");
  LCK(cudaMalloc(&l->dZ5t, sizeof(__nv_bfloat16) * B * j3dg::kOut), "learned workspace");
  LCK(cudaMalloc(&l->dAt, sizeof(__nv_bfloat16) * B * j3dg::kHid), "learned workspace");
  LCK(cudaMalloc(&l->dBt, sizeof(__nv_bfloat16) * B * j3dg::kHid), "learned workspace");
  LCK(cudaMalloc(&l->logits, sizeof(float) * B * j3dg::kOut), "learned workspace");
  LCK(cudaMalloc(&l->labels, sizeof(int32_t) * B), "learned workspace");
  LCK(cudaMalloc(&l->rays, sizeof(j3dg_ray) * B), "learned workspace");
  LCK(cudaMalloc(&l->hits, sizeof(j3dg_hit) * B), "learned workspace");
  LCK(cudaMalloc(&l->top2, sizeof(uint32_t) * 2 * B), "learned workspace");
  return J3DG_OK;
}

__nv_bfloat16* W(j3dg_learned* l, int k) { return l->d_pb + l->L.w[k]; }
__nv_bfloat16* Wt(j3dg_learned* l, int k) { return l->d_pbt + l->L.w[k]; }
const float* Bias(j3dg_learned* l, int k) { return l->d_p + l->L.b[k]; }

int transpose(j3dg_learned* l, const __nv_bfloat16* src, int rows, int cols, __nv_bfloat16* dst, const char* where) {
  j3dg::k_transpose_bf16<<<dim3((cols + 31) / 32, (rows + 31) / 32), dim3(32, 8), 0, LS(l)>>>(src, rows, cols, cols,
                                                                                             dst, rows);
  LCK(cudaGetLastError(), where);
  return J3DG_OK;
}

// the transposed bf16 weights Wt_k [out][in] the forward GEMMs read (after
// every change of d_pb)
int refresh_wt(j3dg_learned* l) {
  for (int k = 0; k < 5; ++k)
    if (int rc = transpose(l, W(l, k), l->L.in[k], l->L.out[k], Wt(l, k), "learned weights")) return rc;
  return J3DG_OK;
}

int gemm(j3dg_learned* l, const j3dg::UmmaArgs& g, const char* where) {
  cudaError_t e = j3dg::umma_gemm_bf16(g, l->ctx->d_status, LS(l));
  if (e == cudaErrorInvalidValue) return j3dg::ctx_fail(l->ctx, J3DG_ERR_INVALID_ARGUMENT, std::string(where) + ": bad GEMM shape");
  LCK(e, where);
  return J3DG_OK;
}

j3dg::UmmaArgs umma(const __nv_bfloat16* A, const __nv_bfloat16* Bt, void* C, int M, int N, int K, int epi) {
  j3dg::UmmaArgs g{};
  g.A = A;
  g.Bt = Bt;
  g.C = C;
  g.M = M;
  g.N = N;
  g.K = K;
  g.lda = K;
  g.ldb = K;
  g.ldc = N;
  g.epi = epi;
  g.splits = 1;
  return g;
}

// forward over X (B rows) on the tcgen05 GEMMs: H1..H4 (and with train,
// their transposes for the weight gradients), logits
int forward(j3dg_learned* l, uint32_t B, bool train = false) {
  const __nv_bfloat16* in = l->X;
  int in_dim = j3dg::kIn;
  for (int k = 0; k < 4; ++k) {
    j3dg::UmmaArgs g = umma(in, Wt(l, k), l->H[k], (int)B, j3dg::kHid, in_dim, j3dg::EPI_BIAS_GELU);
    g.bias = Bias(l, k);
    g.Z = l->Z[k];
    if (train) {
      g.Ct = l->Ht[k];
      g.ldct = (int)B;
    }
    if (int rc = gemm(l, g, "learned forward")) return rc;
    in = l->H[k];
    in_dim = j3dg::kHid;
  }
  j3dg::UmmaArgs g = umma(l->H[3], Wt(l, 4), l->logits, (int)B, j3dg::kOut, j3dg::kHid, j3dg::EPI_BIAS_F32);
  g.bias = Bias(l, 4);
  return gemm(l, g, "learned forward");
}

// split-K of a weight gradient over the batch: about one CTA per SM
int splits_for(j3dg_learned* l, int M, int N, uint32_t B) {
  const int tiles = (M / 128) * (N % 256 == 0 ? N / 256 : N / 128);
  const int want = std::max(1, l->ctx->sm_count / std::max(1, tiles));
  return std::max(1, std::min(want, (int)(B / 256)));
}

// softmax CE + backward into l->d_g (all gradients overwritten), on the
// tcgen05 GEMMs; forward(l, B, true) ran before
int backward(j3dg_learned* l, uint32_t B, float inv_valid) {
  j3dg::k_softmax_ce<<<(B + 7) / 8, 256, 0, LS(l)>>>(l->logits, l->labels, B, l->n_clusters, inv_valid, l->dZ5,
                                                       l->d_loss, l->d_correct);
  LCK(cudaGetLastError(), "learned softmax");
  if (int rc = transpose(l, l->dZ5, (int)B, j3dg::kOut, l->dZ5t, "learned backward")) return rc;
  float* g = l->d_g;
  // layer 5: dW5 = H4^T dZ5, db5 = colsum(dZ5), dZ4 = (dZ5 W5^T) * gelu'(Z4)
  {
    j3dg::UmmaArgs a = umma(l->Ht[3], l->dZ5t, g + l->L.w[4], j3dg::kHid, j3dg::kOut, (int)B, j3dg::EPI_F32_ACCUM);
    a.splits = splits_for(l, j3dg::kHid, j3dg::kOut, B);
    LCK(cudaMemsetAsync(g + l->L.w[4], 0, sizeof(float) * j3dg::kHid * j3dg::kOut, LS(l)), "learned backward");
    if (int rc = gemm(l, a, "learned backward")) return rc;
    LCK(cudaMemsetAsync(g + l->L.b[4], 0, sizeof(float) * j3dg::kOut, LS(l)), "learned backward");
    j3dg::k_colsum<<<dim3((j3dg::kOut + 255) / 256, (B + 127) / 128), 256, 0, LS(l)>>>(l->dZ5, B, j3dg::kOut,
                                                                                        g + l->L.b[4]);
    j3dg::UmmaArgs d = umma(l->dZ5, W(l, 4), l->dA, (int)B, j3dg::kHid, j3dg::kOut, j3dg::EPI_GELU_BWD);
    d.Z = l->Z[3];
    d.Ct = l->dAt;
    d.ldct = (int)B;
    if (int rc = gemm(l, d, "learned backward")) return rc;
  }
  __nv_bfloat16 *dcur = l->dA, *dcur_t = l->dAt, *dnext = l->dB, *dnext_t = l->dBt;
  for (int k = 3; k >= 0; --k) {
    const __nv_bfloat16* in_t = k ? l->Ht[k - 1] : l->Xt;
    const int in_dim = k ? j3dg::kHid : j3dg::kIn;
    j3dg::UmmaArgs a = umma(in_t, dcur_t, g + l->L.w[k], in_dim, j3dg::kHid, (int)B, j3dg::EPI_F32_ACCUM);
    a.splits = splits_for(l, in_dim, j3dg::kHid, B);
    LCK(cudaMemsetAsync(g + l->L.w[k], 0, sizeof(float) * in_dim * j3dg::kHid, LS(l)), "learned backward");
    if (int rc = gemm(l, a, "learned backward")) return rc;
    LCK(cudaMemsetAsync(g + l->L.b[k], 0, sizeof(float) * j3dg::kHid, LS(l)), "learned backward");
    j3dg::k_colsum<<<dim3(1, (B + 127) / 128), 128, 0, LS(l)>>>(dcur, B, j3dg::kHid, g + l->L.b[k]);
    if (k > 0) {
      j3dg::UmmaArgs d = umma(dcur, W(l, k), dnext, (int)B, j3dg::kHid, j3dg::kHid, j3dg::EPI_GELU_BWD);
      d.Z = l->Z[k - 1];
      d.Ct = dnext_t;
      d.ldct = (int)B;
      if (int rc = gemm(l, d, "learned backward")) return rc;
      std::swap(dcur, dnext);
      std::swap(dcur_t, dnext_t);
    }
  }
  LCK(cudaGetLastError(), "learned backward");
  return J3DG_OK;
}

int features(j3dg_learned* l, const j3dg_ray* d_rays, uint32_t n, uint32_t n_pad) {
  j3dg::k_features<<<(n_pad + 127) / 128, 128, 0, LS(l)>>>(d_rays, n, n_pad, l->center[0], l->center[1], l->center[2],
                                                            l->inv_scale, l->X);
  LCK(cudaGetLastError(), "learned features");
  return J3DG_OK;
}

uint32_t pad128(uint32_t n) { return (n + 127u) & ~127u; }

}  // namespace

extern "C" {

int j3dg_learned_create(j3dg_ctx* c, const j3dg_mesh* mesh, const j3dg_learned_opts* opts, j3dg_learned** out) {
  if (!c || !mesh || !out) return J3DG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (mesh->width != 4) return j3dg::ctx_fail(c, J3DG_ERR_UNSUPPORTED, "learned: needs a 4-wide BVH");
  cudaSetDevice(c->device);
  j3dg_learned* l = new (std::nothrow) j3dg_learned();
  if (!l) return J3DG_ERR_OUT_OF_MEMORY;
  l->ctx = c;
  l->hold.attach(c);
  l->mesh = mesh;
  l->opts.cluster_depth = 6;
  l->opts.batch = 16384;
  l->opts.lr = 2e-3f;
  l->opts.seed = 0x6A3D0003ull;
  if (opts) {
    if (opts->cluster_depth) l->opts.cluster_depth = opts->cluster_depth;
    if (opts->batch) l->opts.batch = opts->batch;
    if (opts->lr > 0.f) l->opts.lr = opts->lr;
    l->opts.seed = opts->seed;
  }
  if (l->opts.cluster_depth > 6 || l->opts.batch % 128) {
    delete l;
    return j3dg::ctx_fail(c, J3DG_ERR_INVALID_ARGUMENT, "learned: cluster_depth <= 6, batch a multiple of 128");
  }
  // clusters: the refs at cluster_depth below the root (and shallower
  // leaves), found by walking the tree from the root (node numbering is free)
  std::vector<uint32_t> level{mesh->root_ref};
  cudaError_t e = cudaSuccess;
  for (uint32_t d = 0; d < l->opts.cluster_depth && e == cudaSuccess; ++d) {
    std::vector<uint32_t> inner;
    for (uint32_t ref : level)
      if (!(ref & J3DG_LEAF_BIT)) inner.push_back(ref);
    std::vector<uint32_t> refs(4 * inner.size());
    for (size_t i = 0; i < inner.size() && e == cudaSuccess; ++i) {
      if (inner[i] >= mesh->n_nodes) {
        delete l;
        return j3dg::ctx_fail(c, J3DG_ERR_INVALID_ARGUMENT, "learned: corrupt node reference");
      }
      // the child references: float4 6 of the node
      e = cudaMemcpyAsync(&refs[4 * i], (const float4*)mesh->d_nodes + 8 * (size_t)inner[i] + 6, 16,
                          cudaMemcpyDeviceToHost, LS(l));
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(LS(l));
    // children in the order of their parents and slots, leaves kept in place
    size_t li = 0;
    std::vector<uint32_t> ordered;
    for (uint32_t ref : level) {
      if (ref & J3DG_LEAF_BIT) {
        ordered.push_back(ref);
        continue;
      }
      for (int k = 0; k < 4; ++k)
        if (refs[4 * li + k] != J3DG_EMPTY_REF) ordered.push_back(refs[4 * li + k]);
      ++li;
    }
    level.swap(ordered);
  }
  if (e != cudaSuccess) {
    delete l;
    return j3dg::ctx_fail(c, J3DG_ERR_CUDA, "learned: reading nodes failed");
  }
  if (level.size() > (size_t)j3dg::kOut) {
    delete l;
    return j3dg::ctx_fail(c, J3DG_ERR_UNSUPPORTED, "learned: more than 4096 clusters");
  }
  l->h_roots = level;
  l->n_clusters = (uint32_t)level.size();
  const DevInst* dinst = nullptr;
  int rc = j3dg::mesh_devinst(c, mesh, &dinst);
  if (rc) {
    delete l;
    return rc;
  }
  e = cudaMalloc(&l->d_roots, sizeof(uint32_t) * l->n_clusters);
  if (e == cudaSuccess) e = cudaMalloc(&l->d_cluster_of_tri, sizeof(uint16_t) * mesh->nt);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(l->d_roots, l->h_roots.data(), sizeof(uint32_t) * l->n_clusters, cudaMemcpyHostToDevice,
                        LS(l));
  if (e == cudaSuccess) {
    j3dg::k_cluster_map<<<(l->n_clusters + 63) / 64, 64, 0, LS(l)>>>(dinst, l->d_roots, l->n_clusters,
                                                                    l->d_cluster_of_tri, c->d_status);
    e = cudaGetLastError();
  }
  // parameters: N(0, sqrt(2 / fan_in)) weights (seeded, host), zero biases
  const size_t P = l->L.total;
  std::vector<float> hp(P, 0.f);
  uint64_t s = l->opts.seed * 0x9E3779B97F4A7C15ull + 1;
  auto next = [&]() {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int k = 0; k < 5; ++k) {
    const double sd = std::sqrt(2.0 / (k == 0 ? 192.0 : 128.0));
    for (size_t i = 0; i < (size_t)l->L.in[k] * l->L.out[k]; ++i) {
      const double u1 = std::max(next(), 1e-12), u2 = next();
      hp[l->L.w[k] + i] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
    }
    if (k == 0)  // rows of the zero padding features stay zero
      for (int r = 192; r < j3dg::kIn; ++r)
        for (int o = 0; o < j3dg::kHid; ++o) hp[l->L.w[0] + (size_t)r * j3dg::kHid + o] = 0.f;
  }
  if (e == cudaSuccess) e = cudaMalloc(&l->d_p, sizeof(float) * P);
  if (e == cudaSuccess) e = cudaMalloc(&l->d_g, sizeof(float) * P);
  if (e == cudaSuccess) e = cudaMalloc(&l->d_m, sizeof(float) * P);
  if (e == cudaSuccess) e = cudaMalloc(&l->d_v, sizeof(float) * P);
  if (e == cudaSuccess) e = cudaMalloc(&l->d_pb, sizeof(__nv_bfloat16) * P);
  if (e == cudaSuccess) e = cudaMalloc(&l->d_pbt, sizeof(__nv_bfloat16) * P);
  if (e == cudaSuccess) e = cudaMalloc(&l->d_loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&l->d_correct, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemcpyAsync(l->d_p, hp.data(), sizeof(float) * P, cudaMemcpyHostToDevice, LS(l));
  if (e == cudaSuccess) e = cudaMemsetAsync(l->d_m, 0, sizeof(float) * P, LS(l));
  if (e == cudaSuccess) e = cudaMemsetAsync(l->d_v, 0, sizeof(float) * P, LS(l));
  if (e == cudaSuccess) {
    j3dg::k_to_bf16<<<(unsigned)((P + 255) / 256), 256, 0, LS(l)>>>(l->d_p, l->d_pb, P);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && refresh_wt(l) != J3DG_OK) e = cudaErrorUnknown;
  if (e == cudaSuccess) e = cudaStreamSynchronize(LS(l));
  if (e != cudaSuccess) {
    j3dg_learned_destroy(l);
    return j3dg::ctx_fail(c, J3DG_ERR_CUDA, std::string("learned_create: ") + cudaGetErrorString(e));
  }
  // normalisation of ray origins: mesh bbox centre and half of its largest extent
  float ext = 0.f;
  for (int k = 0; k < 3; ++k) {
    l->center[k] = 0.5f * (mesh->min_bb[k] + mesh->max_bb[k]);
    ext = std::max(ext, mesh->max_bb[k] - mesh->min_bb[k]);
  }
  l->inv_scale = ext > 0.f ? 2.f / ext : 1.f;
  l->t_near = ext / 100.f;
  *out = l;
  return J3DG_OK;
}

int j3dg_learned_destroy(j3dg_learned* l) {
  if (!l) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(l->ctx->device);
  cudaStreamSynchronize(LS(l));
  void* ptrs[] = {l->d_roots, l->d_cluster_of_tri, l->d_p, l->d_g, l->d_m, l->d_v, l->d_pb, l->d_pbt, l->X, l->dZ5,
                  l->dA, l->dB, l->Xt, l->dZ5t, l->dAt, l->dBt, l->logits, l->labels, l->d_loss, l->d_correct,
                  l->rays, l->hits, l->top2, l->d_wpack};
  for (void* p : ptrs) cudaFree(p);
  for (int k = 0; k < 4; ++k) {
    cudaFree(l->H[k]);
    cudaFree(l->Z[k]);
    cudaFree(l->Ht[k]);
  }
  delete l;
  return J3DG_OK;
}

int j3dg_learned_info(const j3dg_learned* l, uint32_t* n_clusters, uint64_t* n_params) {
  if (!l) return J3DG_ERR_INVALID_ARGUMENT;
  if (n_clusters) *n_clusters = l->n_clusters;
  if (n_params) *n_params = l->L.total;
  return J3DG_OK;
}

int j3dg_learned_get_params(j3dg_learned* l, float* out) {
  if (!l || !out) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(l->ctx->device);
  LCK(cudaMemcpyAsync(out, l->d_p, sizeof(float) * l->L.total, cudaMemcpyDeviceToHost, LS(l)), "get_params");
  LCK(cudaStreamSynchronize(LS(l)), "get_params");
  return J3DG_OK;
}

int j3dg_learned_set_params(j3dg_learned* l, const float* in) {
  if (!l || !in) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(l->ctx->device);
  const size_t P = l->L.total;
  LCK(cudaMemcpyAsync(l->d_p, in, sizeof(float) * P, cudaMemcpyHostToDevice, LS(l)), "set_params");
  j3dg::k_to_bf16<<<(unsigned)((P + 255) / 256), 256, 0, LS(l)>>>(l->d_p, l->d_pb, P);
  if (int rc = refresh_wt(l)) return rc;
  LCK(cudaStreamSynchronize(LS(l)), "set_params");
  return J3DG_OK;
}

// Loss and gradients for a batch of given features (B x 256, fp32; rounded
// to bf16 as the network reads them) and labels; for gradient checks.
int j3dg_learned_loss_grad(j3dg_learned* l, const float* feats, const int32_t* labels, uint32_t B, float* loss,
                           float* grads) {
  if (!l || !feats || !labels || B == 0 || B % 128) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(l->ctx->device);
  if (int rc = alloc_workspace(l, std::max(B, l->opts.batch))) return rc;
  std::vector<__nv_bfloat16> xb((size_t)B * j3dg::kIn);
  for (size_t i = 0; i < xb.size(); ++i) xb[i] = __float2bfloat16(feats[i]);
  uint32_t valid = 0;
  for (uint32_t i = 0; i < B; ++i) valid += labels[i] >= 0;
  LCK(cudaMemcpyAsync(l->X, xb.data(), sizeof(__nv_bfloat16) * xb.size(), cudaMemcpyHostToDevice, LS(l)), "loss_grad");
  LCK(cudaMemcpyAsync(l->labels, labels, sizeof(int32_t) * B, cudaMemcpyHostToDevice, LS(l)), "loss_grad");
  LCK(cudaMemsetAsync(l->d_loss, 0, sizeof(float), LS(l)), "loss_grad");
  LCK(cudaMemsetAsync(l->d_correct, 0, sizeof(uint32_t), LS(l)), "loss_grad");
  if (int rc = transpose(l, l->X, (int)B, j3dg::kIn, l->Xt, "loss_grad")) return rc;
  if (int rc = forward(l, B, true)) return rc;
  if (int rc = backward(l, B, valid ? 1.f / (float)valid : 0.f)) return rc;
  float ls = 0.f;
  LCK(cudaMemcpyAsync(&ls, l->d_loss, sizeof(float), cudaMemcpyDeviceToHost, LS(l)), "loss_grad");
  if (grads) LCK(cudaMemcpyAsync(grads, l->d_g, sizeof(float) * l->L.total, cudaMemcpyDeviceToHost, LS(l)), "loss_grad");
  LCK(cudaStreamSynchronize(LS(l)), "loss_grad");
  if (loss) *loss = valid ? ls / (float)valid : 0.f;
  return J3DG_OK;
}

int j3dg_learned_train(j3dg_learned* l, uint64_t n_rays, float r0, float r1, float* final_loss, float* accuracy,
                       float* seconds) {
  if (!l || n_rays == 0 || !(r1 >= r0) || r0 <= 0.f) return J3DG_ERR_INVALID_ARGUMENT;
  j3dg_ctx* c = l->ctx;
  cudaSetDevice(c->device);
  const uint32_t B = l->opts.batch;
  if (int rc = alloc_workspace(l, B)) return rc;
  const auto t0 = std::chrono::steady_clock::now();
  const uint64_t steps = (n_rays + B - 1) / B;
  const float b1 = 0.9f, b2 = 0.999f;
  float last_loss = 0.f, last_acc = 0.f;
  std::vector<int32_t> lab(B);
  for (uint64_t s = 0; s < steps; ++s) {
    j3dg::k_train_rays<<<(B + 127) / 128, 128, 0, LS(l)>>>((uint32_t)l->opts.seed, (uint32_t)(s * B), B, l->center[0],
                                                           l->center[1], l->center[2], r0, r1, l->t_near, l->rays);
    LCK(cudaGetLastError(), "train rays");
    if (int rc = j3dg::ray_query_device(c, l->mesh, l->rays, B, l->hits)) return rc;
    j3dg::k_labels<<<(B + 127) / 128, 128, 0, LS(l)>>>(l->hits, B, B, l->d_cluster_of_tri, l->labels);
    if (int rc = features(l, l->rays, B, B)) return rc;
    LCK(cudaMemsetAsync(l->d_loss, 0, sizeof(float), LS(l)), "train");
    LCK(cudaMemsetAsync(l->d_correct, 0, sizeof(uint32_t), LS(l)), "train");
    if (int rc = transpose(l, l->X, (int)B, j3dg::kIn, l->Xt, "train")) return rc;
    if (int rc = forward(l, B, true)) return rc;
    // hit fraction of the training rays is ~ constant; scale by the batch
    if (int rc = backward(l, B, 1.f / (float)B)) return rc;
    ++l->adam_t;
    const float c1 = 1.f / (1.f - std::pow(b1, (float)l->adam_t)), c2 = 1.f / (1.f - std::pow(b2, (float)l->adam_t));
    j3dg::k_adam<<<(unsigned)((l->L.total + 255) / 256), 256, 0, LS(l)>>>(l->d_p, l->d_g, l->d_m, l->d_v, l->d_pb,
                                                                         l->L.total, l->opts.lr, b1, b2, 1e-8f, c1, c2);
    LCK(cudaGetLastError(), "adam");
    if (int rc = refresh_wt(l)) return rc;
    if (s + 1 == steps || (s % 64) == 63) {
      float ls = 0.f;
      uint32_t corr = 0;
      LCK(cudaMemcpyAsync(&ls, l->d_loss, sizeof(float), cudaMemcpyDeviceToHost, LS(l)), "train");
      LCK(cudaMemcpyAsync(&corr, l->d_correct, sizeof(uint32_t), cudaMemcpyDeviceToHost, LS(l)), "train");
      LCK(cudaMemcpyAsync(lab.data(), l->labels, sizeof(int32_t) * B, cudaMemcpyDeviceToHost, LS(l)), "train");
      LCK(cudaStreamSynchronize(LS(l)), "train");
      uint32_t valid = 0;
      for (int32_t x : lab) valid += x >= 0;
      last_loss = valid ? ls / (float)valid : 0.f;
      last_acc = valid ? (float)corr / (float)valid : 0.f;
    }
  }
  LCK(cudaStreamSynchronize(LS(l)), "train");
  if (final_loss) *final_loss = last_loss;
  if (accuracy) *accuracy = last_acc;
  if (seconds) *seconds = std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
  return J3DG_OK;
}

// top-2 clusters per ray on device arrays: the fused tcgen05 kernel
static int predict_fused(j3dg_learned* l, const j3dg_ray* d_rays, uint32_t n, uint32_t* d_top2) {
  const j3dg::Layout& L = l->L;
  // packed operands with the bias rows: K = 208 for layer 1, 144 for layers 2..5
  const int Kp[5] = {j3dg::kIn1, j3dg::kHidB, j3dg::kHidB, j3dg::kHidB, j3dg::kHidB};
  const int kb[5] = {j3dg::kBiasIn, j3dg::kHid, j3dg::kHid, j3dg::kHid, j3dg::kHid};
  size_t total = 0;
  for (int k = 0; k < 5; ++k) total += (size_t)Kp[k] * L.out[k];
  if (!l->d_wpack) LCK(cudaMalloc(&l->d_wpack, sizeof(__nv_bfloat16) * total), "learned pack");
  j3dg::FusedArgs a;
  size_t off = 0;
  for (int k = 0; k < 5; ++k) {
    const size_t cnt = (size_t)Kp[k] * L.out[k];
    j3dg::k_pack_fused<<<(unsigned)((cnt + 255) / 256), 256, 0, LS(l)>>>(
        l->d_p + L.w[k], l->d_p + L.b[k], Kp[k], kb[k], L.out[k], k == 4 ? l->n_clusters : (uint32_t)L.out[k],
        l->d_wpack + off);
    LCK(cudaGetLastError(), "learned pack");
    a.w[k] = l->d_wpack + off;
    off += cnt;
  }
  a.rays = d_rays;
  a.n = n;
  a.cx = l->center[0];
  a.cy = l->center[1];
  a.cz = l->center[2];
  a.inv_s = l->inv_scale;
  a.n_clusters = l->n_clusters;
  a.hint_back = 256u * (uint32_t)std::max(1, l->ctx->sm_count);  // one CTA per SM: one wave back
  a.top2 = d_top2;
  a.status = l->ctx->d_status;
  LCK(cudaFuncSetAttribute(j3dg::k_learned_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)j3dg::kFusedSmem),
      "learned fused");
  j3dg::k_learned_fused<<<(n + 255) / 256, j3dg::kFusedThreads, j3dg::kFusedSmem, LS(l)>>>(a);
  LCK(cudaGetLastError(), "learned fused");
  return J3DG_OK;
}

// top-2 clusters per ray on device arrays: impl 1 fused tcgen05 kernel,
// impl 0 the layer-by-layer tcgen05 GEMMs + a top-2 pass over the logits
static int predict_device(j3dg_learned* l, const j3dg_ray* d_rays, uint32_t n, uint32_t* d_top2, int impl = 1) {
  if (impl == 1) return predict_fused(l, d_rays, n, d_top2);
  const uint32_t B = l->opts.batch;
  if (int rc = alloc_workspace(l, B)) return rc;
  for (uint32_t off = 0; off < n; off += B) {
    const uint32_t m = std::min(B, n - off);
    const uint32_t mp = pad128(m);
    if (int rc = features(l, d_rays + off, m, mp)) return rc;
    if (int rc = forward(l, mp)) return rc;
    j3dg::k_top2<<<(m + 7) / 8, 256, 0, LS(l)>>>(l->logits, m, l->n_clusters, d_top2 + 2 * (size_t)off);
    LCK(cudaGetLastError(), "top2");
  }
  return J3DG_OK;
}

int j3dg_learned_predict(j3dg_learned* l, const j3dg_ray* rays, uint32_t n, uint32_t* top2) {
  return j3dg_learned_predict_impl(l, rays, n, top2, 1);
}

int j3dg_learned_predict_impl(j3dg_learned* l, const j3dg_ray* rays, uint32_t n, uint32_t* top2, int impl) {
  if (!l || (n && (!rays || !top2)) || (impl != 0 && impl != 1)) return J3DG_ERR_INVALID_ARGUMENT;
  if (n == 0) return J3DG_OK;
  cudaSetDevice(l->ctx->device);
  j3dg_ray* dr = nullptr;
  uint32_t* dt = nullptr;
  LCK(cudaMallocAsync((void**)&dr, sizeof(j3dg_ray) * n, LS(l)), "predict");
  LCK(cudaMallocAsync((void**)&dt, sizeof(uint32_t) * 2 * n, LS(l)), "predict");
  LCK(cudaMemcpyAsync(dr, rays, sizeof(j3dg_ray) * n, cudaMemcpyDefault, LS(l)), "predict");
  int rc = predict_device(l, dr, n, dt, impl);
  if (rc == J3DG_OK) LCK(cudaMemcpyAsync(top2, dt, sizeof(uint32_t) * 2 * n, cudaMemcpyDefault, LS(l)), "predict");
  cudaFreeAsync(dr, LS(l));
  cudaFreeAsync(dt, LS(l));
  LCK(cudaStreamSynchronize(LS(l)), "predict");
  if (rc == J3DG_OK) rc = j3dg_ctx_synchronize(l->ctx);
  return rc;
}

}  // extern "C"

namespace j3dg {

// Learned closest hits of device rays into device hits, queued on the
// context stream (no synchronisation): top-2 clusters by the fused network,
// then the exact traversal seeded by them.
int learned_hits_device(j3dg_learned* l, const j3dg_ray* d_rays, uint32_t n, j3dg_hit* d_hits) {
  if (n == 0) return J3DG_OK;
  uint32_t* dt = nullptr;
  LCK(cudaMallocAsync((void**)&dt, sizeof(uint32_t) * 2 * n, LS(l)), "learned hits");
  int rc = predict_device(l, d_rays, n, dt);
  const DevInst* dinst = nullptr;
  if (rc == J3DG_OK) rc = mesh_devinst(l->ctx, l->mesh, &dinst);
  if (rc == J3DG_OK) {
    k_rays_learned<<<(n + 127) / 128, 128, 0, LS(l)>>>(dinst, d_rays, n, dt, l->d_roots, l->n_clusters, d_hits,
                                                      l->ctx->d_status, ctx_counters(l->ctx), nullptr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = ctx_fail(l->ctx, J3DG_ERR_CUDA, std::string("learned hits: ") + cudaGetErrorString(e));
  }
  cudaFreeAsync(dt, LS(l));
  return rc;
}

const j3dg_mesh* learned_mesh(const j3dg_learned* l) { return l->mesh; }
j3dg_ctx* learned_ctx(const j3dg_learned* l) { return l->ctx; }

}  // namespace j3dg

extern "C" {

int j3dg_learned_find_closest(j3dg_learned* l, const j3dg_ray* rays, uint32_t n, j3dg_hit* hits) {
  return j3dg_learned_find_closest_stats(l, rays, n, hits, nullptr);
}

int j3dg_learned_find_closest_stats(j3dg_learned* l, const j3dg_ray* rays, uint32_t n, j3dg_hit* hits,
                                    uint64_t stats[4]) {
  if (!l || (n && (!rays || !hits))) return J3DG_ERR_INVALID_ARGUMENT;
  if (stats)
    for (int k = 0; k < 4; ++k) stats[k] = 0;
  if (n == 0) return J3DG_OK;
  j3dg_ctx* c = l->ctx;
  cudaSetDevice(c->device);
  cudaPointerAttributes ar, ah;
  const bool rays_dev = cudaPointerGetAttributes(&ar, rays) == cudaSuccess && ar.type == cudaMemoryTypeDevice;
  const bool hits_dev = cudaPointerGetAttributes(&ah, hits) == cudaSuccess && ah.type == cudaMemoryTypeDevice;
  cudaGetLastError();
  j3dg_ray* dr = const_cast<j3dg_ray*>(rays);
  j3dg_hit* dh = hits;
  uint32_t* dt = nullptr;
  if (!rays_dev) {
    LCK(cudaMallocAsync((void**)&dr, sizeof(j3dg_ray) * n, LS(l)), "learned find");
    LCK(cudaMemcpyAsync(dr, rays, sizeof(j3dg_ray) * n, cudaMemcpyHostToDevice, LS(l)), "learned find");
  }
  if (!hits_dev) LCK(cudaMallocAsync((void**)&dh, sizeof(j3dg_hit) * n, LS(l)), "learned find");
  LCK(cudaMallocAsync((void**)&dt, sizeof(uint32_t) * 2 * n, LS(l)), "learned find");
  unsigned long long* d_phase = nullptr;
  if (stats) {
    LCK(cudaMallocAsync((void**)&d_phase, sizeof(unsigned long long) * 4, LS(l)), "learned find");
    LCK(cudaMemsetAsync(d_phase, 0, sizeof(unsigned long long) * 4, LS(l)), "learned find");
  }
  int rc = predict_device(l, dr, n, dt);
  const DevInst* dinst = nullptr;
  if (rc == J3DG_OK) rc = j3dg::mesh_devinst(c, l->mesh, &dinst);
  if (rc == J3DG_OK) {
    unsigned long long* counters = j3dg::ctx_counters(c);
    j3dg::k_rays_learned<<<(n + 127) / 128, 128, 0, LS(l)>>>(dinst, dr, n, dt, l->d_roots, l->n_clusters, dh,
                                                            c->d_status, counters, d_phase);
    LCK(cudaGetLastError(), "learned find");
  }
  if (stats) {
    unsigned long long h[4] = {0, 0, 0, 0};
    LCK(cudaMemcpyAsync(h, d_phase, sizeof(h), cudaMemcpyDeviceToHost, LS(l)), "learned find");
    LCK(cudaStreamSynchronize(LS(l)), "learned find");
    for (int k = 0; k < 4; ++k) stats[k] = h[k];
    cudaFreeAsync(d_phase, LS(l));
  }
  if (!hits_dev) {
    LCK(cudaMemcpyAsync(hits, dh, sizeof(j3dg_hit) * n, cudaMemcpyDeviceToHost, LS(l)), "learned find");
    cudaFreeAsync(dh, LS(l));
  }
  if (!rays_dev) cudaFreeAsync(dr, LS(l));
  cudaFreeAsync(dt, LS(l));
  LCK(cudaStreamSynchronize(LS(l)), "learned find");
  uint32_t st = 0;
  LCK(cudaMemcpy(&st, c->d_status, sizeof(st), cudaMemcpyDeviceToHost), "learned find");
  if (st) return j3dg::ctx_fail(c, J3DG_ERR_DEVICE_STATUS, "learned find: device status raised");
  return rc;
}

// Checkpoint: a small header and the fp32 parameters.
int j3dg_learned_save(j3dg_learned* l, const char* path) {
  if (!l || !path) return J3DG_ERR_INVALID_ARGUMENT;
  std::vector<float> p(l->L.total);
  if (int rc = j3dg_learned_get_params(l, p.data())) return rc;
  FILE* f = fopen(path, "wb");
  if (!f) return j3dg::ctx_fail(l->ctx, J3DG_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
  const uint32_t hdr[4] = {0x4A334C4Du, 1u, l->n_clusters, (uint32_t)l->L.total};
  bool ok = fwrite(hdr, sizeof(hdr), 1, f) == 1 && fwrite(p.data(), sizeof(float), p.size(), f) == p.size();
  ok = (fclose(f) == 0) && ok;
  return ok ? J3DG_OK : j3dg::ctx_fail(l->ctx, J3DG_ERR_INVALID_ARGUMENT, "checkpoint write failed");
}

int j3dg_learned_load(j3dg_learned* l, const char* path) {
  if (!l || !path) return J3DG_ERR_INVALID_ARGUMENT;
  FILE* f = fopen(path, "rb");
  if (!f) return j3dg::ctx_fail(l->ctx, J3DG_ERR_INVALID_ARGUMENT, std::string("cannot read ") + path);
  uint32_t hdr[4];
  std::vector<float> p(l->L.total);
  bool ok = fread(hdr, sizeof(hdr), 1, f) == 1 && hdr[0] == 0x4A334C4Du && hdr[1] == 1u && hdr[2] == l->n_clusters &&
            hdr[3] == (uint32_t)l->L.total && fread(p.data(), sizeof(float), p.size(), f) == p.size();
  fclose(f);
  if (!ok) return j3dg::ctx_fail(l->ctx, J3DG_ERR_INVALID_ARGUMENT, "checkpoint does not match this network");
  return j3dg_learned_set_params(l, p.data());
}

}  // extern "C"
