// umma_gemm.cu -- bf16 GEMM on the tcgen05 tensor cores with the
// accumulator in tensor memory, and the fused epilogues the network's
// training and layer-by-layer inference need:
//   C[M x N] = epilogue(A[M x K] . Bt[N x K]^T)   (A and Bt row-major, K-major)
// One CTA of 4 warps per 128 x BN tile. K advances in chunks of 64 through a
// two-stage shared-memory ring: all threads copy the next chunk into the
// canonical no-swizzle layout while the tensor core works on the previous
// one; thread 0 issues the four K = 16 MMAs of a chunk and commits them to
// the stage's mbarrier, which frees the stage for the chunk after next.
// The epilogue moves each warp's 32 accumulator rows out of TMEM with
// tcgen05.ld. Every wait is bounded (clock budget); on timeout the kernel
// raises J3DG_DEV_VISIT_CAP in the status word, skips the epilogue and still
// frees its TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>

#include "../../include/j3dg.h"
#include "internal.h"
#include "mlp.cuh"
#include "umma.cuh"

namespace j3dg {

namespace {

const int kChunkK = 64;                     // K per stage
const long long kWaitBudget = 500000000ll;  // ~0.25 s at 2 GHz
const uint32_t kTmemCols = 512;             // whole TMEM: one CTA per SM

template <int BN>
struct GemmSmem {
  static constexpr uint32_t a_bytes = 128 * kChunkK * 2;  // 16 KB
  static constexpr uint32_t b_bytes = BN * kChunkK * 2;
  static constexpr uint32_t stage_bytes = a_bytes + b_bytes;
  // + alignment slack; at least 120 KB so that one CTA runs per SM (each
  // takes all 512 TMEM columns)
  static constexpr uint32_t total = 2 * stage_bytes + 1024 > 122880u ? 2 * stage_bytes + 1024 : 122880u;
};

// Copies rows [r0, r0 + rows) x K-chunk [k0, k0 + 64) of a row-major bf16
// matrix into the canonical layout (8 core matrices along K).
__device__ __forceinline__ void copy_chunk(const __nv_bfloat16* __restrict__ src, int ld, int r0, int rows, int k0,
                                           uint8_t* dst) {
  const int pieces = rows * (kChunkK / 8);
  for (int p = threadIdx.x; p < pieces; p += blockDim.x) {
    const int row = p >> 3, kg = p & 7;
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(src + (size_t)(r0 + row) * ld + k0 + kg * 8));
    *reinterpret_cast<uint4*>(dst + umma::tile_offset(row, kg * 8, kChunkK / 8)) = v;
  }
}

// The epilogue of thread `lane` of warp w: accumulator row m0 + 32 w + lane,
// BN columns from n0, 16 per TMEM load.
//   EPI_F32         C (float) = acc
//   EPI_F32_ACCUM   C (float) += acc, with atomics (split-K: blockIdx.z
//                   takes one K range; C starts at zero)
//   EPI_BIAS_F32    C (float) = acc + bias
//   EPI_BIAS_GELU   Z (bf16) = acc + bias; C (bf16) = gelu(Z)
//   EPI_GELU_BWD    C (bf16) = acc * gelu'(Z), Z given
// With Ct, the bf16 C is also written transposed (Ct[n][m], row stride
// ldct): the next GEMMs read it K-major. Rounding is per element, bias ->
// bf16 -> GELU -> bf16, as the inference kernel rounds.
template <int BN, int EPI>
__device__ __forceinline__ void epilogue(const UmmaArgs& g, uint32_t taddr, int m0, int n0, int warp, int lane) {
  const int row = m0 + warp * 32 + lane;
#pragma unroll 1
  for (int j = 0; j < BN / 16; ++j) {
    float v[16];
    umma::ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)(j * 16), v);
    const int col = n0 + j * 16;
    if (EPI == EPI_F32 || EPI == EPI_F32_ACCUM || EPI == EPI_BIAS_F32) {
      float* c = static_cast<float*>(g.C) + (size_t)row * g.ldc + col;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float4 o = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        if (EPI == EPI_BIAS_F32) {
          const float4 b = __ldg(reinterpret_cast<const float4*>(g.bias + col) + q);
          o = make_float4(o.x + b.x, o.y + b.y, o.z + b.z, o.w + b.w);
        }
        if (EPI == EPI_F32_ACCUM)
          atomicAdd(reinterpret_cast<float4*>(c) + q, o);
        else
          reinterpret_cast<float4*>(c)[q] = o;
      }
    } else {
      __nv_bfloat16 out[16];
      __nv_bfloat16* z = g.Z + (size_t)row * g.ldc + col;
      if (EPI == EPI_BIAS_GELU) {
        __nv_bfloat16 zz[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          zz[i] = __float2bfloat16_rn(v[i] + __ldg(g.bias + col + i));
          out[i] = __float2bfloat16_rn(gelu_f(__bfloat162float(zz[i])));
        }
        reinterpret_cast<uint4*>(z)[0] = reinterpret_cast<const uint4*>(zz)[0];
        reinterpret_cast<uint4*>(z)[1] = reinterpret_cast<const uint4*>(zz)[1];
      } else {  // EPI_GELU_BWD
        __nv_bfloat16 zz[16];
        reinterpret_cast<uint4*>(zz)[0] = reinterpret_cast<const uint4*>(z)[0];
        reinterpret_cast<uint4*>(zz)[1] = reinterpret_cast<const uint4*>(z)[1];
#pragma unroll
        for (int i = 0; i < 16; ++i) out[i] = __float2bfloat16_rn(v[i] * gelu_grad_f(__bfloat162float(zz[i])));
      }
      __nv_bfloat16* c = static_cast<__nv_bfloat16*>(g.C) + (size_t)row * g.ldc + col;
      reinterpret_cast<uint4*>(c)[0] = reinterpret_cast<const uint4*>(out)[0];
      reinterpret_cast<uint4*>(c)[1] = reinterpret_cast<const uint4*>(out)[1];
      if (g.Ct) {
#pragma unroll
        for (int i = 0; i < 16; ++i) g.Ct[(size_t)(col + i) * g.ldct + row] = out[i];
      }
    }
  }
}

template <int BN, int EPI>
__global__ void __launch_bounds__(128, 1) k_umma_gemm(const UmmaArgs g, uint32_t* status, int withhold) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t taddr_s;
  uint8_t* sm = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * 128, n0 = blockIdx.x * BN;
  using L = GemmSmem<BN>;

  // a CTA that timed out raised the status word: the rest of the grid stops
  if (*reinterpret_cast<volatile uint32_t*>(status) & J3DG_DEV_VISIT_CAP) return;
  if (warp == 0) {
    umma::tmem_alloc(umma::smem_u32(&taddr_s), kTmemCols);
    umma::tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    umma::mbar_init(umma::smem_u32(&mbar[0]), 1);
    umma::mbar_init(umma::smem_u32(&mbar[1]), 1);
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t taddr = taddr_s;
  constexpr uint32_t idesc = umma::idesc_bf16_f32(128, BN);

  // this CTA's K range (split-K over blockIdx.z)
  const int nk_all = g.K / kChunkK;
  const int kc0 = (int)((long long)nk_all * blockIdx.z / gridDim.z);
  const int kc1 = (int)((long long)nk_all * (blockIdx.z + 1) / gridDim.z);
  const int nk = kc1 - kc0;
  bool ok = true;
  for (int it = 0; it < nk; ++it) {
    const int s = it & 1;
    uint8_t* sA = sm + s * L::stage_bytes;
    uint8_t* sB = sA + L::a_bytes;
    if (it >= 2) ok = umma::mbar_wait(umma::smem_u32(&mbar[s]), ((it - 2) >> 1) & 1, kWaitBudget);
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    copy_chunk(g.A, g.lda, m0, 128, (kc0 + it) * kChunkK, sA);
    copy_chunk(g.Bt, g.ldb, n0, BN, (kc0 + it) * kChunkK, sB);
    umma::fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0 && !withhold) {  // withhold: nothing completes the barrier (failure-path test)
      umma::fence_after_sync();
      const uint32_t a0 = umma::smem_u32(sA), b0 = umma::smem_u32(sB);
#pragma unroll
      for (int k = 0; k < kChunkK / 16; ++k)
        umma::mma_bf16(taddr, umma::desc(a0 + k * 256, 128, (kChunkK / 8) * 128),
                       umma::desc(b0 + k * 256, 128, (kChunkK / 8) * 128), idesc, (it | k) != 0);
      umma::commit(umma::smem_u32(&mbar[s]));
    }
  }
  if (ok && nk > 0) ok = umma::mbar_wait(umma::smem_u32(&mbar[(nk - 1) & 1]), ((nk - 1) >> 1) & 1, kWaitBudget);
  ok = __syncthreads_and(ok);
  umma::fence_after_sync();
  if (ok && nk > 0) {
    epilogue<BN, EPI>(g, taddr, m0, n0, warp, lane);
  } else if (!ok && threadIdx.x == 0) {
    atomicOr(status, J3DG_DEV_VISIT_CAP);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    umma::fence_after_sync();
    umma::tmem_dealloc(taddr, kTmemCols);
  }
}

template <int BN, int EPI>
cudaError_t launch(const UmmaArgs& g, uint32_t* status, cudaStream_t st, int withhold) {
  const uint32_t smem = GemmSmem<BN>::total;
  cudaError_t e = cudaFuncSetAttribute(k_umma_gemm<BN, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(g.N / BN, g.M / 128, EPI == EPI_F32_ACCUM ? g.splits : 1);
  k_umma_gemm<BN, EPI><<<grid, 128, smem, st>>>(g, status, withhold);
  return cudaGetLastError();
}

template <int BN>
cudaError_t launch_epi(const UmmaArgs& g, uint32_t* status, cudaStream_t st, int withhold) {
  switch (g.epi) {
    case EPI_F32: return launch<BN, EPI_F32>(g, status, st, withhold);
    case EPI_F32_ACCUM: return launch<BN, EPI_F32_ACCUM>(g, status, st, withhold);
    case EPI_BIAS_F32: return launch<BN, EPI_BIAS_F32>(g, status, st, withhold);
    case EPI_BIAS_GELU: return launch<BN, EPI_BIAS_GELU>(g, status, st, withhold);
    case EPI_GELU_BWD: return launch<BN, EPI_GELU_BWD>(g, status, st, withhold);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t umma_gemm_bf16(const UmmaArgs& g, uint32_t* status, cudaStream_t st, int withhold) {
  const bool bf16_out = g.epi == EPI_BIAS_GELU || g.epi == EPI_GELU_BWD;
  if (g.M <= 0 || g.N <= 0 || g.K <= 0 || g.M % 128 || g.K % kChunkK || g.lda % 8 || g.ldb % 8 ||
      g.ldc % (bf16_out ? 16 : 4) || ((uintptr_t)g.A & 15) || ((uintptr_t)g.Bt & 15) || ((uintptr_t)g.C & 15) ||
      (bf16_out && (!g.Z || ((uintptr_t)g.Z & 15))) || ((g.epi == EPI_BIAS_F32 || g.epi == EPI_BIAS_GELU) && !g.bias) ||
      (g.epi == EPI_BIAS_F32 && ((uintptr_t)g.bias & 15)) || (g.Ct && (!bf16_out || g.ldct < g.M)) ||
      (g.epi == EPI_F32_ACCUM && (g.splits < 1 || g.splits > g.K / kChunkK)))
    return cudaErrorInvalidValue;
  if (g.N % 256 == 0) return launch_epi<256>(g, status, st, withhold);
  if (g.N % 128 == 0) return launch_epi<128>(g, status, st, withhold);
  return cudaErrorInvalidValue;
}

}  // namespace j3dg

namespace j3dg {
int ctx_fail(j3dg_ctx* c, int code, const std::string& msg);
}

extern "C" int j3dg_gemm_bf16(j3dg_ctx* c, const void* A, const void* Bt, float* C, uint32_t M, uint32_t N, uint32_t K,
                              int impl) {
  if (!c || !A || !Bt || !C) return J3DG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  ++c->stream_ops;
  cudaStream_t st = (cudaStream_t)c->stream;
  cudaError_t e;
  if (impl >= 0 && impl <= 2) {
    j3dg::UmmaArgs g{};
    g.A = (const __nv_bfloat16*)A;
    g.Bt = (const __nv_bfloat16*)Bt;
    g.C = C;
    g.M = (int)M;
    g.N = (int)N;
    g.K = (int)K;
    g.lda = g.ldb = (int)K;
    g.ldc = (int)N;
    g.epi = j3dg::EPI_F32;
    if (impl == 0) {  // split-K into a zeroed C
      g.epi = j3dg::EPI_F32_ACCUM;
      g.splits = std::max(1, std::min(4, (int)K / 64));
      e = cudaMemsetAsync(C, 0, sizeof(float) * (size_t)M * N, st);
      if (e == cudaSuccess) e = j3dg::umma_gemm_bf16(g, c->d_status, st, 0);
    } else {
      e = j3dg::umma_gemm_bf16(g, c->d_status, st, impl == 2);
    }
  } else {
    return j3dg::ctx_fail(c, J3DG_ERR_INVALID_ARGUMENT, "gemm_bf16: impl must be 0, 1 or 2");
  }
  if (e == cudaErrorInvalidValue) return j3dg::ctx_fail(c, J3DG_ERR_INVALID_ARGUMENT, "gemm_bf16: unsupported shape");
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return j3dg::ctx_fail(c, J3DG_ERR_CUDA, std::string("gemm_bf16: ") + cudaGetErrorString(e));
  return j3dg_ctx_synchronize(c);
}

