// mlp_gemm.cu -- bf16 tensor-core GEMM (mma.sync m16n8k16, fp32 accumulate)
// with the fused epilogues of the ray -> cluster network; see mlp.cuh.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp.cuh"

namespace j3dg {

namespace {

const int BM = 128, BN = 128, BK = 32, KPAD = 40;  // smem rows padded to 80 B

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldmatrix_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smem_addr(p)));
}

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Loads this thread's share of a 128 x 32 operand tile into registers.
// rows_contig: memory rows are the tile's 128 rows (k contiguous);
// otherwise memory rows are the 32 k's (the 128 contiguous).
template <bool ROWS_CONTIG>
__device__ __forceinline__ void load_tile(const __nv_bfloat16* base, int ld, int r0, int k0, uint4 (&v)[2]) {
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int idx = t + j * 256;
    if (ROWS_CONTIG) {
      const int row = idx >> 2, chunk = idx & 3;
      v[j] = *reinterpret_cast<const uint4*>(base + (size_t)(r0 + row) * ld + k0 + chunk * 8);
    } else {
      const int krow = idx >> 4, chunk = idx & 15;
      v[j] = *reinterpret_cast<const uint4*>(base + (size_t)(k0 + krow) * ld + r0 + chunk * 8);
    }
  }
}

template <bool ROWS_CONTIG>
__device__ __forceinline__ void store_tile(__nv_bfloat16 (*S)[KPAD], const uint4 (&v)[2]) {
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int idx = t + j * 256;
    if (ROWS_CONTIG) {
      const int row = idx >> 2, chunk = idx & 3;
      *reinterpret_cast<uint4*>(&S[row][chunk * 8]) = v[j];
    } else {
      const int krow = idx >> 4, chunk = idx & 15;
      const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&v[j]);
#pragma unroll
      for (int q = 0; q < 8; ++q) S[chunk * 8 + q][krow] = e[q];
    }
  }
}

template <bool AT, bool BT, int EPI>
__global__ void __launch_bounds__(256) k_gemm(const GemmArgs g) {
  __shared__ __align__(16) __nv_bfloat16 As[2][BM][KPAD];
  __shared__ __align__(16) __nv_bfloat16 Bs[2][BN][KPAD];
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 2) * 64, wn = (warp & 3) * 32;
  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;

  uint4 ra[2], rb[2];
  load_tile<!AT>(g.A, g.lda, m0, 0, ra);
  load_tile<BT>(g.B, g.ldb, n0, 0, rb);
  store_tile<!AT>(As[0], ra);
  store_tile<BT>(Bs[0], rb);
  __syncthreads();
  const int nk = g.K / BK;
  for (int kt = 0; kt < nk; ++kt) {
    const int cur = kt & 1;
    if (kt + 1 < nk) {
      load_tile<!AT>(g.A, g.lda, m0, (kt + 1) * BK, ra);
      load_tile<BT>(g.B, g.ldb, n0, (kt + 1) * BK, rb);
    }
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[4][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 4; ++i)
        ldmatrix_x4(af[i][0], af[i][1], af[i][2], af[i][3],
                    &As[cur][wm + i * 16 + (lane & 15)][kk + (lane >> 4) * 8]);
#pragma unroll
      for (int j = 0; j < 4; j += 2)
        ldmatrix_x4(bf[j][0], bf[j][1], bf[j + 1][0], bf[j + 1][1],
                    &Bs[cur][wn + j * 8 + (lane & 7) + ((lane >> 4) << 3)][kk + ((lane >> 3) & 1) * 8]);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j][0], bf[j][1]);
    }
    if (kt + 1 < nk) {
      store_tile<!AT>(As[cur ^ 1], ra);
      store_tile<BT>(Bs[cur ^ 1], rb);
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = m0 + wm + i * 16 + (lane >> 2) + h * 8;
        const int col = n0 + wn + j * 8 + (lane & 3) * 2;
        float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
        const size_t o = (size_t)row * g.ldc + col;
        if (EPI == EPI_F32) {
          *reinterpret_cast<float2*>(static_cast<float*>(g.C) + o) = make_float2(v0, v1);
        } else if (EPI == EPI_F32_ACCUM) {
          float2* p = reinterpret_cast<float2*>(static_cast<float*>(g.C) + o);
          float2 c = *p;
          *p = make_float2(c.x + v0, c.y + v1);
        } else if (EPI == EPI_BIAS_F32) {
          *reinterpret_cast<float2*>(static_cast<float*>(g.C) + o) = make_float2(v0 + g.bias[col], v1 + g.bias[col + 1]);
        } else if (EPI == EPI_BIAS_GELU) {
          const __nv_bfloat162 z = __floats2bfloat162_rn(v0 + g.bias[col], v1 + g.bias[col + 1]);
          *reinterpret_cast<__nv_bfloat162*>(g.Z + o) = z;
          const float2 zf = __bfloat1622float2(z);
          *reinterpret_cast<__nv_bfloat162*>(static_cast<__nv_bfloat16*>(g.C) + o) =
              __floats2bfloat162_rn(gelu_f(zf.x), gelu_f(zf.y));
        } else if (EPI == EPI_GELU_BWD) {
          const float2 zf = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(g.Z + o));
          *reinterpret_cast<__nv_bfloat162*>(static_cast<__nv_bfloat16*>(g.C) + o) =
              __floats2bfloat162_rn(v0 * gelu_grad_f(zf.x), v1 * gelu_grad_f(zf.y));
        }
      }
}

template <bool AT, bool BT>
cudaError_t gemm_epi(const GemmArgs& g, int epi, cudaStream_t st) {
  dim3 grid(g.N / BN, g.M / BM);
  switch (epi) {
    case EPI_F32: k_gemm<AT, BT, EPI_F32><<<grid, 256, 0, st>>>(g); break;
    case EPI_F32_ACCUM: k_gemm<AT, BT, EPI_F32_ACCUM><<<grid, 256, 0, st>>>(g); break;
    case EPI_BIAS_GELU: k_gemm<AT, BT, EPI_BIAS_GELU><<<grid, 256, 0, st>>>(g); break;
    case EPI_BIAS_F32: k_gemm<AT, BT, EPI_BIAS_F32><<<grid, 256, 0, st>>>(g); break;
    case EPI_GELU_BWD: k_gemm<AT, BT, EPI_GELU_BWD><<<grid, 256, 0, st>>>(g); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t gemm_bf16(const GemmArgs& g, bool at, bool bt, int epi, cudaStream_t st) {
  if (g.M % BM || g.N % BN || g.K % BK || g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaErrorInvalidValue;
  if (at) return bt ? gemm_epi<true, true>(g, epi, st) : gemm_epi<true, false>(g, epi, st);
  return bt ? gemm_epi<false, true>(g, epi, st) : gemm_epi<false, false>(g, epi, st);
}

}  // namespace j3dg
