// mlp.cuh -- bf16 tensor-core GEMM (tcgen05, accumulator in tensor memory)
// with fused epilogues for the ray -> cluster network of the learned-tmax
// traversal (umma_gemm.cu), and the network's activation.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace j3dg {

enum Epilogue : int {
  EPI_F32 = 0,            // C (float) = acc
  EPI_F32_ACCUM = 1,      // C (float) += acc (split-K over `splits` K ranges, atomics; C zeroed first)
  EPI_BIAS_GELU = 2,      // Z (bf16) = acc + bias; C (bf16) = gelu(Z)
  EPI_BIAS_F32 = 3,       // C (float) = acc + bias
  EPI_GELU_BWD = 4,       // C (bf16) = acc * gelu'(Z), Z given (bf16)
};

// C[M x N] = epilogue(A[M x K] . Bt[N x K]^T). M % 128, N % 128, K % 64 ==
// 0; lda, ldb multiples of 8; 16-byte aligned pointers. Z has C's shape
// and ldc. Ct (optional, bf16 epilogues): C also written transposed,
// Ct[n * ldct + m]. A timed-out wait raises J3DG_DEV_VISIT_CAP.
struct UmmaArgs {
  const __nv_bfloat16* A;
  const __nv_bfloat16* Bt;
  void* C;
  int M, N, K, lda, ldb, ldc;
  int epi;
  const float* bias;
  __nv_bfloat16* Z;
  __nv_bfloat16* Ct;
  int ldct;
  int splits;
};
// withhold != 0 issues no MMA and no commit, so the kernel's bounded wait runs
// out (the failure path, exercised by a test)
cudaError_t umma_gemm_bf16(const UmmaArgs& g, uint32_t* status, cudaStream_t st, int withhold = 0);

// tanh(u) = 1 - 2 / (e^(2u) + 1) with the hardware exp2 approximation: its
// error is a few ulp of 1, which is what the activation adds tanh to; the
// results are rounded to bf16 anyway.
__device__ __forceinline__ float tanh_fast(float u) { return 1.f - __fdividef(2.f, __expf(2.f * u) + 1.f); }

// tanh-form GELU and its derivative (the network's activation)
__device__ __forceinline__ float gelu_f(float x) {
  const float k = 0.7978845608028654f;  // sqrt(2 / pi)
  return 0.5f * x * (1.f + tanh_fast(k * (x + 0.044715f * x * x * x)));
}
__device__ __forceinline__ float gelu_grad_f(float x) {
  const float k = 0.7978845608028654f;
  const float u = k * (x + 0.044715f * x * x * x);
  const float th = tanh_fast(u);
  return 0.5f * (1.f + th) + 0.5f * x * (1.f - th * th) * k * (1.f + 3.f * 0.044715f * x * x);
}

}  // namespace j3dg
