"""The network's bf16 tensor-core GEMMs against an fp32 reference:
impl 1 = tcgen05 with the accumulator in tensor memory, impl 0 = the same
split over K ranges whose CTAs add into C (the weight gradients' form).
C = A . Bt^T with A [M x K], Bt [N x K] bf16; the reference multiplies the
same bf16 values in float64, and the tolerance is 1e-5 of the sum of |a b|
(fp32 accumulation in another order)."""
import numpy as np
import pytest


def _case(M, N, K, seed):
    import torch
    g = torch.Generator().manual_seed(seed)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16)
    Bt = torch.randn(N, K, generator=g).to(torch.bfloat16)
    ref = A.double() @ Bt.double().T
    mag = A.double().abs() @ Bt.double().abs().T
    return A, Bt, ref.numpy(), mag.numpy()


def _run(ctx, A, Bt, impl):
    import torch
    from j3d_gb300 import _ffi
    from j3d_gb300.scene import _check
    M, K = A.shape
    N = Bt.shape[0]
    dA, dB = A.cuda().contiguous(), Bt.cuda().contiguous()
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    _check(ctx.h, _ffi.lib().j3dg_gemm_bf16(ctx.h, dA.data_ptr(), dB.data_ptr(), C.data_ptr(), M, N, K, impl))
    return C.cpu().double().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(128, 128, 64), (128, 256, 64), (256, 384, 320), (512, 1024, 256),
                                   (2048, 4096, 128)])
@pytest.mark.parametrize("impl", [1, 0])
def test_gemm_matches_fp32_reference(gpu_ctx, shape, impl):
    M, N, K = shape
    A, Bt, ref, mag = _case(M, N, K, seed=M + N + K)
    C = _run(gpu_ctx, A, Bt, impl)
    err = np.abs(C - ref)
    assert np.isfinite(C).all()
    assert (err <= 1e-5 * mag + 1e-30).all(), float((err / (mag + 1e-30)).max())


@pytest.mark.gpu
def test_gemm_rejects_unsupported_shapes(gpu_ctx):
    import torch
    from j3d_gb300 import J3dgError, _ffi
    from j3d_gb300.scene import _check
    A = torch.zeros(128, 96, dtype=torch.bfloat16, device="cuda")
    B = torch.zeros(128, 96, dtype=torch.bfloat16, device="cuda")
    C = torch.zeros(128, 128, dtype=torch.float32, device="cuda")
    with pytest.raises(J3dgError):  # K % 64 != 0 on the tcgen05 path
        _check(gpu_ctx.h, _ffi.lib().j3dg_gemm_bf16(gpu_ctx.h, A.data_ptr(), B.data_ptr(), C.data_ptr(),
                                                    128, 128, 96, 1))


@pytest.mark.gpu
def test_bounded_wait_times_out_and_reports(gpu_ctx):
    """The tcgen05 kernel with its MMAs withheld: nothing ever completes its
    mbarrier, the bounded wait runs out, the kernel raises the status word,
    frees its tensor memory and returns; the context keeps working."""
    import torch
    from j3d_gb300 import J3dgError, _ffi
    from j3d_gb300.scene import _check
    A, Bt, ref, mag = _case(128, 128, 64, seed=5)
    dA, dB = A.cuda(), Bt.cuda()
    C = torch.zeros(128, 128, dtype=torch.float32, device="cuda")
    with pytest.raises(J3dgError) as e:
        _check(gpu_ctx.h, _ffi.lib().j3dg_gemm_bf16(gpu_ctx.h, dA.data_ptr(), dB.data_ptr(), C.data_ptr(),
                                                    128, 128, 64, 2))
    assert e.value.status == 5  # J3DG_ERR_DEVICE_STATUS
    assert float(C.abs().max()) == 0.0  # no epilogue ran
    # the status word was cleared by the failing call; the next one works
    Cn = _run(gpu_ctx, A, Bt, 1)
    assert (np.abs(Cn - ref) <= 1e-5 * mag + 1e-30).all()
