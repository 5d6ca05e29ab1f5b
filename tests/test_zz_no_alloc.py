"""j3dg_voxelize_noalloc: the voxel grid for callers that must not allocate
device memory while they run (a viewer or server that reserved its memory
budget up front). It must give exactly what j3dg_voxelize gives, call after
call, although every call reuses one fixed scratch array inside the library;
and it must refuse grids larger than that array instead of allocating.

This file is collected last on purpose, and passes both alone in a fresh
process and after the rest of the suite."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_VOXELS = 1 << 21  # J3DG_NOALLOC_MAX_VOXELS in include/j3dg.h


def _grid(lib, ctx, mesh, max_dim, noalloc, out=None):
    dims = (C.c_uint32 * 3)()
    f = lib.j3dg_voxelize_noalloc if noalloc else lib.j3dg_voxelize
    assert f(ctx.h, mesh.h, max_dim, dims, None, 0) == 0
    n = int(dims[0]) * int(dims[1]) * int(dims[2])
    if out is None:
        out = np.zeros(n, np.uint8)
        ptr = out.ctypes.data
    else:
        ptr = out.data_ptr()
    st = f(ctx.h, mesh.h, max_dim, dims, ptr, n)
    assert st == 0, lib.j3dg_last_error(ctx.h)
    return out, (int(dims[2]), int(dims[1]), int(dims[0]))


def test_noalloc_voxel_grid_equals_the_allocating_call(product_lib, gpu_ctx):
    from j3d_gb300 import Mesh, workloads as W
    lib = product_lib
    rng = np.random.default_rng(17)
    V1, T1 = W.icosphere(4, W.SEED_BASE + 60)
    V2, T2 = W.torus(160, 80, seed=W.SEED_BASE + 61)
    m1 = Mesh(gpu_ctx, V1, T1)
    m2 = Mesh(gpu_ctx, V2, T2)
    m2.set_vertex_colors(rng.uniform(0, 1, size=V2.shape).astype(np.float32))
    # two calls in a row (different meshes and sizes), then the first again:
    # the shared scratch must not carry anything from one call to the next
    for mesh, max_dim in ((m1, 100), (m2, 64), (m1, 100)):
        want, shape = _grid(lib, gpu_ctx, mesh, max_dim, noalloc=False)
        got, shape2 = _grid(lib, gpu_ctx, mesh, max_dim, noalloc=True)
        assert shape == shape2
        assert np.array_equal(got, want), f"{(got != want).sum()} voxels differ"
        assert (want != 0).sum() > 100


def test_noalloc_device_output_and_size_limit(product_lib, gpu_ctx):
    import torch

    from j3d_gb300 import Mesh, workloads as W
    lib = product_lib
    V, T = W.icosphere(3, W.SEED_BASE + 62)
    m = Mesh(gpu_ctx, V, T)
    want, shape = _grid(lib, gpu_ctx, m, 90, noalloc=False)
    dev = torch.zeros(want.size, dtype=torch.uint8, device="cuda")
    got, _ = _grid(lib, gpu_ctx, m, 90, noalloc=True, out=dev)
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy(), want)
    # 1024^3 voxels exceed the fixed scratch: refused with a message, nothing written
    dims = (C.c_uint32 * 3)()
    big = np.zeros(16, np.uint8)
    st = lib.j3dg_voxelize_noalloc(gpu_ctx.h, m.h, 1024, dims, big.ctypes.data, big.size)
    assert st == 1  # J3DG_ERR_INVALID_ARGUMENT
    msg = lib.j3dg_last_error(gpu_ctx.h).decode()
    assert "scratch holds %d" % MAX_VOXELS in msg
    assert int(dims[0]) * int(dims[1]) * int(dims[2]) > MAX_VOXELS
    assert not big.any()


def test_noalloc_calls_allocate_no_device_memory(product_lib, gpu_ctx):
    """What the entry point exists for: once warm, calls with host and with
    device output leave the device's free memory, the context's canvas pool
    and the device's default stream-ordered pool exactly as they were
    (cudaMemGetInfo and the pools' reserved / used bytes, read through
    j3dg_ctx_memory), and every call still gives the allocating call's grid."""
    import torch

    from j3d_gb300 import Mesh, workloads as W
    lib = product_lib
    V, T = W.torus(120, 60, seed=W.SEED_BASE + 63)
    m = Mesh(gpu_ctx, V, T)
    want, _ = _grid(lib, gpu_ctx, m, 110, noalloc=False)
    dev = torch.zeros(want.size, dtype=torch.uint8, device="cuda")
    host = np.zeros(want.size, np.uint8)
    _grid(lib, gpu_ctx, m, 110, noalloc=True)            # warm: the kernels' first launches
    _grid(lib, gpu_ctx, m, 110, noalloc=True, out=dev)
    gpu_ctx.synchronize()
    torch.cuda.synchronize()
    before = gpu_ctx.memory()
    assert before["device_total"] > 0
    dims = (C.c_uint32 * 3)()
    for k in range(6):
        if k % 2:
            dev.zero_()
            torch.cuda.synchronize()
            assert lib.j3dg_voxelize_noalloc(gpu_ctx.h, m.h, 110, dims, dev.data_ptr(), dev.numel()) == 0
            gpu_ctx.synchronize()
            assert np.array_equal(dev.cpu().numpy(), want)
        else:
            host[:] = 0
            assert lib.j3dg_voxelize_noalloc(gpu_ctx.h, m.h, 110, dims, host.ctypes.data, host.size) == 0
            assert np.array_equal(host, want)
        assert gpu_ctx.memory() == before, (k, before, gpu_ctx.memory())
