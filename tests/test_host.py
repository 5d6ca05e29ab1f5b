"""CPU tests of the product library's host side: it loads, exports every
declared symbol, and its host math equals the oracle's bit for bit."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
I16 = np.eye(4, dtype=np.float32).reshape(16)


def declared_symbols():
    text = (ROOT / "include" / "j3dg.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(j3dg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(product_lib):
    syms = declared_symbols()
    assert len(syms) > 40
    missing = [s for s in syms if not hasattr(product_lib, s)]
    assert not missing, missing
    from j3d_gb300 import _ffi
    assert set(_ffi.SIGNATURES) >= set(syms), sorted(set(syms) - set(_ffi.SIGNATURES))
    assert product_lib.j3dg_abi_version() == 1


def test_library_links_no_oracle(product_lib):
    import subprocess
    from j3d_gb300 import LIB_PATH
    out = subprocess.run(["nm", "-D", str(LIB_PATH)], capture_output=True, text=True).stdout
    assert "orc_" not in out


def test_no_gpu_fails_loudly(product_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert product_lib.j3dg_ctx_create(0, C.byref(h)) == 4  # J3DG_ERR_NO_DEVICE, no CPU fallback


def test_camera_math_matches_oracle(product_lib, oracle_mod):
    from j3d_gb300 import scene as S
    O = oracle_mod
    for (w, h) in ((800, 600), (1024, 768), (1920, 1080), (600, 800), (1, 1)):
        for vfov in (None, 60.0, 31.0):
            cam = S.make_default_camera() if vfov is None else S.camera_for_vfov(vfov)
            ocam = O.camera_with_focal(cam.focal_length)
            for fit in (0, 1):
                cam.fit_film = fit
                ocam.fit_film = fit
                P = S.make_projection_matrix(cam, w, h)
                assert np.array_equal(P.view(np.uint32), O.make_projection_matrix(ocam, w, h).view(np.uint32))
                assert np.array_equal(S.invert_projection_matrix(P).view(np.uint32),
                                      O.invert_projection_matrix(P).view(np.uint32))
    # default camera: 35 mm, 1.024 x 0.768 in film, near 0.1, far FLT_MAX, Overscan (camera.cpp:5-16)
    c = S.make_default_camera()
    assert (c.focal_length, c.near_clipping_plane, c.fit_film) == (35.0, np.float32(0.1), 1)
    # 60 degree vertical field of view through the film gate
    P = S.make_projection_matrix(S.camera_for_vfov(60.0), 1024, 768)
    assert abs(np.degrees(2 * np.arctan(-1.0 / P[5])) - 60.0) < 1e-4


def test_scene_math_matches_oracle(product_lib, oracle_mod):
    from j3d_gb300 import scene as S, workloads as W
    O = oracle_mod
    rng = np.random.default_rng(3)
    for _ in range(20):
        cs = W.cameras(1, int(rng.integers(1 << 40)), 1, 5)[0]
        assert np.array_equal(S.invert_orthonormal(cs).view(np.uint32), O.invert_orthonormal(cs).view(np.uint32))
    mn = np.array([-1.25, -0.5, 0.1], np.float32)
    mx = np.array([2.0, 0.75, 3.3], np.float32)
    lib = product_lib
    cs = np.zeros(16, np.float32); inv = np.zeros(16, np.float32); piv = np.zeros(3, np.float32)
    from j3d_gb300._ffi import fptr
    lib.j3dg_unzoom(fptr(mn), fptr(mx), np.float32(3.2), fptr(cs), fptr(inv), fptr(piv))
    ocs, oinv, opiv = O.unzoom(mn, mx, 3.2)
    assert np.array_equal(cs, ocs) and np.array_equal(inv, oinv) and np.array_equal(piv, opiv)


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_matcaps_match_oracle(product_lib, oracle_mod, kind):
    from j3d_gb300 import scene as S
    a, ca = S.make_matcap(kind)
    b, cb = oracle_mod.make_matcap(kind)
    assert ca == cb and np.array_equal(a, b)
    # red wax default cavity colour (matcap.cpp:167)
    if kind == 0:
        assert ca == 0xFF7D7DFF


def test_background_matches_oracle(product_lib, oracle_mod):
    from j3d_gb300 import scene as S
    for (w, h, t, b) in ((37, 29, 0xff000000, 0xff404040), (64, 480, 0xff102030, 0xffa0b0c0)):
        assert np.array_equal(S.fill_background(w, h, t, b), oracle_mod.fill_background(w, h, t, b))


def test_synthetic_meshes_deterministic(product_lib):
    from j3d_gb300 import workloads as W
    V, T = W.icosphere(6)
    assert V.shape == (40962, 3) and T.shape == (81920, 3)
    V2, T2 = W.icosphere(6)
    assert np.array_equal(V, V2) and np.array_equal(T, T2)
    assert T.max() == 40961
    r = np.linalg.norm(V.astype(np.float64), axis=1)
    assert 0.55 < r.min() and r.max() < 1.45
    Vt, Tt = W.torus(53, 26)
    assert Vt.shape == (53 * 26, 3) and Tt.shape == (2 * 53 * 26, 3) and Tt.max() == 53 * 26 - 1
    # every edge of the closed torus grid is shared by exactly two triangles
    e = np.sort(np.concatenate([Tt[:, [0, 1]], Tt[:, [1, 2]], Tt[:, [2, 0]]]), axis=1)
    _, cnt = np.unique(e, axis=0, return_counts=True)
    assert (cnt == 2).all()
    poses = W.cameras(32, 123, 2.5, 4.0)
    R = poses.reshape(32, 4, 4)[:, :3, :3].astype(np.float64)
    assert np.allclose(np.einsum("nij,nkj->nik", R, R), np.eye(3), atol=1e-5)
    dist = np.linalg.norm(poses.reshape(32, 4, 4)[:, 3, :3], axis=1)
    assert (dist >= 2.5 - 1e-5).all() and (dist <= 4.0 + 1e-5).all()


def test_normals_and_bbox_oracle_restatement(oracle_mod, product_lib):
    from j3d_gb300 import workloads as W
    V, T = W.icosphere(2)
    N = oracle_mod.compute_triangle_normals(V, T)
    e1 = V[T[:, 1]].astype(np.float64) - V[T[:, 0]]
    e2 = V[T[:, 2]].astype(np.float64) - V[T[:, 0]]
    n = np.cross(e1, e2)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    assert np.allclose(N, n, atol=1e-6)
    mn, mx = oracle_mod.compute_bb(V)
    assert np.array_equal(mn, V.min(axis=0)) and np.array_equal(mx, V.max(axis=0))


def test_oracle_generators_equal_product_generators(product_lib):
    """The oracle's numpy restatement of the seeded workloads (used by the CPU
    baseline, which must not load the product library) gives the product's
    bytes: icosphere subdivision order and displacement, torus grid, cameras,
    and the 60-degree focal length."""
    import oracle.workloads as OW
    from j3d_gb300 import scene as S
    from j3d_gb300 import workloads as W
    for lvl in range(0, 6):
        a, b = W.icosphere(lvl, W.SEED_BASE + 40 + lvl), OW.icosphere(lvl, W.SEED_BASE + 40 + lvl)
        assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32)) and np.array_equal(a[1], b[1]), lvl
    for nu, nv, seed in ((3, 3, 1), (10, 7, 2), (301, 149, W.SEED_BASE + 1)):
        a, b = W.torus(nu, nv, seed=seed), OW.torus(nu, nv, seed=seed)
        assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32)) and np.array_equal(a[1], b[1]), (nu, nv)
    for n, seed, r0, r1 in ((32, W.SEED_BASE + 1 + (1 << 32), 2.5, 4.0), (300, 7, 2.0, 5.0)):
        assert np.array_equal(W.cameras(n, seed, r0, r1).view(np.uint32), OW.cameras(n, seed, r0, r1).view(np.uint32))
    for vfov in (60.0, 45.0, 31.0, 90.0, 1.0):
        assert S.lib().j3dg_focal_for_vfov(vfov, 0.768) == OW.focal_for_vfov(vfov, 0.768)
    c0 = W.config0()
    V, T, poses, w, h = OW.config0()
    assert np.array_equal(c0.vertices, V) and np.array_equal(c0.triangles, T) and np.array_equal(c0.poses, poses)
    assert (c0.width, c0.height) == (w, h)
