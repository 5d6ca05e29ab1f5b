"""Point-cloud splat (canvas::render_pointclouds_on_image, canvas.cpp:952-1030):
the oracle against a hand-computed case, then the device pass (one 64-bit
atomicMax per point, a resolve per cloud) against the oracle's sequential
restatement, bit-exact on the G-buffer and the image."""
import numpy as np
import pytest

from j3d_gb300._ffi import PIXEL_DTYPE


def _blank(w, h):
    pix = np.zeros((h, w), PIXEL_DTYPE)
    pix["object_id"] = 0xFFFFFFFF
    pix["depth"] = np.finfo(np.float32).max
    return pix


def test_oracle_known_answer(oracle_mod):
    O = oracle_mod
    w = h = 4
    P = np.zeros(16, np.float32)
    P[0], P[5], P[10], P[11], P[14] = 1.0, -1.0, -1.0, -1.0, -0.2
    I = np.eye(4, dtype=np.float32).reshape(16)
    pix = _blank(w, h)
    pix[3, 3]["db_id"] = 7           # a mesh pixel at depth 1 hides farther points there
    pix[3, 3]["depth"] = 1.0
    im = np.full((h, w), 0x11223344, np.uint32)
    V = np.array([[0, 0, -2], [-1, 1, -2], [0, 0, -4], [0, 0, -2], [0, 0, 1], [0, 0, -0.05],
                  [1.5, -1.5, -2], [0.375, -0.375, -0.5]], np.float32)
    col = np.arange(1, 9, dtype=np.uint32) * 0x01010101
    O.render_pointclouds(pix, im, P, I, 0.1, [(V, col, I, 3)])
    # (0,0,-2): s = (0, 0) -> pixel (2, 2); the farther and the equal-depth later points lose
    assert (pix[2, 2]["object_id"], pix[2, 2]["depth"], pix[2, 2]["db_id"], im[2, 2]) == (0, 2.0, 3, col[0])
    # (-1,1,-2): s = (-0.5, -0.5) -> (1, 1)
    assert (pix[1, 1]["object_id"], im[1, 1]) == (1, col[1])
    # behind the camera / before the near plane: not drawn; the mesh pixel keeps
    # its record against the point at depth 2 and loses to the one at depth 0.5
    assert pix[3, 3]["object_id"] == 7 and pix[3, 3]["db_id"] == 3 and pix[3, 3]["depth"] == np.float32(0.5)
    assert int((pix["db_id"] == 3).sum()) == 3 and int((im == 0x11223344).sum()) == 13


def _scene_with_clouds(ctx, with_mesh=True, n_dense=0):
    from j3d_gb300 import Mesh, PointCloud, Scene, workloads as W
    rng = np.random.default_rng(11)
    sc = Scene()
    keep = {}
    if with_mesh:
        V, T = W.icosphere(4, W.SEED_BASE + 80)
        keep["mesh"] = Mesh(ctx, V, T)
        sc.add_object(keep["mesh"], None, 1)
    d = rng.normal(size=(60000, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    A = (d * np.float32(1.06)).astype(np.float32)
    colA = rng.integers(0, 2 ** 32, len(A), dtype=np.uint64).astype(np.uint32)
    B = (d[:20000] * np.float32(0.93)).astype(np.float32)
    B = np.concatenate([B, B[:5000], (d[:3000] * np.float32(1.3)).astype(np.float32)])  # duplicates tie
    csB = np.eye(4, dtype=np.float32)
    csB[3, :3] = (0.05, -0.02, 0.0)                                   # translated cloud
    keep["A"] = PointCloud(ctx, A, colA)
    keep["B"] = PointCloud(ctx, B)
    sc.add_pointcloud(keep["A"], None, 2)
    sc.add_pointcloud(keep["B"], csB.reshape(16), 3)
    clouds = [(A, colA, np.eye(4, dtype=np.float32).reshape(16), 2), (B, None, csB.reshape(16), 3)]
    if n_dense:
        Dn = (rng.normal(size=(n_dense, 3)) * 0.02 + (0.0, 0.0, 1.2)).astype(np.float32)
        colD = rng.integers(0, 2 ** 32, n_dense, dtype=np.uint64).astype(np.uint32)
        keep["D"] = PointCloud(ctx, Dn, colD)
        sc.add_pointcloud(keep["D"], None, 4)
        clouds.append((Dn, colD, np.eye(4, dtype=np.float32).reshape(16), 4))
    sc.prepare_scene()
    sc.unzoom()
    return sc, clouds, keep


def _run(ctx, oracle_mod, sc, clouds, w=400, h=300, one_bit=False):
    from j3d_gb300 import Canvas, Matcap, settings
    mc = Matcap.make(ctx, 0)
    cv = Canvas(ctx, w, h)
    cv.update_settings(settings(shadow=True, edges=False, one_bit=one_bit))
    cv.render_frame(sc, mc)
    pix0, im0 = cv.get_pixels().copy(), cv.get_image().copy()
    cv.render_pointclouds(sc)
    pix1, im1 = cv.get_pixels(), cv.get_image()
    P, _ = cv.get_projection()
    ref_pix = pix0.reshape(h, w).copy()
    ref_im = im0.reshape(h, w).copy()
    oracle_mod.render_pointclouds(ref_pix, ref_im, P, sc.coordinate_system_inv, 0.1, clouds, one_bit=one_bit)
    assert np.array_equal(pix1.reshape(h, w).view(np.uint8), ref_pix.view(np.uint8))
    assert np.array_equal(im1.reshape(h, w), ref_im)
    return pix0.reshape(h, w), ref_pix


@pytest.mark.gpu
def test_splat_over_mesh_matches_oracle(gpu_ctx, oracle_mod):
    sc, clouds, keep = _scene_with_clouds(gpu_ctx)
    before, after = _run(gpu_ctx, oracle_mod, sc, clouds)
    changed = before["db_id"] != after["db_id"]
    assert changed.sum() > 1000                       # cloud A in front of the sphere shows
    assert (after["db_id"] == 3).sum() > 0            # cloud B only where it sticks out
    assert ((after["db_id"] == 1) & (before["db_id"] == 1)).sum() > 0  # mesh still visible


@pytest.mark.gpu
def test_splat_without_mesh_and_one_bit(gpu_ctx, oracle_mod):
    sc, clouds, keep = _scene_with_clouds(gpu_ctx, with_mesh=False)
    _run(gpu_ctx, oracle_mod, sc, clouds, 320, 240, one_bit=True)
    # prepare_scene over clouds only (scene.cpp:50-89) equals the oracle's
    bbs, css = [], []
    for V, _, cs, _ in clouds:
        M = np.asarray(cs, np.float32).reshape(16)
        bbs.append((V.min(0).astype(np.float32), V.max(0).astype(np.float32)))
        css.append(M)
    mn, mx, diag = oracle_mod.prepare_scene(bbs, css)
    assert np.array_equal(sc.min_bb, mn) and np.array_equal(sc.max_bb, mx) and sc.diagonal == np.float32(diag)


@pytest.mark.gpu
def test_dense_cloud_many_points_per_pixel(gpu_ctx, oracle_mod):
    sc, clouds, keep = _scene_with_clouds(gpu_ctx, n_dense=1_000_000)
    _run(gpu_ctx, oracle_mod, sc, clouds, 640, 480)


@pytest.mark.gpu
def test_pointcloud_from_file_and_bounds(gpu_ctx, tmp_path):
    from j3d_gb300 import Geometry, PointCloud
    from oracle import formats as F
    rng = np.random.default_rng(12)
    V = rng.normal(size=(5000, 3)).astype(np.float32)
    col = rng.integers(0, 256, (5000, 3))
    g = Geometry.read_memory(gpu_ctx, F.write_pts(V, intensity=np.zeros(5000), colors=col), "pts")
    pc = PointCloud(gpu_ctx, geometry=g)
    mn, mx = pc.bounds()
    assert np.array_equal(mn, V.min(0)) and np.array_equal(mx, V.max(0))
    pc2 = PointCloud(gpu_ctx, V)
    assert all(np.array_equal(a, b) for a, b in zip(pc2.bounds(), (mn, mx)))
