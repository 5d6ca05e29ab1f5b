"""Batched frames (many canvases, scenes, resolutions and modes in one
persistent launch, optionally a captured CUDA graph) render exactly what
the same frames render one by one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(ctx):
    from j3d_gb300 import Canvas, Matcap, Mesh, Scene, camera_for_vfov, settings, workloads as W
    meshes = [Mesh(ctx, *W.icosphere(3, W.SEED_BASE + 30)), Mesh(ctx, *W.torus(90, 45, seed=W.SEED_BASE + 31)),
              Mesh(ctx, *W.icosphere(5, W.SEED_BASE + 32))]
    poses = W.cameras(6, W.SEED_BASE + 33, 2.5, 4.0)
    res = [(256, 256), (160, 90), (512, 256), (96, 128), (333, 211), (64, 64)]
    modes = [dict(shadow=True, edges=False), dict(shadow=False, edges=False), dict(shadow=True, edges=True),
             dict(shadow=True, edges=False, wireframe=True), dict(shadow=True, edges=False),
             dict(shadow=True, one_bit=True)]
    mcs = [Matcap.make(ctx, 0), Matcap.make(ctx, 2)]
    frames = []
    for i in range(6):
        sc = Scene()
        sc.add_object(meshes[i % 3], db_id=i + 1)
        if i == 4:  # two objects
            sc.add_object(meshes[(i + 1) % 3], W.translation(0.8, 0.1, -0.3), db_id=99)
        sc.prepare_scene()
        sc.unzoom()
        sc.set_pose(poses[i])
        cv = Canvas(ctx, *res[i])
        cv.set_camera(camera_for_vfov(60.0 if i % 2 == 0 else 45.0))
        cv.set_background_color(0xff000000 + i, 0xff404040)
        cv.update_settings(settings(**modes[i]))
        frames.append((cv, sc, mcs[i % 2]))
    return meshes, frames, poses


def _one_by_one(frames):
    out = []
    for cv, sc, mc in frames:
        cv.render_frame(sc, mc)
        out.append((cv.get_pixels(), cv.get_image()))
    return out


def test_render_batch_equals_single_frames(gpu_ctx):
    from j3d_gb300 import render_batch
    meshes, frames, _ = _setup(gpu_ctx)
    ref = _one_by_one(frames)
    for cv, _, _ in frames:  # scribble, so stale results cannot pass
        cv.render_scene(None)
    render_batch(gpu_ctx, frames)
    for i, (cv, sc, mc) in enumerate(frames):
        assert np.array_equal(cv.get_pixels().view(np.uint8), ref[i][0].view(np.uint8)), f"frame {i}"
        assert np.array_equal(cv.get_image(), ref[i][1]), f"frame {i}"
        assert (ref[i][0]["object_id"] != 0xFFFFFFFF).any()


def test_graph_batch_replays_and_follows_scene_updates(gpu_ctx):
    from j3d_gb300 import Batch
    meshes, frames, poses = _setup(gpu_ctx)
    b = Batch(gpu_ctx, frames)
    for rep in range(2):
        for cv, _, _ in frames:
            cv.render_scene(None)
        b.launch()
        gpu_ctx.synchronize()
        ref = _one_by_one(frames)
        for cv, _, _ in frames:
            cv.render_scene(None)
        b.launch()
        for i, (cv, sc, mc) in enumerate(frames):
            assert np.array_equal(cv.get_pixels().view(np.uint8), ref[i][0].view(np.uint8)), f"rep {rep} frame {i}"
            assert np.array_equal(cv.get_image(), ref[i][1])
        # move every camera, then replay again
        for i, (cv, sc, mc) in enumerate(frames):
            sc.set_pose(poses[(i + 1 + rep) % len(poses)])
            b.set_scene(i, sc)
    b.close()


def test_config2_batch_matches_oracle(gpu_ctx, oracle_mod):
    """Batched frames at the batched configuration's shape: 64 meshes with
    triangle counts log-uniform in 10k-2M (icospheres and tori), 16 seeded
    cameras each, resolutions drawn from {256^2, 512^2, 768x512, 1024^2}:
    all 1024 frames in one graph-captured persistent launch. One seeded frame
    of every mesh (64 whole frames) is compared with the oracle's frame:
    triangle ids, marks and db ids bit-exact, floats within 1e-5 relative,
    RGBA exact (plain shading)."""
    from helpers import compare_gbuffers, oracle_scene

    from j3d_gb300 import Batch, Canvas, Matcap, Mesh, Scene, camera_for_vfov, settings, workloads as W
    O = oracle_mod
    wl = W.config2()
    assert len(wl.meshes) == 64 and wl.poses.shape[:2] == (64, 16)
    tris = [len(T) for _, T in wl.meshes]
    assert 10_000 * 0.85 <= min(tris) and max(tris) <= 2_000_000 * 1.15
    meshes = [Mesh(gpu_ctx, V, T) for V, T in wl.meshes]
    mc = Matcap.make(gpu_ctx, 0)
    frames, k = [], 0
    for i, m in enumerate(meshes):
        for c in range(16):
            sc = Scene()
            sc.add_object(m, db_id=i + 1)
            sc.prepare_scene()
            sc.unzoom()
            sc.set_pose(wl.poses[i][c])
            cv = Canvas(gpu_ctx, *wl.resolutions[k])
            cv.set_camera(camera_for_vfov(60.0))
            cv.set_background_color()
            cv.update_settings(settings(shadow=True, edges=False))
            frames.append((cv, sc, mc))
            k += 1
    g = Batch(gpu_ctx, frames)
    g.launch()
    gpu_ctx.synchronize()
    rng = np.random.default_rng(2024)
    mco, cav = O.make_matcap(0)
    hit_frames = 0
    for i, (V, T) in enumerate(wl.meshes):
        c = int(rng.integers(0, 16))
        cv, sc, _ = frames[16 * i + c]
        w, h = wl.resolutions[16 * i + c]
        m, views, _ = oracle_scene(O, V, T, wl.poses[i][c:c + 1], w, h)
        op = O.fresh_pixels(w, h)
        oi = np.zeros((h, w), np.uint32)
        O.render_frame(op, oi, O.fill_background(w, h), [(m, np.eye(4, dtype=np.float32).reshape(16), i + 1)],
                       views[0], O.settings(shadow=True, edges=False), mco, cav)
        gp = cv.get_pixels()
        assert compare_gbuffers(gp, op, f"mesh {i} ({len(T)} tris) camera {c} {w}x{h}") == 0
        assert np.array_equal(cv.get_image(), oi), f"mesh {i} camera {c}: RGBA"
        hit_frames += int((gp["object_id"] != 0xFFFFFFFF).any())
    assert hit_frames > 48
    g.close()
    for cv, _, _ in frames:
        cv.close()


def test_build_many_equals_single_builds(gpu_ctx):
    """j3dg_mesh_build_many: meshes built concurrently on their own streams
    give the same closest hits as meshes built one by one (the tree of each
    may differ in node order, never in its hits), with per-mesh leaf sizes;
    a bad mesh fails the call and leaves no mesh behind."""
    from j3d_gb300 import J3dgError, Mesh, SceneObject, build_meshes, find_closest
    from j3d_gb300 import workloads as W
    from test_gpu_parity import _random_rays
    srcs = [W.icosphere(lvl, W.SEED_BASE + 120 + lvl) for lvl in (2, 3, 4, 5)]
    srcs += [W.torus(nu, nv, seed=W.SEED_BASE + 130 + nu) for nu, nv in ((40, 20), (120, 60), (300, 150), (90, 45))]
    leaves = [1, 2, 4, 2, 8, 2, 1, 4]
    many = build_meshes(gpu_ctx, srcs, leaves, max_concurrent=4)
    rays = _random_rays(8000, 21)
    for i, ((V, T), m) in enumerate(zip(srcs, many)):
        assert m.info().n_triangles == len(T)
        one = Mesh(gpu_ctx, V, T, leaves[i])
        a = find_closest(gpu_ctx, [SceneObject(m)], rays)
        b = find_closest(gpu_ctx, [SceneObject(one)], rays)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"mesh {i}"
        assert a["found"].any()
        one.close()
    bad = [srcs[0], (srcs[1][0], np.zeros((0, 3), np.uint32))]
    with pytest.raises(J3dgError):
        build_meshes(gpu_ctx, bad)


@pytest.mark.parametrize("width,mixed", [(2, False), (4, False), (8, False), (4, True)])
def test_batch_rebuilds_its_meshes_in_the_graph(gpu_ctx, oracle_mod, width, mixed):
    """Batch(rebuild=True): every launch first rebuilds the BVHs of its
    scenes' meshes (built rebuildable) inside the graph, on forked capture
    streams with device-driven level loops, then renders. After two launches
    every mesh's node array equals the one its standalone build made, byte
    for byte (the rebuild is the same build), and one frame of every mesh
    equals the oracle's. Meshes from 2 triangles (a single leaf) to 80k, on
    both sides of the SAH / PLOC split, 12 of them so that lanes rebuild
    several meshes in turn; half built one by one, half by build_meshes (the
    concurrent builds); BVH widths 2, 4 and 8, and at width 4 the two
    builders mixed (LBVH meshes among default ones, so that lanes keep
    scratch for both)."""
    from helpers import compare_gbuffers, oracle_scene

    from j3d_gb300 import (Batch, Canvas, J3dgError, Matcap, Mesh, Scene, build_meshes, camera_for_vfov, settings,
                           workloads as W)
    O = oracle_mod
    quad_V = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32)
    quad_T = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    srcs = [(quad_V, quad_T)]
    srcs += [W.icosphere(k, W.SEED_BASE + 90 + k) for k in (1, 2, 3, 4, 5, 6)]
    srcs += [W.torus(nu, nv, seed=W.SEED_BASE + 100 + nu) for nu, nv in ((8, 4), (40, 20), (120, 60), (200, 100),
                                                                           (282, 141))]
    meshes = [Mesh(gpu_ctx, V, T, width=width, build="lbvh" if mixed and k % 2 else "ploc", rebuildable=True)
              for k, (V, T) in enumerate(srcs[:6])]
    meshes += build_meshes(gpu_ctx, srcs[6:], width=width, build="lbvh" if mixed else "ploc", rebuildable=True)
    nodes0 = [m.nodes() for m in meshes]
    mc = Matcap.make(gpu_ctx, 0)
    poses = W.cameras(len(meshes), W.SEED_BASE + 110, 2.5, 3.5)
    frames, sizes = [], []
    for i, m in enumerate(meshes):
        sc = Scene()
        sc.add_object(m, db_id=i + 1)
        sc.prepare_scene()
        sc.unzoom()
        sc.set_pose(poses[i])
        w, h = (320, 240) if i % 2 else (256, 256)
        cv = Canvas(gpu_ctx, w, h)
        cv.set_camera(camera_for_vfov(60.0))
        cv.set_background_color()
        cv.update_settings(settings(shadow=True, edges=False))
        frames.append((cv, sc, mc))
        sizes.append((w, h))
    g = Batch(gpu_ctx, frames, rebuild=True)
    for _ in range(2):
        g.launch()
    gpu_ctx.synchronize()
    for i, m in enumerate(meshes):
        assert np.array_equal(m.nodes().view(np.uint32), nodes0[i].view(np.uint32)), f"mesh {i}: rebuilt nodes"
    mco, cav = O.make_matcap(0)
    for i, (V, T) in enumerate(srcs):
        cv, sc, _ = frames[i]
        w, h = sizes[i]
        om, views, _ = oracle_scene(O, V, T, poses[i:i + 1], w, h)
        op = O.fresh_pixels(w, h)
        oi = np.zeros((h, w), np.uint32)
        O.render_frame(op, oi, O.fill_background(w, h), [(om, np.eye(4, dtype=np.float32).reshape(16), i + 1)],
                       views[0], O.settings(shadow=True, edges=False), mco, cav)
        assert compare_gbuffers(cv.get_pixels(), op, f"rebuild batch, mesh {i} ({len(T)} tris)") == 0
        assert np.array_equal(cv.get_image(), oi), f"rebuild batch, mesh {i}: RGBA"
    g.close()
    # a mesh built without the flag cannot be rebuilt
    plain = Mesh(gpu_ctx, *srcs[3], width=width)
    sc = Scene()
    sc.add_object(plain)
    sc.prepare_scene()
    sc.unzoom()
    sc.set_pose(poses[3])
    with pytest.raises(J3dgError):
        Batch(gpu_ctx, [(frames[0][0], sc, mc)], rebuild=True)
    for cv, _, _ in frames:
        cv.close()
