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
