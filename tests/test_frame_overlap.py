"""Overlapped frames of one canvas (j3dg_ctx_set_frame_overlap): a traced
frame starts while the canvas's previous frame finishes its last pixels, and
per-pixel frame stamps keep each pixel's writes in frame order. Bar: every
canvas state equals, byte for byte, the state that frames run strictly one
after the other leave (overlap off; those frames are compared with the
oracle by the other tests), including the fields a miss keeps from the
frame before (canvas.cpp:859-866); a persistent canvas over a sequence of
overlapped frames equals the oracle's; a wait that runs out raises the
status word and leaves the context usable."""
import numpy as np
import pytest

from helpers import NO_ID, compare_gbuffers, oracle_scene

pytestmark = pytest.mark.gpu


def _canvas(ctx, w, h, edges=False):
    from j3d_gb300 import Canvas, camera_for_vfov, settings
    cv = Canvas(ctx, w, h)
    cv.set_camera(camera_for_vfov(60.0))
    cv.set_background_color()
    cv.update_settings(settings(shadow=True, edges=edges))
    return cv


def _same(a, b, where):
    (pa, ia), (pb, ib) = a, b
    bad = np.flatnonzero((pa.view(np.uint8).reshape(-1, 32) != pb.view(np.uint8).reshape(-1, 32)).any(axis=1))
    assert bad.size == 0, f"{where}: {bad.size} G-buffer records differ, first at {bad[:8]}"
    assert np.array_equal(ia, ib), f"{where}: RGBA differs at {np.flatnonzero(ia.reshape(-1) != ib.reshape(-1))[:8]}"


def _pairs(ctx, sc, poses, w, h, mc, edges=False, where=""):
    """For every k: frames k-1 and k back to back into a canvas with overlap
    on, and the same two into a canvas with overlap off; both canvases carry
    the whole sequence, and their states after every pair are equal."""
    cv_on, cv_off = _canvas(ctx, w, h, edges), _canvas(ctx, w, h, edges)
    try:
        for k in range(1, len(poses)):
            states = []
            for cv, on in ((cv_on, True), (cv_off, False)):
                ctx.set_frame_overlap(on)
                for p in (poses[k - 1], poses[k]):
                    sc.set_pose(p)
                    cv.render_frame(sc, mc)
                states.append((cv.get_pixels(), cv.get_image()))
            _same(states[0], states[1], f"{where} frames {k - 1}, {k}")
    finally:
        ctx.set_frame_overlap(True)
        cv_on.close()
        cv_off.close()


def test_full_size_torus_overlapped_frames_equal_serial(gpu_ctx):
    """The 28.09M-triangle torus at 1920x1080, the benchmark's 32 cameras:
    every consecutive pair of frames rendered back to back into one canvas
    (the second starts during the first one's tail) leaves the canvas that
    the same frames run one after the other leave."""
    from j3d_gb300 import Matcap, workloads as W
    from helpers import gpu_scene
    wl = W.config1()
    mesh, sc = gpu_scene(gpu_ctx, wl.vertices, wl.triangles, wl.poses[0])
    mc = Matcap.make(gpu_ctx, 0)
    _pairs(gpu_ctx, sc, wl.poses, wl.width, wl.height, mc, where="torus28M")
    mesh.close()


@pytest.mark.parametrize("edges", [False, True])
def test_many_objects_overlapped_frames_equal_serial(gpu_ctx, edges):
    """240 objects through the top level (the TOP kernels), small frames (the
    latency build), plain and edges shading (a shading kernel after every
    frame): pairs as above, then a sequence of 12 frames back to back."""
    from j3d_gb300 import Matcap, Mesh, Scene, workloads as W
    from test_top_level import _scene
    meshes, insts = _scene(seed=11)
    gm = [Mesh(gpu_ctx, V, T) for V, T in meshes]
    sc = Scene()
    for mi, cs, db in insts:
        sc.add_object(gm[mi], cs, db)
    sc.prepare_scene()
    sc.unzoom()
    poses = [W.translation(0.3, -0.2, 24.0)] + list(W.cameras(11, W.SEED_BASE + 120, 10.0, 18.0))
    mc = Matcap.make(gpu_ctx, 0)
    _pairs(gpu_ctx, sc, poses[:5], 640, 480, mc, edges, where=f"240 objects, edges={edges}")
    states = []
    for on in (True, False):
        gpu_ctx.set_frame_overlap(on)
        cv = _canvas(gpu_ctx, 640, 480, edges)
        for p in poses:
            sc.set_pose(p)
            cv.render_frame(sc, mc)
        states.append((cv.get_pixels(), cv.get_image()))
        cv.close()
    gpu_ctx.set_frame_overlap(True)
    _same(states[0], states[1], f"240 objects, 12 frames, edges={edges}")


def test_alternating_canvases_overlap(gpu_ctx):
    """Frames alternating between two canvases (the end-to-end pattern: one
    canvas renders while the other's frame finishes) equal serial frames."""
    from j3d_gb300 import Matcap, workloads as W
    from helpers import gpu_scene
    V, T = W.torus(600, 300, seed=W.SEED_BASE + 121)
    poses = W.cameras(10, W.SEED_BASE + 122, 2.5, 4.0)
    mesh, sc = gpu_scene(gpu_ctx, V, T, poses[0])
    mc = Matcap.make(gpu_ctx, 0)
    out = []
    for on in (True, False):
        gpu_ctx.set_frame_overlap(on)
        cvs = [_canvas(gpu_ctx, 1280, 720), _canvas(gpu_ctx, 1280, 720)]
        for k, p in enumerate(poses):
            sc.set_pose(p)
            cvs[k & 1].render_frame(sc, mc)
        out.append([(c.get_pixels(), c.get_image()) for c in cvs])
        for c in cvs:
            c.close()
    gpu_ctx.set_frame_overlap(True)
    for j in range(2):
        _same(out[0][j], out[1][j], f"alternating canvases, canvas {j}")


def test_overlapped_sequence_matches_oracle(gpu_ctx, oracle_mod):
    """Four frames back to back into one canvas with overlap (cameras that
    leave parts of the frame empty, so misses keep fields of the frame
    before) against the oracle rendering the same four frames into one
    persistent pixel buffer."""
    from j3d_gb300 import Matcap, workloads as W
    from helpers import gpu_scene
    O = oracle_mod
    V, T = W.torus(160, 80, seed=W.SEED_BASE + 123)
    poses = [W.translation(0.0, 0.0, 3.0), W.translation(0.9, 0.3, 2.6), W.translation(-0.7, -0.5, 3.4),
             W.cameras(1, W.SEED_BASE + 124, 2.0, 3.0)[0]]
    w, h = 480, 360
    mesh, sc = gpu_scene(gpu_ctx, V, T, poses[0])
    mc = Matcap.make(gpu_ctx, 0)
    cv = _canvas(gpu_ctx, w, h)
    for p in poses:
        sc.set_pose(p)
        cv.render_frame(sc, mc)
    gp, gi = cv.get_pixels(), cv.get_image()
    om, views, _ = oracle_scene(O, V, T, poses, w, h)
    mco, cav = O.make_matcap(0)
    op = O.fresh_pixels(w, h)
    oi = np.zeros((h, w), np.uint32)
    for v in views:
        O.render_frame(op, oi, O.fill_background(w, h), [(om, np.eye(4, dtype=np.float32).reshape(16), 1)], v,
                       O.settings(shadow=True, edges=False), mco, cav)
    assert compare_gbuffers(gp, op, "overlapped sequence") == 0
    assert np.array_equal(gi, oi)
    miss = gp["object_id"] == NO_ID
    assert miss.sum() > 1000 and (~miss).sum() > 1000
    assert (gp["mark"][miss] != 0).sum() > 0  # misses that keep an earlier frame's mark
    cv.close()


def test_frame_wait_runs_out_and_context_recovers(gpu_ctx):
    """A frame told to wait for a frame number that no frame wrote: its waits
    run out (half a second), it raises J3DG_DEV_WAIT_TIMEOUT, the next
    synchronising call returns the device status error, and the context and
    canvas keep working (the next frames equal serial frames)."""
    from j3d_gb300 import J3dgError, Matcap, workloads as W
    from helpers import gpu_scene
    V, T = W.icosphere(5, W.SEED_BASE + 125)
    poses = W.cameras(3, W.SEED_BASE + 126, 2.5, 3.5)
    mesh, sc = gpu_scene(gpu_ctx, V, T, poses[0])
    mc = Matcap.make(gpu_ctx, 0)
    cv = _canvas(gpu_ctx, 256, 192)
    cv.render_frame(sc, mc)
    cv.get_pixels()
    cv.expect_frame(0x7EADBEEF)
    sc.set_pose(poses[1])
    cv.render_frame(sc, mc)
    with pytest.raises(J3dgError) as e:
        cv.get_pixels()
    assert e.value.status == 5 and "16 frame wait timeout" in str(e.value)
    assert gpu_ctx.device_status() == 0
    ref = _canvas(gpu_ctx, 256, 192)
    for c, on in ((cv, True), (ref, False)):
        gpu_ctx.set_frame_overlap(on)
        for p in poses:
            sc.set_pose(p)
            c.render_frame(sc, mc)
    gpu_ctx.set_frame_overlap(True)
    _same((cv.get_pixels(), cv.get_image()), (ref.get_pixels(), ref.get_image()), "after the timeout")
    cv.close()
    ref.close()


def test_downloads_of_overlapped_frames(gpu_ctx):
    """The end-to-end pattern: frames alternate between two canvases and each
    frame's G-buffer and image are downloaded asynchronously (copy stream)
    right after it is queued, while the next frame, on the other canvas,
    overlaps it. Every downloaded frame equals the frame run serially."""
    torch = pytest.importorskip("torch")
    from j3d_gb300 import Matcap, workloads as W
    from helpers import gpu_scene
    V, T = W.torus(600, 300, seed=W.SEED_BASE + 127)
    poses = W.cameras(8, W.SEED_BASE + 128, 2.5, 4.0)
    mesh, sc = gpu_scene(gpu_ctx, V, T, poses[0])
    mc = Matcap.make(gpu_ctx, 0)
    w, h = 1280, 720
    runs = []
    for on in (True, False):
        gpu_ctx.set_frame_overlap(on)
        cvs = [_canvas(gpu_ctx, w, h), _canvas(gpu_ctx, w, h)]
        hp = [torch.empty(h * w * 32, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
        hi = [torch.empty(h * w * 4, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
        frames = []
        for k, p in enumerate(poses):
            c = cvs[k & 1]
            c.download_wait()
            if k >= 2:
                frames.append((hp[k & 1].numpy().copy(), hi[k & 1].numpy().copy()))
            sc.set_pose(p)
            c.render_frame(sc, mc)
            c.download_async(hp[k & 1].numpy(), hi[k & 1].numpy())
        for k in (len(poses), len(poses) + 1):
            cvs[k & 1].download_wait()
            frames.append((hp[k & 1].numpy().copy(), hi[k & 1].numpy().copy()))
        runs.append(frames)
        for c in cvs:
            c.close()
    gpu_ctx.set_frame_overlap(True)
    assert len(runs[0]) == len(runs[1]) == len(poses)
    for k, (a, b) in enumerate(zip(*runs)):
        assert np.array_equal(a[0], b[0]), f"downloaded frame {k}: G-buffer differs"
        assert np.array_equal(a[1], b[1]), f"downloaded frame {k}: image differs"


def test_mixed_sequences_overlap_equal_serial(gpu_ctx):
    """A seeded random sequence of 60 calls over three canvases of different
    sizes and two scenes: plain frames (which may overlap), edges-mode frames,
    rectangles (update_canvas), rasterised frames, render_scene +
    canvas_to_image, asynchronous downloads and synchronous reads in
    between. Run with overlap on and off: every read and every final canvas
    is identical."""
    torch = pytest.importorskip("torch")
    from j3d_gb300 import (PRIMARY_AUTO, PRIMARY_RASTER, Matcap, Mesh, Scene, settings, workloads as W)
    rng = np.random.default_rng(2024)
    V1, T1 = W.torus(400, 200, seed=W.SEED_BASE + 130)
    V2, T2 = W.icosphere(5, W.SEED_BASE + 131)
    m1, m2 = Mesh(gpu_ctx, V1, T1), Mesh(gpu_ctx, V2, T2)
    scenes = []
    for m in (m1, m2):
        sc = Scene()
        sc.add_object(m, db_id=len(scenes) + 1)
        sc.prepare_scene()
        sc.unzoom()
        scenes.append(sc)
    poses = W.cameras(16, W.SEED_BASE + 132, 2.2, 3.8)
    sizes = [(640, 480), (800, 600), (320, 240)]
    ops = []
    for _ in range(60):
        ops.append((int(rng.integers(0, 100)), int(rng.integers(0, 3)), int(rng.integers(0, 2)),
                    int(rng.integers(0, 16)), rng.uniform(size=4)))
    mc = Matcap.make(gpu_ctx, 0)
    runs = []
    for on in (True, False):
        gpu_ctx.set_frame_overlap(on)
        cvs = [_canvas(gpu_ctx, w, h) for w, h in sizes]
        bufs = [(torch.zeros(h * w * 32, dtype=torch.uint8, pin_memory=True),
                 torch.zeros(h * w * 4, dtype=torch.uint8, pin_memory=True)) for w, h in sizes]
        reads = []
        for kind, ci, si, pi, u in ops:
            cv, sc = cvs[ci], scenes[si]
            w, h = sizes[ci]
            sc.set_pose(poses[pi])
            if kind < 55:  # plain frame
                cv.render_frame(sc, mc)
            elif kind < 63:  # edges mode (a shading kernel after the frame)
                cv.update_settings(settings(shadow=True, edges=True))
                cv.render_frame(sc, mc)
                cv.update_settings(settings(shadow=True, edges=False))
            elif kind < 71:  # a rectangle
                x0, x1 = sorted((int(u[0] * w), int(u[1] * w)))
                y0, y1 = sorted((int(u[2] * h), int(u[3] * h)))
                cv.update_canvas(x0, y0, x1, y1, sc)
            elif kind < 77:  # rasterised primary hits
                gpu_ctx.set_primary_mode(PRIMARY_RASTER)
                cv.render_frame(sc, mc)
                gpu_ctx.set_primary_mode(PRIMARY_AUTO)
            elif kind < 82:  # render_scene + canvas_to_image
                cv.render_scene(sc)
                cv.canvas_to_image(mc)
            elif kind < 92:  # asynchronous download, read at the next wait
                cv.download_wait()
                cv.download_async(bufs[ci][0].numpy(), bufs[ci][1].numpy())
            else:  # synchronous read
                reads.append((cv.get_pixels(), cv.get_image()))
        for ci, cv in enumerate(cvs):
            cv.download_wait()
            reads.append((bufs[ci][0].numpy().copy(), bufs[ci][1].numpy().copy()))
            reads.append((cv.get_pixels(), cv.get_image()))
            cv.close()
        runs.append(reads)
    gpu_ctx.set_frame_overlap(True)
    gpu_ctx.set_primary_mode(PRIMARY_AUTO)
    assert gpu_ctx.device_status() == 0
    assert len(runs[0]) == len(runs[1])
    for k, (a, b) in enumerate(zip(*runs)):
        assert np.array_equal(np.asarray(a[0]).view(np.uint8), np.asarray(b[0]).view(np.uint8)), f"read {k}: G-buffer"
        assert np.array_equal(np.asarray(a[1]).view(np.uint8), np.asarray(b[1]).view(np.uint8)), f"read {k}: image"
