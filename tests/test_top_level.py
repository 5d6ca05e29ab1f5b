"""Scenes of many objects through the per-frame top level (the two-level
structure of qbvh_two_level_with_transformations, canvas.cpp:762, 786, 854):
240 instances of four meshes under random rigid transforms, rendered on the
GPU through the top-level BVH and compared with the oracle, which walks the
objects one after the other. Bar: hit mask, triangle id, db id and marks
bit-exact, t / u / v / barycentrics within 1e-5 relative, RGBA exact in the
plain mode and within 1 LSB in the edges mode; ray batches bit-exact."""
import numpy as np
import pytest

from helpers import NO_ID, compare_gbuffers, compare_rgba

pytestmark = pytest.mark.gpu


def _rigid(rng, spread):
    """Column-major float32 4x4: a random rotation (unit quaternion) and a translation."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    M = np.eye(4)
    M[:3, :3] = R
    M[:3, 3] = rng.uniform(-spread, spread, size=3)
    return M.T.reshape(16).astype(np.float32)  # column-major storage


def _scene(n_inst=240, seed=5):
    from j3d_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    meshes = [W.icosphere(3, W.SEED_BASE + 70), W.torus(48, 24, seed=W.SEED_BASE + 71),
              W.icosphere(2, W.SEED_BASE + 72), W.torus(20, 10, R=0.6, r=0.2, seed=W.SEED_BASE + 73)]
    insts = []
    for k in range(n_inst):
        insts.append((k % len(meshes), _rigid(rng, 6.0), 100 + k))
    return meshes, insts


def _gpu_and_oracle(ctx, O, meshes, insts):
    from j3d_gb300 import Mesh, Scene
    gm = [Mesh(ctx, V, T) for V, T in meshes]
    om = [O.Mesh(V, T) for V, T in meshes]
    sc = Scene()
    for mi, cs, db in insts:
        sc.add_object(gm[mi], cs, db)
    sc.prepare_scene()
    sc.unzoom()
    objs = [(om[mi], cs, db) for mi, cs, db in insts]
    return gm, om, sc, objs


def _oracle_view(O, sc_min, sc_max, diag, css, pose, w, h):
    from oracle.workloads import focal_for_vfov
    mn, mx, d = O.prepare_scene([(a, b) for a, b in zip(sc_min, sc_max)], css)
    _, _, piv = O.unzoom(mn, mx, d)
    cam = O.camera_with_focal(focal_for_vfov(60.0, 0.768))
    Pi = O.invert_projection_matrix(O.make_projection_matrix(cam, w, h))
    return O.view(pose, O.invert_orthonormal(pose), piv, d, Pi, cam.near_clipping_plane), (mn, d)


@pytest.mark.parametrize("top", [True, False])
def test_many_objects_frames_match_oracle(gpu_ctx, oracle_mod, top):
    """Frames of 240 objects equal the oracle's, walked through the top level
    and (the same context switched off) object after object."""
    from j3d_gb300 import Canvas, Matcap, camera_for_vfov, settings
    from j3d_gb300 import workloads as W
    O = oracle_mod
    meshes, insts = _scene()
    gm, om, sc, objs = _gpu_and_oracle(gpu_ctx, O, meshes, insts)
    gpu_ctx.set_top_level(top)
    try:
        w, h = 320, 240
        poses = [W.translation(0.3, -0.2, 24.0), W.cameras(1, 91, 14.0, 16.0)[0], W.translation(-2.0, 1.0, 9.0)]
        for k, pose in enumerate(poses):
            sc.set_pose(pose)
            v, (mn, d) = _oracle_view(O, [om[mi].min_bb for mi, _, _ in insts], [om[mi].max_bb for mi, _, _ in insts],
                                      None, [cs for _, cs, _ in insts], pose, w, h)
            assert np.array_equal(sc.min_bb, mn) and sc.diagonal == d
            for kw in (dict(shadow=True, edges=False), dict(shadow=True, edges=True)):
                cv = Canvas(gpu_ctx, w, h)
                cv.set_camera(camera_for_vfov(60.0))
                cv.set_background_color()
                cv.update_settings(settings(**kw))
                mc = Matcap.make(gpu_ctx, 0)
                cv.render_frame(sc, mc)
                gp, gi = cv.get_pixels(), cv.get_image()
                cv.close()
                mco, cav = O.make_matcap(0)
                op = O.fresh_pixels(w, h)
                oi = np.zeros((h, w), np.uint32)
                O.render_frame(op, oi, O.fill_background(w, h), objs, v, O.settings(**kw), mco, cav)
                where = f"240 objects, pose {k}, {kw}, top={top}"
                assert compare_gbuffers(gp, op, where) == 0
                compare_rgba(gi, oi, 1 if kw["edges"] else 0, where)
                hit = gp["object_id"] != NO_ID
                assert hit.mean() > 0.05, where
                assert len(np.unique(gp["db_id"][hit])) > 20, where
                assert ((gp["mark"] & 1) != 0).sum() > 100, where
    finally:
        gpu_ctx.set_top_level(True)


def test_many_objects_ray_batches_match_oracle(gpu_ctx, oracle_mod):
    """find_closest / find_any over 240 objects: bit-exact against the oracle."""
    from j3d_gb300 import SceneObject, find_closest
    O = oracle_mod
    meshes, insts = _scene(seed=6)
    gm, om, sc, objs = _gpu_and_oracle(gpu_ctx, O, meshes, insts)
    rng = np.random.default_rng(12)
    n = 30000
    o = rng.uniform(-9, 9, size=(n, 3)).astype(np.float32)
    d = (rng.uniform(-1, 1, size=(n, 3)) - o * 0.1).astype(np.float32)
    rays = np.zeros(n, O.RAY_DTYPE)
    rays["orig"][:, :3] = o
    rays["orig"][:, 3] = 1
    rays["dir"][:, :3] = d
    rays["t_near"] = rng.uniform(0, 0.5, n).astype(np.float32)
    rays["t_far"] = np.where(rng.uniform(size=n) < 0.2, rng.uniform(0.5, 8, n), 3.4e38).astype(np.float32)
    objs_g = [SceneObject(gm[mi], cs, db) for mi, cs, db in insts]
    for any_hit in (False, True):
        hg = find_closest(gpu_ctx, objs_g, rays, any_hit=any_hit)
        ho, _ = O.find_closest(objs, rays, any_hit=any_hit)
        assert np.array_equal(hg["found"], ho["found"])
        if not any_hit:
            assert np.array_equal(hg.view(np.uint8), ho.view(np.uint8))
        assert hg["found"].mean() > 0.05
        assert len(np.unique(hg["two_level_index"][hg["found"] == 1])) > 50


def test_many_objects_in_a_batch_match_oracle(gpu_ctx, oracle_mod):
    """A graph-captured batch mixing a 240-object scene with one-object
    scenes: every frame equals the oracle's, before and after the pose of
    the 240-object frame is swapped between replays."""
    from j3d_gb300 import Batch, Canvas, Matcap, Scene, camera_for_vfov, settings
    from j3d_gb300 import workloads as W
    O = oracle_mod
    meshes, insts = _scene(seed=7)
    gm, om, sc, objs = _gpu_and_oracle(gpu_ctx, O, meshes, insts)
    single = Scene()
    single.add_object(gm[1], None, 5)
    single.prepare_scene()
    single.unzoom()
    single.set_pose(W.translation(0.0, 0.0, 3.0))
    sc.set_pose(W.translation(0.5, 0.0, 22.0))
    mc = Matcap.make(gpu_ctx, 0)
    frames = []
    for k, s in enumerate((sc, single, sc, single)):
        w, h = (256, 192) if k % 2 else (320, 240)
        cv = Canvas(gpu_ctx, w, h)
        cv.set_camera(camera_for_vfov(60.0))
        cv.set_background_color()
        cv.update_settings(settings(shadow=True, edges=False))
        frames.append((cv, s, w, h))
    b = Batch(gpu_ctx, [(cv, s, mc) for cv, s, _, _ in frames])
    mco, cav = O.make_matcap(0)
    # the oracle's canvases live across launches like the GPU's: a miss keeps
    # the mark and barycentrics of the frame before (canvas.cpp:859-866)
    opix = [O.fresh_pixels(w, h) for _, _, w, h in frames]

    def check(poses):
        b.launch()
        gpu_ctx.synchronize()
        for k, (cv, s, w, h) in enumerate(frames):
            if s is sc:
                v, _ = _oracle_view(O, [om[mi].min_bb for mi, _, _ in insts], [om[mi].max_bb for mi, _, _ in insts],
                                    None, [cs for _, cs, _ in insts], poses[k], w, h)
                ob = objs
            else:
                ob = [(om[1], np.eye(4, dtype=np.float32).reshape(16), 5)]
                v, _ = _oracle_view(O, [om[1].min_bb], [om[1].max_bb], None, [ob[0][1]], poses[k], w, h)
            op = opix[k]
            oi = np.zeros((h, w), np.uint32)
            O.render_frame(op, oi, O.fill_background(w, h), ob, v, O.settings(shadow=True, edges=False), mco, cav)
            assert compare_gbuffers(cv.get_pixels(), op, f"batch frame {k}") == 0
            assert np.array_equal(cv.get_image(), oi)

    check([sc.coordinate_system, single.coordinate_system, sc.coordinate_system, single.coordinate_system])
    sc2 = Scene()
    for mi, cs, db in insts:
        sc2.add_object(gm[mi], cs, db)
    sc2.prepare_scene()
    sc2.unzoom()
    sc2.set_pose(W.translation(-1.0, 0.5, 18.0))
    b.set_scene(2, sc2)
    check([sc.coordinate_system, single.coordinate_system, sc2.coordinate_system, single.coordinate_system])
