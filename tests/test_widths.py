"""BVH widths 2 and 8 (the autotuner's other choices) against the oracle:
the builder's cost-optimal collapse at each width, the width-specialised
traversal kernels and the top level at that width must give the oracle's
closest hits and frames bit for bit, as width 4 does."""
import numpy as np
import pytest

from helpers import NO_ID, compare_gbuffers, compare_rgba, gpu_scene, oracle_scene

pytestmark = pytest.mark.gpu
I16 = np.eye(4, dtype=np.float32).reshape(16)
WIDTHS = [2, 8]


def _frame(ctx, sc, w, h, kw):
    from j3d_gb300 import Canvas, Matcap, camera_for_vfov, settings
    cv = Canvas(ctx, w, h)
    cv.set_camera(camera_for_vfov(60.0))
    cv.set_background_color()
    cv.update_settings(settings(**kw))
    cv.render_frame(sc, Matcap.make(ctx, 0))
    out = cv.get_pixels(), cv.get_image()
    cv.close()
    return out


@pytest.mark.parametrize("width", WIDTHS)
def test_width_frames_match_oracle(gpu_ctx, oracle_mod, width):
    """Icosphere level 6 at 1024x768 and a torus, primary + shadow, plain
    and edges shading, leaf sizes 1, 2 and 4."""
    from j3d_gb300 import Mesh, Scene
    from j3d_gb300 import workloads as W
    O = oracle_mod
    wl = W.config0()
    cases = [(wl.vertices, wl.triangles, wl.poses[0], 1024, 768)]
    Vt, Tt = W.torus(400, 200, seed=W.SEED_BASE + 80)
    cases.append((Vt, Tt, W.cameras(1, W.SEED_BASE + 81, 2.5, 3.5)[0], 640, 360))
    for V, T, pose, w, h in cases:
        m, views, _ = oracle_scene(O, V, T, pose[None], w, h)
        for leaf in (1, 2, 4):
            mesh = Mesh(gpu_ctx, V, T, leaf, "ploc", width)
            info = mesh.info()
            assert info.width == width and info.n_nodes > 0
            sc = Scene()
            sc.add_object(mesh)
            sc.prepare_scene()
            sc.unzoom()
            sc.set_pose(pose)
            for kw in (dict(shadow=True, edges=False), dict(shadow=True, edges=True)):
                gp, gi = _frame(gpu_ctx, sc, w, h, kw)
                op = O.fresh_pixels(w, h)
                oi = np.zeros((h, w), np.uint32)
                mc, cav = O.make_matcap(0)
                O.render_frame(op, oi, O.fill_background(w, h), [(m, I16, 1)], views[0], O.settings(**kw), mc, cav)
                where = f"width {width} leaf {leaf} {len(T)} tris {kw}"
                assert compare_gbuffers(gp, op, where) == 0
                compare_rgba(gi, oi, 1 if kw["edges"] else 0, where)
                assert (gp["object_id"] != NO_ID).mean() > 0.05
            mesh.close()


@pytest.mark.parametrize("width", WIDTHS)
@pytest.mark.parametrize("case", ["stacked", "n65", "n1000", "flat"])
def test_width_builder_edge_cases_match_brute_force(gpu_ctx, oracle_mod, width, case):
    from j3d_gb300 import Mesh, SceneObject, find_closest
    from test_gpu_parity import _random_rays
    O = oracle_mod
    rng = np.random.default_rng(sum(case.encode()) + width)
    if case == "stacked":
        base = rng.uniform(-1, 1, size=(3, 3)).astype(np.float32)
        V = np.concatenate([np.tile(base, (600, 1)), rng.uniform(-1, 1, size=(300, 3)).astype(np.float32)])
        T = np.arange(len(V), dtype=np.uint32).reshape(-1, 3)
    elif case == "flat":
        V = rng.uniform(-1, 1, size=(3000, 3)).astype(np.float32)
        V[:, 2] = 0.25
        T = rng.integers(0, len(V), size=(2000, 3)).astype(np.uint32)
    else:
        nt = int(case[1:])
        c = rng.uniform(-1, 1, size=(nt, 1, 3)).astype(np.float32)
        V = (c + rng.uniform(-0.15, 0.15, size=(nt, 3, 3)).astype(np.float32)).reshape(-1, 3)
        T = np.arange(3 * nt, dtype=np.uint32).reshape(-1, 3)
    mesh = Mesh(gpu_ctx, V, T, 2, "ploc", width)
    m = O.Mesh(V, T)
    rays = _random_rays(20000, 7)
    for any_hit in (False, True):
        hg = find_closest(gpu_ctx, [SceneObject(mesh, I16, 1)], rays, any_hit=any_hit)
        ho, _ = O.find_closest([(m, I16, 1)], rays, brute=True, any_hit=any_hit)
        assert np.array_equal(hg["found"], ho["found"])
        if not any_hit:
            assert np.array_equal(hg.view(np.uint8), ho.view(np.uint8))
    assert hg["found"].any()


@pytest.mark.parametrize("width", WIDTHS)
def test_width_many_objects_and_batch_match_oracle(gpu_ctx, oracle_mod, width):
    """64 objects through a top level of the same width, a frame and a
    graph-captured batch, against the oracle; widths may not mix, and the
    queries that need 4-wide trees refuse other widths."""
    from j3d_gb300 import Batch, Canvas, J3dgError, Matcap, Mesh, Scene, camera_for_vfov, settings
    from j3d_gb300 import workloads as W
    from j3d_gb300.learned import Learned
    from test_top_level import _oracle_view, _rigid
    O = oracle_mod
    rng = np.random.default_rng(30 + width)
    meshes = [W.icosphere(3, W.SEED_BASE + 82), W.torus(60, 30, seed=W.SEED_BASE + 83)]
    gm = [Mesh(gpu_ctx, V, T, 2, "ploc", width) for V, T in meshes]
    om = [O.Mesh(V, T) for V, T in meshes]
    insts = [(k % 2, _rigid(rng, 4.0), 10 + k) for k in range(64)]
    sc = Scene()
    for mi, cs, db in insts:
        sc.add_object(gm[mi], cs, db)
    sc.prepare_scene()
    sc.unzoom()
    pose = W.translation(0.2, 0.1, 16.0)
    sc.set_pose(pose)
    objs = [(om[mi], cs, db) for mi, cs, db in insts]
    w, h = 256, 192
    v, _ = _oracle_view(O, [om[mi].min_bb for mi, _, _ in insts], [om[mi].max_bb for mi, _, _ in insts], None,
                        [cs for _, cs, _ in insts], pose, w, h)
    mco, cav = O.make_matcap(0)
    op = O.fresh_pixels(w, h)
    oi = np.zeros((h, w), np.uint32)
    O.render_frame(op, oi, O.fill_background(w, h), objs, v, O.settings(shadow=True, edges=False), mco, cav)
    gp, gi = _frame(gpu_ctx, sc, w, h, dict(shadow=True, edges=False))
    assert compare_gbuffers(gp, op, f"64 objects width {width}") == 0
    assert np.array_equal(gi, oi)
    assert len(np.unique(gp["db_id"][gp["object_id"] != NO_ID])) > 10
    mc = Matcap.make(gpu_ctx, 0)
    frames = []
    for k in range(3):
        cv = Canvas(gpu_ctx, w, h)
        cv.set_camera(camera_for_vfov(60.0))
        cv.set_background_color()
        cv.update_settings(settings(shadow=True, edges=False))
        frames.append((cv, sc, mc))
    b = Batch(gpu_ctx, frames)
    b.launch()
    gpu_ctx.synchronize()
    for cv, _, _ in frames:
        assert compare_gbuffers(cv.get_pixels(), op, f"batch width {width}") == 0
        assert np.array_equal(cv.get_image(), oi)
    b.close()
    four = Mesh(gpu_ctx, *meshes[0])
    mixed = Scene()
    mixed.add_object(gm[0])
    mixed.add_object(four, W.translation(3.0, 0.0, 0.0), 2)
    mixed.prepare_scene()
    mixed.unzoom()
    with pytest.raises(J3dgError):
        _frame(gpu_ctx, mixed, 64, 48, dict(shadow=True, edges=False))
    with pytest.raises(J3dgError):
        Learned(gpu_ctx, gm[0])
    import ctypes as C
    from j3d_gb300 import _ffi
    dims = (C.c_uint32 * 3)()
    assert _ffi.lib().j3dg_voxelize(gpu_ctx.h, gm[0].h, 32, dims, None, 0) == 6  # J3DG_ERR_UNSUPPORTED
