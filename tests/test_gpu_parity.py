"""GPU parity: the CUDA path through the C-ABI against the CPU oracle.

Bar: hit mask, triangle id, object id and shadow mark bit-exact; t, u, v
and barycentrics within 1e-5 relative (bit-exact expected); RGBA8 within
1 LSB (plain shading bit-exact; acosf in the edges mode may differ by 1).
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import FLT_MAX, NO_ID, compare_gbuffers, compare_rgba, gpu_scene, oracle_scene

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
I16 = np.eye(4, dtype=np.float32).reshape(16)


def gpu_frame(ctx, sc, w, h, st, vfov=60.0, kind=0, background=True, expect=None):
    """Renders one frame; expect: the primary-hit method the frame must have
    used ("trace" / "raster"), or None."""
    from j3d_gb300 import PRIMARY_RASTER, PRIMARY_TRACE, Canvas, Matcap, camera_for_vfov
    cv = Canvas(ctx, w, h)
    cv.set_camera(camera_for_vfov(vfov))
    if background:
        cv.set_background_color()
    cv.update_settings(st)
    mc = Matcap.make(ctx, kind)
    cv.render_frame(sc, mc)
    if expect is not None:
        assert cv.last_primary() == {"trace": PRIMARY_TRACE, "raster": PRIMARY_RASTER}[expect]
    return cv.get_pixels(), cv.get_image(), cv, mc


def oracle_frame(O, m, v, w, h, st, kind=0, objs=None):
    mc, cav = O.make_matcap(kind)
    pix = O.fresh_pixels(w, h)
    im = np.zeros((h, w), np.uint32)
    O.render_frame(pix, im, O.fill_background(w, h), objs or [(m, I16, 1)], v, st, mc, cav)
    return pix, im


def gst(**kw):
    from j3d_gb300 import settings
    return settings(**kw)


def test_icosphere_config0_parity_and_golden(gpu_ctx, oracle_mod, primary):
    from j3d_gb300 import workloads as W
    O = oracle_mod
    wl = W.config0()
    mesh, sc = gpu_scene(gpu_ctx, wl.vertices, wl.triangles, wl.poses[0])
    m, views, (mn, mx, diag, piv, P, Pi) = oracle_scene(O, wl.vertices, wl.triangles, wl.poses, wl.width, wl.height)
    # the scene set-up agrees bit for bit (bbox from the GPU reduction)
    assert np.array_equal(sc.min_bb, mn) and np.array_equal(sc.max_bb, mx) and sc.diagonal == diag
    assert np.array_equal(np.asarray(sc.pivot), piv)
    # normals computed on the GPU equal the oracle's
    assert np.array_equal(mesh.triangle_normals().view(np.uint32), m.normals().view(np.uint32))
    gold = json.loads((GOLDEN / "golden.json").read_text())["icosphere_L6_1024x768"]
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    for mode, kw in (("plain", dict(shadow=True, edges=False)), ("edges", dict(shadow=True, edges=True))):
        gp, gi, cv, mc = gpu_frame(gpu_ctx, sc, wl.width, wl.height, gst(**kw), expect=primary)
        assert np.array_equal(cv.get_projection()[0], P)
        op, oi = oracle_frame(O, m, views[0], wl.width, wl.height, O.settings(**kw))
        compare_gbuffers(gp, op, f"config0 {mode}")
        assert sha(gp) == gold["frames"][0][mode]["gbuffer_sha"]
        if mode == "plain":
            assert np.array_equal(gi, oi)
            assert sha(gi) == gold["frames"][0][mode]["rgba_sha"]
        else:
            compare_rgba(gi, oi, 1, "config0 edges")


def test_icosphere_config0_golden_with_lbvh_tree(gpu_ctx):
    """The LBVH tree differs from the default (PLOC) tree but the frame is bit
    for bit the committed golden frame (results do not depend on the tree)."""
    from j3d_gb300 import workloads as W
    wl = W.config0()
    mesh, sc = gpu_scene(gpu_ctx, wl.vertices, wl.triangles, wl.poses[0], build="lbvh")
    gold = json.loads((GOLDEN / "golden.json").read_text())["icosphere_L6_1024x768"]
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    gp, gi, cv, mc = gpu_frame(gpu_ctx, sc, wl.width, wl.height, gst(shadow=True, edges=False))
    assert sha(gp) == gold["frames"][0]["plain"]["gbuffer_sha"]
    assert sha(gi) == gold["frames"][0]["plain"]["rgba_sha"]
    ploc = gpu_scene(gpu_ctx, wl.vertices, wl.triangles, wl.poses[0])[0]
    assert mesh.info().n_nodes != ploc.info().n_nodes or mesh.info().max_depth != ploc.info().max_depth


@pytest.mark.parametrize("leaf,build", [(1, "lbvh"), (2, "lbvh"), (4, "lbvh"), (8, "lbvh"), (1, "ploc"),
                                        (2, "ploc"), (8, "ploc")])
def test_torus_cameras_parity(gpu_ctx, oracle_mod, leaf, build, primary):
    from j3d_gb300 import workloads as W
    O = oracle_mod
    V, T = W.torus(300, 150, seed=W.SEED_BASE + 1)
    poses = W.cameras(4, W.SEED_BASE + 11, 2.5, 4.0)
    m, views, _ = oracle_scene(O, V, T, poses, 480, 270)
    mesh = None
    for i, p in enumerate(poses):
        mesh, sc = gpu_scene(gpu_ctx, V, T, p, leaf=leaf, build=build) if mesh is None else (mesh, sc)
        sc.set_pose(p)
        gp, gi, _, _ = gpu_frame(gpu_ctx, sc, 480, 270, gst(shadow=True, edges=False), expect=primary)
        op, oi = oracle_frame(O, m, views[i], 480, 270, O.settings(shadow=True, edges=False))
        assert compare_gbuffers(gp, op, f"torus cam {i}") == 0
        assert np.array_equal(gi, oi)
        assert (gp["object_id"] != NO_ID).any()


@pytest.mark.parametrize("case", ["inside_box", "looking_away", "off_centre"])
def test_camera_placements_match_oracle(gpu_ctx, oracle_mod, case, primary):
    """Frames with the camera inside the mesh's box (in the torus hole),
    looking away from the mesh (every ray misses), or with the mesh across
    the image edge equal the oracle's."""
    from j3d_gb300 import workloads as W
    O = oracle_mod
    V, T = W.torus(200, 100, seed=W.SEED_BASE + 3)
    if case == "inside_box":
        poses = W.cameras(3, W.SEED_BASE + 21, 0.05, 0.6)
    elif case == "looking_away":
        poses = W.cameras(3, W.SEED_BASE + 22, 2.5, 4.0)
        poses[:, 0:3] *= -1.0  # rotate 180 degrees about the camera's y axis
        poses[:, 8:11] *= -1.0
    else:
        poses = W.cameras(3, W.SEED_BASE + 23, 2.5, 4.0, target=(1.6, 0.4, -0.9))
    m, views, _ = oracle_scene(O, V, T, poses, 320, 200)
    mesh, sc = gpu_scene(gpu_ctx, V, T, poses[0])
    hits = 0
    for i, p in enumerate(poses):
        sc.set_pose(p)
        # a camera inside the mesh's box, or facing away, has triangles behind it: traced
        gp, gi, _, _ = gpu_frame(gpu_ctx, sc, 320, 200, gst(shadow=True, edges=False),
                                 expect="trace" if case in ("inside_box", "looking_away") else primary)
        op, oi = oracle_frame(O, m, views[i], 320, 200, O.settings(shadow=True, edges=False))
        assert compare_gbuffers(gp, op, f"{case} cam {i}") == 0
        assert np.array_equal(gi, oi)
        hits += int((gp["object_id"] != NO_ID).sum())
    if case == "looking_away":
        assert hits == 0
    else:
        assert hits > 0


@pytest.mark.parametrize("mode", ["wireframe", "one_bit", "noshadow_edges", "shading_off"])
def test_shading_modes(gpu_ctx, oracle_mod, mode, primary):
    from j3d_gb300 import workloads as W
    O = oracle_mod
    V, T = W.icosphere(4)
    pose = W.translation(0.1, -0.05, 2.6)
    kw = {"wireframe": dict(shadow=True, edges=False, wireframe=True),
          "one_bit": dict(shadow=True, one_bit=True),
          "noshadow_edges": dict(shadow=False, edges=True),
          "shading_off": dict(shadow=True, edges=False, shading=False)}[mode]
    mesh, sc = gpu_scene(gpu_ctx, V, T, pose)
    m, views, _ = oracle_scene(O, V, T, [pose], 320, 200)
    for kind in (0, 3):
        gp, gi, _, _ = gpu_frame(gpu_ctx, sc, 320, 200, gst(**kw), kind=kind, expect=primary)
        op, oi = oracle_frame(O, m, views[0], 320, 200, O.settings(**kw), kind=kind)
        compare_gbuffers(gp, op, mode)
        compare_rgba(gi, oi, 1 if "edges" in mode else 0, mode)


@pytest.mark.parametrize("case", ["large", "overflow", "duplicates"])
def test_raster_large_triangles_overflow_and_ties(gpu_ctx, oracle_mod, case):
    """Rasterised primary hits against the oracle where the raster takes its
    other routes: triangles with many candidate pixels (the pixel-parallel
    list), more such triangles than the list holds on a 16x16 canvas (the
    frame is traced on the device instead), and every triangle twice (equal
    t everywhere: the smaller triangle id must win, as in the traversal)."""
    from j3d_gb300 import PRIMARY_AUTO, PRIMARY_RASTER, workloads as W
    O = oracle_mod
    if case == "large":
        V, T = W.icosphere(1)
        w, h = 320, 200
    elif case == "overflow":
        rng = np.random.default_rng(7)
        k = np.arange(400, dtype=np.float32)
        base = np.array([[-2.0, -2.0, 0.0], [2.0, -2.0, 0.0], [0.0, 2.0, 0.0]], np.float32)
        V = (base[None] + rng.uniform(-0.2, 0.2, size=(400, 3, 3)).astype(np.float32))
        V[:, :, 2] = -0.002 * k[:, None] + rng.uniform(-5e-4, 5e-4, size=(400, 3)).astype(np.float32)
        V = V.reshape(-1, 3).astype(np.float32)
        T = np.arange(1200, dtype=np.uint32).reshape(400, 3)
        w, h = 16, 16
    else:
        V, T = W.icosphere(3, W.SEED_BASE + 9)
        T = np.concatenate([T, T]).astype(np.uint32)
        w, h = 320, 200
    pose = W.translation(0.1, -0.05, 2.6)
    mesh, sc = gpu_scene(gpu_ctx, V, T, pose)
    m, views, _ = oracle_scene(O, V, T, [pose], w, h)
    gpu_ctx.set_primary_mode(PRIMARY_RASTER)
    try:
        for kw in (dict(shadow=True, edges=False), dict(shadow=True, edges=True)):
            gp, gi, _, _ = gpu_frame(gpu_ctx, sc, w, h, gst(**kw), expect="raster")
            op, oi = oracle_frame(O, m, views[0], w, h, O.settings(**kw))
            assert compare_gbuffers(gp, op, case) == 0
            compare_rgba(gi, oi, 1 if kw["edges"] else 0, case)
            hit = gp["object_id"] != NO_ID
            assert hit.mean() > 0.2
            if case == "duplicates":
                assert (gp["object_id"][hit] < T.shape[0] // 2).all()
    finally:
        gpu_ctx.set_primary_mode(PRIMARY_AUTO)


def test_ray_batches_match_oracle(gpu_ctx, oracle_mod):
    from j3d_gb300 import Mesh, SceneObject, find_closest, workloads as W
    O = oracle_mod
    V, T = W.icosphere(5, W.SEED_BASE + 3)
    mesh = Mesh(gpu_ctx, V, T)
    m = O.Mesh(V, T)
    rng = np.random.default_rng(11)
    n = 20000
    o = rng.uniform(-3, 3, size=(n, 3)).astype(np.float32)
    d = (rng.uniform(-1, 1, size=(n, 3)) - o * 0.3).astype(np.float32)
    rays = np.zeros(n, O.RAY_DTYPE)
    rays["orig"][:, :3] = o
    rays["orig"][:, 3] = 1
    rays["dir"][:, :3] = d
    rays["t_near"] = rng.uniform(0, 0.5, n).astype(np.float32)
    rays["t_far"] = np.where(rng.uniform(size=n) < 0.2, rng.uniform(0.5, 3, n), FLT_MAX).astype(np.float32)
    cs2 = W.translation(0.9, 0.0, 0.2)
    objs_g = [SceneObject(mesh, I16, 1), SceneObject(mesh, cs2, 2)]
    objs_o = [(m, I16, 1), (m, cs2, 2)]
    for any_hit in (False, True):
        hg = find_closest(gpu_ctx, objs_g, rays, any_hit=any_hit)
        ho, _ = O.find_closest(objs_o, rays, any_hit=any_hit)
        assert np.array_equal(hg["found"], ho["found"])
        if not any_hit:
            assert np.array_equal(hg.view(np.uint8), ho.view(np.uint8))
        assert hg["found"].mean() > 0.05


def _random_rays(n, seed, spread=3.0):
    import oracle.oracle as O
    rng = np.random.default_rng(seed)
    o = rng.uniform(-spread, spread, size=(n, 3)).astype(np.float32)
    d = (rng.uniform(-1, 1, size=(n, 3)) - o * 0.3).astype(np.float32)
    rays = np.zeros(n, O.RAY_DTYPE)
    rays["orig"][:, :3] = o
    rays["orig"][:, 3] = 1
    rays["dir"][:, :3] = d
    rays["t_near"] = np.float32(1e-4)
    rays["t_far"] = FLT_MAX
    return rays


@pytest.mark.parametrize("case", ["stacked", "n64", "n65", "n129", "n1000", "flat", "lbvh_stacked"])
def test_builder_edge_cases_match_brute_force(gpu_ctx, oracle_mod, case):
    """Meshes that steer the builder into its edge cases give the oracle's
    brute-force closest hits: every triangle's centroid in one bin (the SAH
    split falls back to a split by position), sizes around the 64-triangle
    range where PLOC takes over, a flat mesh (zero extent on one axis)."""
    from j3d_gb300 import Mesh, SceneObject, find_closest
    O = oracle_mod
    rng = np.random.default_rng(sum(case.encode()))
    if case in ("stacked", "lbvh_stacked"):
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
    mesh = Mesh(gpu_ctx, V, T, 2, "lbvh" if case.startswith("lbvh") else "ploc")
    m = O.Mesh(V, T)
    rays = _random_rays(20000, 7)
    hg = find_closest(gpu_ctx, [SceneObject(mesh, I16, 1)], rays)
    ho, _ = O.find_closest([(m, I16, 1)], rays, brute=True)
    assert np.array_equal(hg.view(np.uint8), ho.view(np.uint8))
    assert hg["found"].any()


def test_update_canvas_rect_empty_and_null_scene(gpu_ctx, oracle_mod, primary):
    from j3d_gb300 import PRIMARY_RASTER, PRIMARY_TRACE, Canvas, Matcap, Scene, camera_for_vfov, workloads as W
    O = oracle_mod
    V, T = W.icosphere(3)
    pose = W.translation(0, 0, 3)
    mesh, sc = gpu_scene(gpu_ctx, V, T, pose)
    m, views, _ = oracle_scene(O, V, T, [pose], 96, 64)
    cv = Canvas(gpu_ctx, 96, 64)
    cv.set_camera(camera_for_vfov(60.0))
    cv.update_settings(gst(shadow=True, edges=False))
    cv.update_canvas(-5, 7, 50, 1000, sc)  # clamped like canvas.cpp:681-698
    assert cv.last_primary() == (PRIMARY_TRACE if primary == "trace" else PRIMARY_RASTER)
    op = O.fresh_pixels(96, 64)
    O.update_canvas(op, [(m, I16, 1)], views[0], O.settings(shadow=True, edges=False), rect=(0, 7, 50, 63))
    assert compare_gbuffers(cv.get_pixels(), op, "rect") == 0
    empty = Scene()
    empty.set_pose(pose)
    cv.update_canvas(0, 0, 95, 63, empty)
    px = cv.get_pixels()
    assert (px["object_id"] == NO_ID).all() and (px["depth"] == FLT_MAX).all()
    cv.set_background_color(0xff112233, 0xff445566)
    cv.render_scene(None)
    assert np.array_equal(cv.get_image(), O.fill_background(96, 64, 0xff112233, 0xff445566))
    # canvas_to_image from a caller G-buffer (host) equals the oracle's shading
    mc = Matcap.make(gpu_ctx, 1)
    omc, ocav = O.make_matcap(1)
    full = O.fresh_pixels(96, 64)
    O.update_canvas(full, [(m, I16, 1)], views[0], O.settings(shadow=True))
    cv.render_scene(None)
    cv.update_settings(gst(shadow=True, edges=True))
    cv.canvas_to_image(mc, pixels=full)
    oim = O.fill_background(96, 64, 0xff112233, 0xff445566)
    O.canvas_to_image(full, oim, views[0], O.settings(shadow=True, edges=True), omc, ocav)
    compare_rgba(cv.get_image(), oim, 1, "to_image_from")


def test_multi_object_textured_and_vertex_colours(gpu_ctx, oracle_mod, primary):
    from j3d_gb300 import PRIMARY_RASTER, PRIMARY_TRACE, Canvas, Matcap, Mesh, Scene, camera_for_vfov, workloads as W
    O = oracle_mod
    V, T = W.icosphere(4, W.SEED_BASE + 5)
    rng = np.random.default_rng(2)
    colors = rng.uniform(0, 1, size=V.shape).astype(np.float32)
    uv = rng.uniform(-0.1, 1.1, size=(T.shape[0], 6)).astype(np.float32)
    tex = rng.integers(0, 1 << 32, size=(37, 53), dtype=np.uint64).astype(np.uint32)
    gm = Mesh(gpu_ctx, V, T)
    gm2 = Mesh(gpu_ctx, V, T)
    gm.set_vertex_colors(colors)
    gm2.set_uv(uv)
    gm2.set_texture(tex)
    om = O.Mesh(V, T)
    om.set_vertex_colors(colors)
    om2 = O.Mesh(V, T)
    om2.set_uv(uv)
    om2.set_texture(tex)
    cs2 = W.translation(1.2, 0.3, -0.5)
    sc = Scene()
    sc.add_object(gm, I16, 7)
    sc.add_object(gm2, cs2, 9)
    sc.prepare_scene()
    sc.unzoom()
    pose = W.translation(0.5, 0.2, 4.0)
    sc.set_pose(pose)
    mn, mx, diag = O.prepare_scene([(om.min_bb, om.max_bb), (om2.min_bb, om2.max_bb)], [I16, cs2])
    assert np.array_equal(sc.min_bb, mn) and sc.diagonal == diag
    _, _, piv = O.unzoom(mn, mx, diag)
    cam = camera_for_vfov(60.0)
    P = O.make_projection_matrix(O.camera_with_focal(cam.focal_length), 400, 300)
    v = O.view(pose, O.invert_orthonormal(pose), piv, diag, O.invert_projection_matrix(P), 0.1)
    objs = [(om, I16, 7), (om2, cs2, 9)]
    for kw in (dict(shadow=True, edges=False), dict(shadow=True, edges=False, shading=False),
               dict(shadow=True, edges=True)):
        cv = Canvas(gpu_ctx, 400, 300)
        cv.set_camera(cam)
        cv.set_background_color()
        cv.update_settings(gst(**kw))
        mc = Matcap.make(gpu_ctx, 0)
        cv.render_frame(sc, mc)
        assert cv.last_primary() == (PRIMARY_TRACE if primary == "trace" else PRIMARY_RASTER)
        op, oi = oracle_frame(O, None, v, 400, 300, O.settings(**kw), objs=objs)
        gp = cv.get_pixels()
        compare_gbuffers(gp, op, "textured")
        assert set(np.unique(gp["db_id"])) == {0, 7, 9}
        assert ((gp["mark"] & 2) != 0).sum() > 1000
        compare_rgba(cv.get_image(), oi, 1 if kw.get("edges") else 0, "textured")


def test_full_size_torus_frames_match_oracle(gpu_ctx, oracle_mod, primary):
    """28.09M-triangle torus at 1920x1080, all 32 cameras of the benchmark,
    primary + shadow + plain shading: every frame's G-buffer and RGBA image
    equal the oracle's full frame (SHA-256 digests of triangle ids / db ids /
    marks, of the hit records' float bits, of every G-buffer byte and of the
    image, from tests/golden/traffic.json, made by make_traffic.py), and so
    do the per-frame hit and shadowed pixel counts and the ray total. A frame
    whose digests differ is rendered by the oracle and compared pixel by
    pixel, which names the first differing pixels; float fields may then
    differ within 1e-5 relative, nothing else may."""
    import oracle.workloads as OW
    from helpers import frame_digests
    from j3d_gb300 import workloads as W
    O = oracle_mod
    wl = W.config1()
    ref = json.loads((GOLDEN / "traffic.json").read_text())["config1"]
    assert len(ref["digests"]) == len(wl.poses) == 32
    assert np.array_equal(wl.poses.view(np.uint32), OW.cameras(32, W.SEED_BASE + 1 + (1 << 32), 2.5, 4.0).view(np.uint32))
    mesh, sc = gpu_scene(gpu_ctx, wl.vertices, wl.triangles, wl.poses[0])
    info = mesh.info()
    assert info.n_triangles == 28_090_000 and info.n_vertices == 14_045_000
    hits, shadowed, differ = [], [], []
    for i, pose in enumerate(wl.poses):
        sc.set_pose(pose)
        gp, gi, cv, _ = gpu_frame(gpu_ctx, sc, wl.width, wl.height, gst(shadow=True, edges=False), expect=primary)
        cv.close()
        hits.append(int((gp["object_id"] != NO_ID).sum()))
        shadowed.append(int(((gp["mark"] & 1) != 0).sum()))
        if frame_digests(gp, gi) != ref["digests"][i]:
            differ.append(i)
    assert hits == ref["hit_pixels"] and shadowed == ref["shadowed_pixels"]
    assert len(wl.poses) * wl.width * wl.height + sum(hits) == ref["rays"]
    if differ:
        # name the first differing pixels of up to two frames against the oracle's own frame
        m, views, _ = oracle_scene(O, wl.vertices, wl.triangles, wl.poses[differ[:2]], wl.width, wl.height)
        for k, i in enumerate(differ[:2]):
            sc.set_pose(wl.poses[i])
            gp, gi, cv, _ = gpu_frame(gpu_ctx, sc, wl.width, wl.height, gst(shadow=True, edges=False))
            op, oi = oracle_frame(O, m, views[k], wl.width, wl.height, O.settings(shadow=True, edges=False))
            assert frame_digests(op, oi) == ref["digests"][i], "oracle frame differs from its own digest"
            compare_gbuffers(gp, op, f"torus28M cam {i}")
            compare_rgba(gi, oi, 0, f"torus28M cam {i}")
        for i in differ:
            sc.set_pose(wl.poses[i])
            gp, gi, cv, _ = gpu_frame(gpu_ctx, sc, wl.width, wl.height, gst(shadow=True, edges=False))
            cv.close()
            d = frame_digests(gp, gi)
            assert d["ids"] == ref["digests"][i]["ids"], f"cam {i}: triangle / db ids or marks differ"
            assert d["rgba"] == ref["digests"][i]["rgba"], f"cam {i}: RGBA differs"
    print(f"torus28M ({primary}): {32 - len(differ)}/32 frames bit-identical to the oracle, "
          f"{len(differ)} within tolerance")


def test_async_download_overlaps_and_keeps_frame(gpu_ctx):
    """download_async copies the frame queued before it even when the next
    frame is rendered into the same canvas right after (the render waits for
    the copy on the device); the copy equals get_pixels / get_image."""
    import torch
    from j3d_gb300 import workloads as W
    V, T = W.icosphere(4, W.SEED_BASE + 95)
    poses = [W.translation(0, 0, 3.0), W.translation(0.4, 0, 2.5)]
    mesh, sc = gpu_scene(gpu_ctx, V, T, poses[0])
    gp_a, gi_a, cv, mc = gpu_frame(gpu_ctx, sc, 320, 240, gst(shadow=True, edges=False))
    hp = torch.zeros(320 * 240 * 32, dtype=torch.uint8, pin_memory=True)
    hi = torch.zeros(320 * 240 * 4, dtype=torch.uint8, pin_memory=True)
    cv.render_frame(sc, mc)
    cv.download_async(hp, hi)
    sc.set_pose(poses[1])
    cv.render_frame(sc, mc)  # frame B into the same buffers
    cv.download_wait()
    assert np.array_equal(hp.numpy().view(gp_a.dtype).reshape(gp_a.shape), gp_a)
    assert np.array_equal(hi.numpy().view(np.uint32).reshape(gi_a.shape), gi_a)
    gp_b = cv.get_pixels()
    assert not np.array_equal(gp_b, gp_a)


def test_canvas_resize_and_churn_keep_frames(gpu_ctx, oracle_mod):
    """Canvas buffers are freed in stream order: a resize right after
    download_async still delivers the downloaded frame, the resized canvas
    renders the oracle's frame, and canvases created and destroyed in a loop
    (the pattern of a server evicting canvases under an HBM cap) all render
    the oracle's frame."""
    import torch
    from j3d_gb300 import Canvas, camera_for_vfov
    from j3d_gb300 import workloads as W
    O = oracle_mod
    V, T = W.icosphere(4, W.SEED_BASE + 96)
    pose = W.translation(0.2, -0.1, 2.8)
    mesh, sc = gpu_scene(gpu_ctx, V, T, pose)
    st = gst(shadow=True, edges=False)
    gp_a, gi_a, cv, mc = gpu_frame(gpu_ctx, sc, 320, 240, st)
    hp = torch.zeros(320 * 240 * 32, dtype=torch.uint8, pin_memory=True)
    hi = torch.zeros(320 * 240 * 4, dtype=torch.uint8, pin_memory=True)
    cv.render_frame(sc, mc)
    cv.download_async(hp, hi)
    cv.resize(200, 150)
    cv.download_wait()
    assert np.array_equal(hp.numpy().view(gp_a.dtype).reshape(gp_a.shape), gp_a)
    assert np.array_equal(hi.numpy().view(np.uint32).reshape(gi_a.shape), gi_a)
    ref = {}
    for w, h in ((200, 150), (320, 240)):
        m, views, _ = oracle_scene(O, V, T, [pose], w, h)
        ref[(w, h)] = oracle_frame(O, m, views[0], w, h, O.settings(shadow=True, edges=False))
    cv.set_camera(camera_for_vfov(60.0))
    cv.set_background_color()
    cv.render_frame(sc, mc)
    assert compare_gbuffers(cv.get_pixels(), ref[(200, 150)][0], "resized") == 0
    assert np.array_equal(cv.get_image(), ref[(200, 150)][1])
    for i in range(12):
        w, h = (200, 150) if i % 2 else (320, 240)
        c2 = Canvas(gpu_ctx, w, h)
        c2.set_camera(camera_for_vfov(60.0))
        c2.set_background_color()
        c2.update_settings(st)
        c2.render_frame(sc, mc)
        assert compare_gbuffers(c2.get_pixels(), ref[(w, h)][0], f"churn {i}") == 0
        assert np.array_equal(c2.get_image(), ref[(w, h)][1])
        c2.close()


def test_context_refuses_to_close_under_live_objects(gpu_ctx):
    """j3dg_ctx_destroy refuses while meshes, canvases, ... made from the
    context are alive (the context stays usable); Context.close() closes
    them first (newest first) and then the context."""
    from j3d_gb300 import Canvas, Context, J3dgError, Matcap, Mesh, _ffi
    from j3d_gb300 import workloads as W
    from j3d_gb300.scene import _check
    V, T = W.icosphere(2, W.SEED_BASE + 97)
    ctx = Context(0)
    mesh = Mesh(ctx, V, T)
    cv = Canvas(ctx, 64, 48)
    mc = Matcap.make(ctx, 0)
    with pytest.raises(J3dgError) as e:
        _check(ctx.h, _ffi.lib().j3dg_ctx_destroy(ctx.h))
    assert e.value.status == _ffi.J3DG_ERR_INVALID_ARGUMENT
    assert b"3 object" in _ffi.lib().j3dg_last_error(ctx.h)
    cv.render_frame(gpu_scene(ctx, V, T, W.translation(0, 0, 3.0))[1], mc)  # still works
    ctx.close()
    assert ctx.h is None and mesh.h is None and cv.h is None and mc.h is None
