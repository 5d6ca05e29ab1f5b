"""CPU tests of the oracle: known answers, BVH == brute force, golden fixtures."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import FLT_MAX, NO_ID, oracle_scene

GOLDEN = Path(__file__).resolve().parent / "golden"
I16 = np.eye(4, dtype=np.float32).reshape(16)


def rays_from(orig, dirs, t_near=0.0, t_far=FLT_MAX):
    import oracle.oracle as O
    r = np.zeros(len(dirs), O.RAY_DTYPE)
    r["orig"][:, :3] = orig
    r["orig"][:, 3] = 1
    r["dir"][:, :3] = dirs
    r["t_near"] = t_near
    r["t_far"] = t_far
    return r


def test_known_answer_unit_triangle(oracle_mod):
    O = oracle_mod
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    T = np.array([[0, 1, 2]], np.uint32)
    m = O.Mesh(V, T)
    # straight down onto (0.25, 0.25): t = 2, u = 0.25, v = 0.25
    r = rays_from(np.array([[0.25, 0.25, 2.0]], np.float32), np.array([[0, 0, -1]], np.float32))
    h, _ = O.find_closest([(m, I16, 1)], r)
    assert h["found"][0] == 1 and h["distance"][0] == 2.0 and h["u"][0] == 0.25 and h["v"][0] == 0.25
    assert h["object_id"][0] == 0 and h["two_level_index"][0] == 0
    # outside the triangle
    r = rays_from(np.array([[0.75, 0.75, 2.0]], np.float32), np.array([[0, 0, -1]], np.float32))
    assert O.find_closest([(m, I16, 1)], r)[0]["found"][0] == 0
    # vertex and edge grazing hits are inside (u >= 0, v >= 0, u + v <= 1)
    for p in ([0, 0, 2], [1, 0, 2], [0, 1, 2], [0.5, 0.5, 2], [0.5, 0, 2]):
        r = rays_from(np.array([p], np.float32), np.array([[0, 0, -1]], np.float32))
        assert O.find_closest([(m, I16, 1)], r)[0]["found"][0] == 1, p
    # t_near and t_far bound the hit (t in (t_near, t_far))
    r = rays_from(np.array([[0.25, 0.25, 2.0]], np.float32), np.array([[0, 0, -1]], np.float32), t_near=2.0)
    assert O.find_closest([(m, I16, 1)], r)[0]["found"][0] == 0
    r = rays_from(np.array([[0.25, 0.25, 2.0]], np.float32), np.array([[0, 0, -1]], np.float32), t_far=2.0)
    assert O.find_closest([(m, I16, 1)], r)[0]["found"][0] == 0
    # parallel ray: det == 0
    r = rays_from(np.array([[0.25, 0.25, 0.0]], np.float32), np.array([[1, 0, 0]], np.float32))
    assert O.find_closest([(m, I16, 1)], r)[0]["found"][0] == 0


def test_ties_break_to_smaller_id(oracle_mod):
    O = oracle_mod
    # the same triangle three times: equal t, the smallest id wins
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    T = np.array([[0, 1, 2], [0, 1, 2], [0, 1, 2]], np.uint32)[[2, 1, 0]]
    for leaf in (1, 4):
        m = O.Mesh(V, T, leaf)
        r = rays_from(np.array([[0.2, 0.2, 1.0]], np.float32), np.array([[0, 0, -1]], np.float32))
        h, _ = O.find_closest([(m, I16, 1)], r)
        assert h["object_id"][0] == 0
    # shared edge: a ray through the edge hits both; the smaller id wins
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], np.float32)
    T = np.array([[1, 3, 2], [0, 1, 2]], np.uint32)
    m = O.Mesh(V, T, 1)
    r = rays_from(np.array([[0.5, 0.5, 1.0]], np.float32), np.array([[0, 0, -1]], np.float32))
    h, _ = O.find_closest([(m, I16, 1)], r)
    assert h["found"][0] == 1 and h["object_id"][0] == 0
    # two instances at the same depth: the smaller instance index wins
    h, _ = O.find_closest([(m, I16, 1), (m, I16, 2)], r)
    assert h["two_level_index"][0] == 0


def _random_rays(rng, n, box_lo, box_hi, spread=3.0):
    o = rng.uniform(box_lo - spread, box_hi + spread, size=(n, 3)).astype(np.float32)
    target = rng.uniform(box_lo, box_hi, size=(n, 3)).astype(np.float32)
    return o, (target - o).astype(np.float32)


@pytest.mark.parametrize("leaf", [1, 2, 4, 8])
def test_bvh_equals_brute_force_random_rays(oracle_mod, leaf, product_lib):
    from j3d_gb300 import workloads as W
    O = oracle_mod
    V, T = W.icosphere(4, W.SEED_BASE + 7)
    m = O.Mesh(V, T, leaf)
    rng = np.random.default_rng(leaf)
    o, d = _random_rays(rng, 4000, m.min_bb, m.max_bb)
    r = rays_from(o, d, t_near=1e-3)
    for any_hit in (False, True):
        a, sa = O.find_closest([(m, I16, 1)], r, any_hit=any_hit)
        b, _ = O.find_closest([(m, I16, 1)], r, brute=True, any_hit=any_hit)
        if any_hit:
            assert np.array_equal(a["found"], b["found"])
        else:
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    assert sa.node_visits > 0


def test_bvh_equals_brute_force_two_level(oracle_mod, product_lib):
    from j3d_gb300 import workloads as W
    O = oracle_mod
    V, T = W.icosphere(3, W.SEED_BASE + 8)
    m = O.Mesh(V, T, 4)
    cs2 = W.translation(0.7, 0.1, -0.3)
    rot = np.array([0, 0, 1, 0, 0, 1, 0, 0, -1, 0, 0, 0, 0.2, -0.5, 0.4, 1], np.float32)  # 90 deg about y
    objs = [(m, I16, 3), (m, cs2, 4), (m, rot, 5)]
    rng = np.random.default_rng(5)
    o, d = _random_rays(rng, 3000, np.array([-1.5, -1.5, -1.5]), np.array([1.5, 1.5, 1.5]))
    r = rays_from(o, d, t_near=1e-3)
    a, _ = O.find_closest(objs, r)
    b, _ = O.find_closest(objs, r, brute=True)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    assert len(set(a["two_level_index"][a["found"] == 1].tolist())) == 3


def test_golden_fixtures(oracle_mod, product_lib):
    """The oracle reproduces the committed golden frames (hashes + sampled records)."""
    from j3d_gb300 import workloads as W
    O = oracle_mod
    gold = json.loads((GOLDEN / "golden.json").read_text())
    samples = np.load(GOLDEN / "golden_samples.npz")
    wl = W.config0()
    cases = {"icosphere_L6_1024x768": (wl.vertices, wl.triangles, wl.poses, wl.width, wl.height)}
    V, T = W.torus(120, 60, seed=W.SEED_BASE + 1)
    cases["torus_120x60_320x240"] = (V, T, W.cameras(3, W.SEED_BASE + 1 + (1 << 32), 2.5, 4.0), 320, 240)
    mc, cav = O.make_matcap(0)
    for name, (V, T, poses, w, h) in cases.items():
        g = gold[name]
        sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
        assert sha(V) + sha(T) == g["mesh_sha"], f"{name}: synthetic mesh changed"
        m, views, (mn, mx, diag, piv, P, Pi) = oracle_scene(O, V, T, poses, w, h)
        assert P.tolist() == g["projection"]
        assert sha(m.normals()) == g["normals_sha"]
        for i, v in enumerate(views):
            for mode, st in (("plain", O.settings(shadow=True, edges=False)), ("edges", O.settings(shadow=True, edges=True))):
                pix = O.fresh_pixels(w, h)
                im = np.zeros((h, w), np.uint32)
                O.render_frame(pix, im, O.fill_background(w, h), [(m, I16, 1)], v, st, mc, cav)
                fr = g["frames"][i][mode]
                assert np.array_equal(pix.reshape(-1)[::97], samples[f"{name}_{i}_{mode}_pix"])
                assert sha(pix) == fr["gbuffer_sha"] and sha(im) == fr["rgba_sha"], f"{name} frame {i} {mode}"


def test_render_region_and_empty_scene(oracle_mod, product_lib):
    from j3d_gb300 import workloads as W
    O = oracle_mod
    V, T = W.icosphere(3)
    poses = W.translation(0, 0, 3)[None]
    m, views, _ = oracle_scene(O, V, T, poses, 64, 48)
    st = O.settings(shadow=True, edges=False)
    full = O.fresh_pixels(64, 48)
    O.update_canvas(full, [(m, I16, 1)], views[0], st)
    part = O.fresh_pixels(64, 48)
    O.update_canvas(part, [(m, I16, 1)], views[0], st, rect=(10, 5, 40, 30))
    assert np.array_equal(part[5:31, 10:41], full[5:31, 10:41])
    assert (part["object_id"][:5] == NO_ID).all()
    empty = O.fresh_pixels(64, 48)
    empty["object_id"] = 7
    O.update_canvas(empty, [], views[0], st)
    assert (empty["object_id"] == NO_ID).all() and (empty["depth"] == FLT_MAX).all()


def test_row_pool_gives_the_same_frame_at_any_thread_count(oracle_mod):
    """The oracle's persistent row pool (workers started once, like
    pooled_parallel_for's thread pool) renders the same G-buffer and image
    with 1, 2, 3 or all threads, call after call."""
    import os
    import oracle.workloads as OW
    O = oracle_mod
    V, T = OW.icosphere(4, OW.SEED_BASE + 7)
    m, views, _ = oracle_scene(O, V, T, OW.translation(0.1, 0.0, 2.6)[None], 160, 120)
    mc, cav = O.make_matcap(0)
    st = O.settings(shadow=True, edges=False)
    frames = []
    for nt in (1, 2, 3, os.cpu_count() or 1, 1, os.cpu_count() or 1):
        pix = O.fresh_pixels(160, 120)
        im = np.zeros((120, 160), np.uint32)
        _, _, s = O.render_frame(pix, im, O.fill_background(160, 120), [(m, I16, 1)], views[0], st, mc, cav,
                                 n_threads=nt)
        frames.append((pix, im, s.rays, s.node_visits, s.tri_tests))
    for f in frames[1:]:
        assert np.array_equal(f[0].view(np.uint8), frames[0][0].view(np.uint8)) and np.array_equal(f[1], frames[0][1])
        assert f[2:] == frames[0][2:]
    assert (frames[0][0]["object_id"] != NO_ID).sum() > 1000
