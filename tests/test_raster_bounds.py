"""The rasterised primary hits rest on one claim: every (pixel, triangle) pair
that the traversal's ray / triangle test accepts has the pixel centre inside
the triangle's candidate rectangle. The rectangle is the projected box of
the triangle, widened by twice the rays' slab padding, plus a 0.05-pixel
margin. Here the oracle's brute-force all-hits query (the same Moller-Trumbore
+ gate, every accepted triangle of every primary ray) is checked against
that rectangle, computed in double precision, with a margin ten times
smaller (0.005 px). So the margin the kernels use has at least a tenfold
reserve on these scenes. CPU only."""
import numpy as np
import pytest

from helpers import oracle_scene

MARGIN_CHECKED = 0.005  # pixels; the kernels use 0.05


def candidate_rect(M, pad, a, b, c, w, h):
    """Projected pixel-centre bounds of the widened box of triangle (a, b, c)
    (interval bounds of clip x, y, w over the box; the kernel's arithmetic in
    double). None when the box reaches the camera plane."""
    lo = np.minimum(np.minimum(a, b), c) - 2.0 * pad
    hi = np.maximum(np.maximum(a, b), c) + 2.0 * pad
    d = hi - lo
    rng = []
    for r in (0, 1, 3):
        base = M[r, :3] @ lo + M[r, 3]
        t = M[r, :3] * d
        rng.append((base + np.minimum(t, 0).sum(), base + np.maximum(t, 0).sum()))
    (xl, xh), (yl, yh), (wl, wh) = rng
    if wl <= 0:
        return None
    x0 = (min(xl / wl, xl / wh) + 1) * w / 2 - 0.5
    x1 = (max(xh / wl, xh / wh) + 1) * w / 2 - 0.5
    y0 = (min(yl / wl, yl / wh) + 1) * h / 2 - 0.5
    y1 = (max(yh / wl, yh / wh) + 1) * h / 2 - 0.5
    return x0, x1, y0, y1


@pytest.mark.parametrize("case", ["icosphere_near", "torus_far", "torus_off_centre"])
def test_accepted_hits_lie_in_the_candidate_rectangles(oracle_mod, case):
    from j3d_gb300 import workloads as W
    O = oracle_mod
    w, h = 48, 36
    if case == "icosphere_near":
        V, T = W.icosphere(3, W.SEED_BASE + 31)
        pose = W.translation(0.05, -0.02, 1.4)
    elif case == "torus_far":
        V, T = W.torus(60, 30, seed=W.SEED_BASE + 32)
        pose = W.cameras(1, W.SEED_BASE + 33, 3.0, 3.5)[0]
    else:
        V, T = W.torus(60, 30, seed=W.SEED_BASE + 34)
        pose = W.cameras(1, W.SEED_BASE + 35, 2.5, 3.0, target=(0.9, 0.2, -0.4))[0]
    m, views, (mn, mx, diag, piv, P, Pi) = oracle_scene(O, V, T, [pose], w, h)
    from j3d_gb300 import camera_for_vfov
    near = camera_for_vfov(60.0).near_clipping_plane
    t_near = np.float32(diag) / np.float32(100.0)
    rays = O.primary_rays(w, h, pose, Pi, near, t_near)
    # object space = world space (identity instance); the camera's rays all
    # start at the eye, so the padding is one number (make_ray's formula)
    eye = rays[0]["orig"].astype(np.float32)
    scale = np.float32(np.max(np.abs(np.concatenate([m.min_bb, m.max_bb]))))
    pad = float((np.float32(np.max(np.abs(eye))) + scale) * np.float32(2.0 ** -19))
    cs = np.asarray(pose, np.float64).reshape(4, 4, order="F")
    Pm = np.asarray(P, np.float64).reshape(4, 4, order="F")
    # clip z (row 2) holds the far plane's terms and is not used
    with np.errstate(all="ignore"):
        M = Pm @ np.linalg.inv(cs)
    assert np.isfinite(M[[0, 1, 3]]).all()
    Vd = V.astype(np.float64)
    checked = 0
    worst = -np.inf  # largest distance (pixels) of an accepted pixel outside its rectangle
    for k, ray in enumerate(rays):
        hits = O.find_all(m, ray, brute=True)
        x, y = k % w, k // w
        for hit in hits:
            tri = T[int(hit["object_id"])]
            r = candidate_rect(M, pad, Vd[tri[0]], Vd[tri[1]], Vd[tri[2]], w, h)
            if r is None:
                continue
            x0, x1, y0, y1 = r
            worst = max(worst, x0 - x, x - x1, y0 - y, y - y1)
            checked += 1
    assert checked > 200 and np.isfinite(worst), f"{case}: only {checked} accepted hits"
    assert worst <= MARGIN_CHECKED, f"{case}: an accepted pixel lies {worst:.4f} px outside its rectangle"
