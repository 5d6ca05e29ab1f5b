"""Shared set-up for parity tests: the same scene given to the GPU path and
to the oracle, built through each side's own restatement of j3d's math."""
from __future__ import annotations

import numpy as np

FLT_MAX = np.float32(np.finfo(np.float32).max)
NO_ID = 0xFFFFFFFF


def oracle_scene(O, V, T, poses, w, h, vfov=60.0, leaf=4, n_threads=None, cs_obj=None):
    """Oracle mesh + per-pose views (prepare_scene/unzoom pivot, 60 deg camera)."""
    from oracle.workloads import focal_for_vfov
    m = O.Mesh(V, T, leaf, n_threads)
    cs_obj = np.eye(4, dtype=np.float32).reshape(16) if cs_obj is None else cs_obj
    mn, mx, diag = O.prepare_scene([(m.min_bb, m.max_bb)], [cs_obj])
    _, _, piv = O.unzoom(mn, mx, diag)
    cam = O.camera_with_focal(focal_for_vfov(vfov, 0.768))
    P = O.make_projection_matrix(cam, w, h)
    Pi = O.invert_projection_matrix(P)
    views = [O.view(p, O.invert_orthonormal(p), piv, diag, Pi, cam.near_clipping_plane) for p in poses]
    return m, views, (mn, mx, diag, piv, P, Pi)


def gpu_scene(ctx, V, T, pose, leaf=2, db_id=1, cs_obj=None, build="ploc"):
    from j3d_gb300 import Mesh, Scene
    mesh = Mesh(ctx, V, T, leaf, build)
    sc = Scene()
    sc.add_object(mesh, cs_obj, db_id)
    sc.prepare_scene()
    sc.unzoom()
    sc.set_pose(pose)
    return mesh, sc


def compare_gbuffers(g, o, where=""):
    """Mask and triangle id bit-exact; t, u, v, barycentrics within 1e-5 relative.

    Returns the number of records that are not bit-identical (for reporting)."""
    g = g.reshape(-1)
    o = o.reshape(-1)
    gm = g["object_id"] != NO_ID
    om = o["object_id"] != NO_ID
    assert np.array_equal(gm, om), f"{where}: hit masks differ at {np.flatnonzero(gm != om)[:10]}"
    assert np.array_equal(g["object_id"], o["object_id"]), f"{where}: triangle ids differ"
    assert np.array_equal(g["db_id"], o["db_id"]), f"{where}: db ids differ"
    assert np.array_equal(g["mark"], o["mark"]), f"{where}: shadow/colour marks differ at {np.flatnonzero(g['mark'] != o['mark'])[:10]}"
    for f in ("depth", "u", "v", "barycentric_u", "barycentric_v"):
        a = g[f][gm].astype(np.float64)
        b = o[f][gm].astype(np.float64)
        tol = 1e-5 * np.maximum(np.abs(b), 1e-30) + 1e-30
        bad = np.abs(a - b) > np.maximum(tol, 1e-5 * 1e-3)
        assert not bad.any(), f"{where}: {f} differs beyond 1e-5 relative at {np.flatnonzero(bad)[:10]}"
    return int((g.view(np.uint8).reshape(-1, 32) != o.view(np.uint8).reshape(-1, 32)).any(axis=1).sum())


def compare_rgba(a, b, lsb=1, where=""):
    a8 = a.view(np.uint8).astype(np.int16)
    b8 = b.view(np.uint8).astype(np.int16)
    d = np.abs(a8 - b8)
    assert d.max() <= lsb, f"{where}: RGBA differs by {d.max()} LSB at {np.flatnonzero(d.reshape(-1) > lsb)[:10]}"
    return int((a != b).sum())


GBUFFER_FLOATS = ("depth", "u", "v", "barycentric_u", "barycentric_v")


def frame_digests(pix, im):
    """SHA-256 digests of one frame, so that a full-size frame can be compared
    with the oracle's without storing it:
      ids     object_id, db_id and mark of every pixel (must be bit-exact)
      floats  the bits of depth, u, v and the barycentrics of the hit pixels
      gbuffer every byte of the 32-byte records
      rgba    the shaded RGBA8 image"""
    import hashlib
    p = pix.reshape(-1)
    hit = p["object_id"] != NO_ID
    ids = hashlib.sha256()
    for f in ("object_id", "db_id", "mark"):
        ids.update(np.ascontiguousarray(p[f]).tobytes())
    fl = hashlib.sha256()
    for f in GBUFFER_FLOATS:
        fl.update(np.ascontiguousarray(p[f][hit]).tobytes())
    return {"ids": ids.hexdigest(), "floats": fl.hexdigest(),
            "gbuffer": hashlib.sha256(np.ascontiguousarray(p).view(np.uint8).tobytes()).hexdigest(),
            "rgba": hashlib.sha256(np.ascontiguousarray(im).tobytes()).hexdigest()}
