"""Serving loop: every request renders the same bytes alone and in the mix,
admission by HBM footprint binds under a low cap, and all requests finish."""
import numpy as np
import pytest

from j3d_gb300.serve import CanvasPool, Request, poisson_requests


def test_poisson_requests_deterministic():
    a = poisson_requests(50, 400.0, ["a", "b"], seed=5)
    b = poisson_requests(50, 400.0, ["a", "b"], seed=5)
    assert [(r.mesh, r.resolution, r.arrival) for r in a] == [(r.mesh, r.resolution, r.arrival) for r in b]
    gaps = np.diff([r.arrival for r in a])
    assert (gaps > 0).all() and 0.5 / 400 < gaps.mean() < 2.0 / 400
    assert CanvasPool.canvas_bytes(1920, 1080) == 1920 * 1080 * 88 + 16384 + 16


def _server(ctx, cap, **kw):
    from j3d_gb300 import workloads as W
    from j3d_gb300.serve import RenderServer
    srv = RenderServer(ctx, cap, keep_images=True, **kw)
    for i, (nu, nv) in enumerate([(120, 60), (300, 150), (60, 30)]):
        assert srv.add_mesh(f"m{i}", *W.torus(nu, nv, seed=W.SEED_BASE + 50 + i))
    return srv


def _alone(ctx, srv, r):
    from j3d_gb300 import Canvas, Matcap, camera_for_vfov, settings
    cv = Canvas(ctx, *r.resolution)
    cv.set_camera(camera_for_vfov(60.0))
    cv.set_background_color()
    cv.update_settings(settings(shadow=True, edges=False))
    cv.render_frame(srv._scene(r), srv.matcap)
    return cv.get_image()


@pytest.mark.gpu
def test_requests_alone_equal_in_the_mix(gpu_ctx):
    srv = _server(gpu_ctx, 8 << 30, max_slots=8)
    reqs = poisson_requests(40, 4000.0, ["m0", "m1", "m2"], seed=11, resolutions=((64, 64), (128, 72), (96, 54)))
    st = srv.run(reqs, realtime=True)
    assert st.requests == 40 and all(r.done >= r.arrival for r in reqs)
    assert st.batches >= 2 and st.mean_batch >= 1.0
    for r in reqs:
        assert np.array_equal(srv.images[r.rid], _alone(gpu_ctx, srv, r)), f"request {r.rid}"


@pytest.mark.gpu
def test_admission_binds_under_a_low_cap(gpu_ctx):
    srv = _server(gpu_ctx, 8 << 30)
    meshes = srv.mesh_bytes
    # room for the meshes and exactly one 128x128 canvas
    srv.cap = meshes + CanvasPool.canvas_bytes(128, 128) + 100
    reqs = poisson_requests(12, 10000.0, ["m0", "m1"], seed=3, resolutions=((128, 128),))
    st = srv.run(reqs, realtime=True)
    assert st.requests == 12 and st.max_in_flight_frames <= 1
    assert srv.peak_bytes <= srv.cap and srv.pool.count == 1
    for r in reqs:
        assert np.array_equal(srv.images[r.rid], _alone(gpu_ctx, srv, r))
    # a mesh larger than the cap is refused, nothing is allocated for it
    from j3d_gb300 import workloads as W
    assert not srv.add_mesh("big", *W.torus(400, 200))


@pytest.mark.gpu
def test_learned_requests_equal_plain_frames(gpu_ctx):
    """With a learned network attached to a mesh, its requests render through
    the learned path; every image equals the plain frame alone, and requests
    of the other meshes still go through the batched plain path."""
    from j3d_gb300.learned import Learned
    srv = _server(gpu_ctx, 8 << 30, max_slots=8)
    net = Learned(gpu_ctx, srv.meshes["m1"], cluster_depth=3, batch=4096, seed=3)
    net.train(4096 * 20)
    srv.attach_learned("m1", net)
    reqs = poisson_requests(30, 3000.0, ["m0", "m1", "m2"], seed=12, resolutions=((64, 64), (128, 72)))
    st = srv.run(reqs, realtime=True)
    assert st.requests == 30 and any(r.mesh == "m1" for r in reqs)
    for r in reqs:
        assert np.array_equal(srv.images[r.rid], _alone(gpu_ctx, srv, r)), f"request {r.rid} ({r.mesh})"
    with pytest.raises(ValueError):
        srv.attach_learned("m0", net)
