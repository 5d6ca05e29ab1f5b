"""All-hits query, voxel grid (vox.cpp:284-380) and picking helpers
(pixel.cpp:6-25, view.cpp:439-459): oracle self-checks on the CPU, GPU
parity through the C-ABI on a GPU."""
import numpy as np
import pytest

from helpers import FLT_MAX, NO_ID, oracle_scene

I16 = np.eye(4, dtype=np.float32).reshape(16)


def axis_rays(O, mesh, n=300, seed=0):
    rng = np.random.default_rng(seed)
    rays = np.zeros(n, O.RAY_DTYPE)
    for i in range(n):
        a = i % 3
        o = rng.uniform(mesh.min_bb, mesh.max_bb).astype(np.float32)
        o[a] = mesh.min_bb[a] - (0.0 if i % 2 else 0.5)
        d = np.zeros(3, np.float32)
        d[a] = 2.0 if a == 2 else 1.0
        rays[i]["orig"][:3] = o
        rays[i]["orig"][3] = 1
        rays[i]["dir"][:3] = d
        rays[i]["t_near"] = 0.0
        rays[i]["t_far"] = FLT_MAX if i % 5 else 1.0
    return rays


def test_oracle_find_all_bvh_equals_brute(oracle_mod, product_lib):
    from j3d_gb300 import workloads as W
    O = oracle_mod
    V, T = W.icosphere(4, W.SEED_BASE + 21)
    m = O.Mesh(V, T)
    rays = axis_rays(O, m)
    total = 0
    for r in rays:
        a = O.find_all(m, r)
        b = O.find_all(m, r, brute=True)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
        d = a["distance"]
        assert (np.diff(d) >= 0).all()
        total += len(a)
    assert total > 200


def test_oracle_voxel_grid_properties(oracle_mod, product_lib):
    from j3d_gb300 import workloads as W
    O = oracle_mod
    V, T = W.icosphere(3)
    m = O.Mesh(V, T)
    g = O.voxelize(m, 24)
    assert g.shape[2] == 24 or max(g.shape) == 24
    # white mesh: every set voxel is colour index 255 (vox.cpp:154-173 of (255,255,255))
    assert set(np.unique(g)) == {0, 255}
    # a closed sphere: the shell is hit, the centre voxel is not
    assert g[g.shape[0] // 2, g.shape[1] // 2, g.shape[2] // 2] == 0
    assert (g != 0).sum() > 500


def test_oracle_picking(oracle_mod, product_lib):
    from j3d_gb300 import scene as S, workloads as W
    O = oracle_mod
    V, T = W.icosphere(3)
    pose = W.translation(0, 0, 3)
    m, views, _ = oracle_scene(O, V, T, [pose], 64, 48)
    pix = O.fresh_pixels(64, 48)
    O.update_canvas(pix, [(m, I16, 1)], views[0], O.settings())
    cs = W.translation(0.5, -0.25, 2.0)
    hits = pix.reshape(-1)[pix.reshape(-1)["object_id"] != NO_ID]
    for p in hits[::37]:
        assert S.get_closest_vertex(p, V, T) == O.get_closest_vertex(p, V, T)
        assert np.array_equal(S.get_world_position(p, V, T, cs), O.get_world_position(p, V, T, cs))
        vid = O.get_closest_vertex(p, V, T)
        assert vid in T[p["object_id"]]
        wp = O.get_world_position(p, V, T, I16)
        assert np.abs(wp).max() < 2.0


@pytest.mark.gpu
def test_gpu_find_all_matches_oracle(gpu_ctx, oracle_mod):
    from j3d_gb300 import Mesh, find_all, workloads as W
    O = oracle_mod
    V, T = W.icosphere(5, W.SEED_BASE + 22)
    m = O.Mesh(V, T)
    gm = Mesh(gpu_ctx, V, T)
    rays = axis_rays(O, m, 2000, seed=3)
    rng = np.random.default_rng(9)
    rays["dir"][::7, :3] = rng.normal(size=(len(rays[::7]), 3)).astype(np.float32)  # some oblique rays
    for cap in (64, 2):
        hits, counts = find_all(gpu_ctx, gm, rays, cap)
        for i, r in enumerate(rays):
            o = O.find_all(m, r)
            assert counts[i] == len(o)
            k = min(cap, len(o))
            assert np.array_equal(hits[i, :k].view(np.uint8), o[:k].view(np.uint8))


@pytest.mark.gpu
@pytest.mark.parametrize("colours", ["white", "vertex", "texture"])
def test_gpu_voxel_grid_matches_oracle(gpu_ctx, oracle_mod, colours):
    from j3d_gb300 import Mesh, voxelize, workloads as W
    O = oracle_mod
    V, T = W.icosphere(4, W.SEED_BASE + 23)
    m = O.Mesh(V, T)
    gm = Mesh(gpu_ctx, V, T)
    rng = np.random.default_rng(4)
    if colours == "vertex":
        c = rng.uniform(0, 1, size=V.shape).astype(np.float32)
        m.set_vertex_colors(c)
        gm.set_vertex_colors(c)
    elif colours == "texture":
        uv = rng.uniform(0, 1, size=(T.shape[0], 6)).astype(np.float32)
        tex = rng.integers(0, 1 << 32, size=(16, 16), dtype=np.uint64).astype(np.uint32)
        m.set_uv(uv)
        m.set_texture(tex)
        gm.set_uv(uv)
        gm.set_texture(tex)
    for max_dim in (1, 17, 64):
        g = voxelize(gpu_ctx, gm, max_dim)
        o = O.voxelize(m, max_dim)
        assert g.shape == o.shape
        assert np.array_equal(g, o), f"{colours} {max_dim}: {(g != o).sum()} voxels differ"
    assert (g != 0).sum() > 1000


@pytest.mark.gpu
def test_gpu_voxel_grid_full_size_torus_properties(gpu_ctx):
    """28.09M triangles: the grid is deterministic and shell-shaped."""
    from j3d_gb300 import Mesh, voxelize, workloads as W
    V, T = W.torus(5300, 2650, seed=W.SEED_BASE + 1)
    gm = Mesh(gpu_ctx, V, T)
    a = voxelize(gpu_ctx, gm, 256)
    b = voxelize(gpu_ctx, gm, 256)
    assert np.array_equal(a, b)
    assert a.shape[2] == 256 or a.shape[0] == 256
    assert set(np.unique(a)) == {0, 255}
    # the torus hole along y is empty at the centre column
    z, y, x = a.shape
    assert not a[z // 2, :, x // 2].any()
