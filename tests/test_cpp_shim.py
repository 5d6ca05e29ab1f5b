"""The C++ shim (include/j3dg_scene.hpp) compiles against the C-ABI and, on a
GPU, drives a frame that matches the oracle."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from helpers import compare_gbuffers, compare_rgba

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "shim_frame.cpp"


def build_shim(tmp_path, src: Path = SRC) -> Path:
    from j3d_gb300 import LIB_PATH
    exe = tmp_path / src.stem
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", f"-I{ROOT / 'include'}", str(src), "-o", str(exe),
           f"-L{LIB_PATH.parent}", "-lj3dgpu", f"-Wl,-rpath,{LIB_PATH.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_and_links(product_lib, tmp_path):
    assert build_shim(tmp_path).exists()
    assert build_shim(tmp_path, ROOT / "tests" / "cpp" / "shim_files.cpp").exists()


@pytest.mark.gpu
def test_shim_files_frame_and_pointcloud(product_lib, gpu_ctx, tmp_path):
    """Files through the shim (read_from_file + add_object, mesh and point
    cloud) give the same frame as the Python mirror of the same calls."""
    from j3d_gb300 import Canvas, Geometry, Matcap, PointCloud, Scene, mesh_from_geometry, settings
    from j3d_gb300 import workloads as W
    from oracle import formats as F
    exe = build_shim(tmp_path, ROOT / "tests" / "cpp" / "shim_files.cpp")
    V, T = W.icosphere(4, W.SEED_BASE + 90)
    rng = np.random.default_rng(4)
    col = rng.integers(0, 256, (len(V), 3))
    (tmp_path / "m.ply").write_bytes(F.write_ply(V, T, colors=col))
    P = (V * np.float32(1.05)).astype(np.float32)[::3]
    (tmp_path / "p.xyz").write_bytes(F.write_xyz(P))
    w, h = 320, 240
    r = subprocess.run([str(exe), str(w), str(h), str(tmp_path / "px.bin"), str(tmp_path / "im.bin"),
                        str(tmp_path / "m.ply"), str(tmp_path / "p.xyz")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    from j3d_gb300._ffi import PIXEL_DTYPE
    gp = np.fromfile(tmp_path / "px.bin", PIXEL_DTYPE)
    gi = np.fromfile(tmp_path / "im.bin", np.uint32)
    g = Geometry.read_file(gpu_ctx, tmp_path / "m.ply")
    mesh = mesh_from_geometry(gpu_ctx, g)
    pc = PointCloud(gpu_ctx, geometry=Geometry.read_file(gpu_ctx, tmp_path / "p.xyz"))
    sc = Scene()
    sc.add_object(mesh, None, 1)
    sc.add_pointcloud(pc, None, 2)
    sc.prepare_scene()
    sc.unzoom()
    cv = Canvas(gpu_ctx, w, h)
    cv.set_background_color()
    cv.update_settings(settings(shadow=True, edges=False, textured=False, vertexcolors=True))
    cv.render_frame(sc, Matcap.make(gpu_ctx, 0))
    cv.render_pointclouds(sc)
    ep, ei = cv.get_pixels(), cv.get_image()
    assert np.array_equal(gp.view(np.uint8), ep.reshape(-1).view(np.uint8))
    assert np.array_equal(gi, ei.reshape(-1))
    assert (ep["db_id"] == 2).sum() > 100 and (ep["db_id"] == 1).sum() > 1000


@pytest.mark.gpu
@pytest.mark.parametrize("edges", [0, 1])
def test_shim_frame_matches_oracle(product_lib, oracle_mod, gpu_ctx, tmp_path, edges):
    O = oracle_mod
    from j3d_gb300 import workloads as W
    from helpers import oracle_scene
    exe = build_shim(tmp_path)
    w, h = 320, 240
    r = subprocess.run([str(exe), "4", str(w), str(h), "3.0", str(edges), str(tmp_path / "p.bin"),
                        str(tmp_path / "i.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    gp = np.fromfile(tmp_path / "p.bin", O.PIXEL_DTYPE).reshape(h, w)
    gi = np.fromfile(tmp_path / "i.bin", np.uint32).reshape(h, w)
    V, T = W.icosphere(4)
    pose = W.translation(0, 0, 3.0)
    m, views, _ = oracle_scene(O, V, T, [pose], w, h)
    st = O.settings(shadow=True, edges=bool(edges))
    mc, cav = O.make_matcap(0)
    op = O.fresh_pixels(w, h)
    oi = np.zeros((h, w), np.uint32)
    O.render_frame(op, oi, O.fill_background(w, h), [(m, np.eye(4, dtype=np.float32).reshape(16), 1)], views[0], st,
                   mc, cav)
    assert compare_gbuffers(gp, op, "shim") == 0
    compare_rgba(gi, oi, 1 if edges else 0, "shim")
