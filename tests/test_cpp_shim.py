"""The C++ shim (include/j3dg_scene.hpp) compiles against the C-ABI and, on a
GPU, drives a frame that matches the oracle."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from helpers import compare_gbuffers, compare_rgba

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "shim_frame.cpp"


def build_shim(tmp_path) -> Path:
    from j3d_gb300 import LIB_PATH
    exe = tmp_path / "shim_frame"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", f"-I{ROOT / 'include'}", str(SRC), "-o", str(exe),
           f"-L{LIB_PATH.parent}", "-lj3dgpu", f"-Wl,-rpath,{LIB_PATH.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_and_links(product_lib, tmp_path):
    assert build_shim(tmp_path).exists()


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
