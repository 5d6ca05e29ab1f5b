"""Per-ray traversal counts of the reference algorithm, for the roofline's
algorithmic bytes: the CPU oracle (4-wide binned-SAH BVH, leaf <= 4, the
reference's qbvh as restated) renders every full frame of a configuration
(primary rays, and shadow rays of the hit pixels) and counts node visits and
triangle tests, and the hit and shadowed pixels of each frame. Written to
tests/golden/traffic.json; bench.py reads the counts, the GPU tests the
per-frame pixels.
Run from the repository root (a few minutes for config 1 on 8 cores):
    python tests/golden/make_traffic.py
"""
from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle.oracle as O  # noqa: E402
from helpers import oracle_scene  # noqa: E402
from j3d_gb300 import build as B  # noqa: E402

OUT = Path(__file__).resolve().parent / "traffic.json"


def count(name, V, T, poses, w, h, threads):
    t0 = time.perf_counter()
    m, views, _ = oracle_scene(O, V, T, poses, w, h, leaf=4, n_threads=threads)
    build_s = time.perf_counter() - t0
    st = O.settings(shadow=True, edges=False)
    rays = visits = tests = 0
    hits, shadowed = [], []
    t0 = time.perf_counter()
    for v in views:
        pix = O.fresh_pixels(w, h)
        s = O.update_canvas(pix, [(m, np.eye(4, dtype=np.float32).reshape(16), 1)], v, st, n_threads=threads)
        rays += s.rays
        visits += s.node_visits
        tests += s.tri_tests
        hits.append(int((pix["object_id"] != 0xFFFFFFFF).sum()))
        shadowed.append(int(((pix["mark"] & 1) != 0).sum()))
    return {"config": name, "frames": len(views), "width": w, "height": h, "triangles": int(T.shape[0]),
            "bvh": "oracle 4-wide binned SAH, leaf <= 4", "rays": int(rays),
            "node_visits_per_ray": round(visits / rays, 4), "tri_tests_per_ray": round(tests / rays, 4),
            "hit_pixels": hits, "shadowed_pixels": shadowed,
            "oracle_build_s": round(build_s, 2), "oracle_trace_s": round(time.perf_counter() - t0, 2)}


def main():
    B.build()
    O.build()
    from j3d_gb300 import workloads as W
    threads = os.cpu_count() or 1
    out = {}
    wl = W.config0()
    out["config0"] = count("icosphere L6, 1024x768, 1 camera", wl.vertices, wl.triangles, wl.poses, wl.width,
                           wl.height, threads)
    print(out["config0"], flush=True)
    wl = W.config1()
    out["config1"] = count("torus 28,090,000 tris, 1920x1080, 32 cameras", wl.vertices, wl.triangles, wl.poses,
                           wl.width, wl.height, threads)
    print(out["config1"], flush=True)
    OUT.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
