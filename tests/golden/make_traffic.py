"""Full-size oracle frames of the benchmark configurations, kept as counts and
digests: the CPU oracle (4-wide binned-SAH BVH, leaf <= 4, the reference's
qbvh as restated) renders every frame of a configuration (background, primary
rays, hit records, shadow rays of the hit pixels, plain matcap shading) and
records per frame
  - node visits and triangle tests (summed; the roofline's algorithmic bytes),
  - the hit and shadowed pixel counts,
  - SHA-256 digests of the G-buffer and RGBA image (tests/helpers.py
    frame_digests), so that the GPU tests compare every full-size frame with
    the oracle's bit for bit without storing 2 GB of frames.
Written to tests/golden/traffic.json. Inputs come from the oracle's own
generators (oracle/workloads.py), so nothing here runs the product.
Run from the repository root (about a minute for config 1 on 8 cores):
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
import oracle.workloads as OW  # noqa: E402
from helpers import frame_digests, oracle_scene  # noqa: E402

OUT = Path(__file__).resolve().parent / "traffic.json"


def count(name, V, T, poses, w, h, threads):
    t0 = time.perf_counter()
    m, views, _ = oracle_scene(O, V, T, poses, w, h, leaf=4, n_threads=threads)
    build_s = time.perf_counter() - t0
    st = O.settings(shadow=True, edges=False)
    mc, cav = O.make_matcap(0)
    bg = O.fill_background(w, h)
    I16 = np.eye(4, dtype=np.float32).reshape(16)
    rays = visits = tests = 0
    hits, shadowed, digests = [], [], []
    t0 = time.perf_counter()
    for v in views:
        pix = O.fresh_pixels(w, h)
        im = np.zeros((h, w), np.uint32)
        _, _, s = O.render_frame(pix, im, bg, [(m, I16, 1)], v, st, mc, cav, n_threads=threads)
        rays += s.rays
        visits += s.node_visits
        tests += s.tri_tests
        hits.append(int((pix["object_id"] != 0xFFFFFFFF).sum()))
        shadowed.append(int(((pix["mark"] & 1) != 0).sum()))
        digests.append(frame_digests(pix, im))
    return {"config": name, "frames": len(views), "width": w, "height": h, "triangles": int(T.shape[0]),
            "bvh": "oracle 4-wide binned SAH, leaf <= 4", "rays": int(rays),
            "node_visits_per_ray": round(visits / rays, 4), "tri_tests_per_ray": round(tests / rays, 4),
            "hit_pixels": hits, "shadowed_pixels": shadowed, "digests": digests,
            "oracle_build_s": round(build_s, 2), "oracle_trace_s": round(time.perf_counter() - t0, 2)}


def main():
    O.build()
    threads = os.cpu_count() or 1
    out = {}
    V, T, poses, w, h = OW.config0()
    out["config0"] = count("icosphere L6, 1024x768, 1 camera", V, T, poses, w, h, threads)
    print({k: v for k, v in out["config0"].items() if k != "digests"}, flush=True)
    V, T, poses, w, h = OW.config1()
    out["config1"] = count("torus 28,090,000 tris, 1920x1080, 32 cameras", V, T, poses, w, h, threads)
    print({k: v for k, v in out["config1"].items() if k != "digests"}, flush=True)
    OUT.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
