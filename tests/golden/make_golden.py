"""Generates the golden fixtures of tests/golden/ with the CPU oracle.

The reference ships no tests or golden vectors (its BVH library is an absent
submodule), so these fixtures pin the oracle against itself over time and
pin the GPU path against the oracle: hashes of full frames plus a sparse
sample of records. Run from the repository root:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle.oracle as O  # noqa: E402
from helpers import oracle_scene  # noqa: E402
from j3d_gb300 import build as B  # noqa: E402

OUT = Path(__file__).resolve().parent
STRIDE = 97


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def frame(O, m, v, w, h, st, mc, cav):
    pix = O.fresh_pixels(w, h)
    im = np.zeros((h, w), np.uint32)
    bg = O.fill_background(w, h)
    O.render_frame(pix, im, bg, [(m, np.eye(4, dtype=np.float32).reshape(16), 1)], v, st, mc, cav)
    return pix, im


def case(name, V, T, poses, w, h, out, npz):
    m, views, (mn, mx, diag, piv, P, Pi) = oracle_scene(O, V, T, poses, w, h)
    mc, cav = O.make_matcap(0)
    rec = {"mesh_sha": sha(V) + sha(T), "nv": int(V.shape[0]), "nt": int(T.shape[0]), "w": w, "h": h,
           "bbox": [mn.tolist(), mx.tolist()], "diagonal": float(diag), "projection": P.tolist(),
           "normals_sha": sha(m.normals()), "frames": []}
    for i, v in enumerate(views):
        fr = {}
        for mode, st in (("plain", O.settings(shadow=True, edges=False)), ("edges", O.settings(shadow=True, edges=True))):
            pix, im = frame(O, m, v, w, h, st, mc, cav)
            fr[mode] = {"gbuffer_sha": sha(pix), "rgba_sha": sha(im),
                        "hits": int((pix["object_id"] != 0xFFFFFFFF).sum()),
                        "shadowed": int(((pix["mark"] & 1) != 0).sum())}
            npz[f"{name}_{i}_{mode}_pix"] = pix.reshape(-1)[::STRIDE]
            npz[f"{name}_{i}_{mode}_rgba"] = im.reshape(-1)[::STRIDE]
        rec["frames"].append(fr)
    out[name] = rec


def main():
    B.build()
    O.build()
    from j3d_gb300 import workloads as W
    out, npz = {}, {}
    wl = W.config0()
    case("icosphere_L6_1024x768", wl.vertices, wl.triangles, wl.poses, wl.width, wl.height, out, npz)
    V, T = W.torus(120, 60, seed=W.SEED_BASE + 1)
    poses = W.cameras(3, W.SEED_BASE + 1 + (1 << 32), 2.5, 4.0)
    case("torus_120x60_320x240", V, T, poses, 320, 240, out, npz)
    (OUT / "golden.json").write_text(json.dumps(out, indent=1, sort_keys=True))
    np.savez_compressed(OUT / "golden_samples.npz", **npz)
    print("wrote", OUT / "golden.json", OUT / "golden_samples.npz")


if __name__ == "__main__":
    main()
