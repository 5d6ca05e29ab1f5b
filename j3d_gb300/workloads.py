"""Seeded synthetic workloads standing in for the meshes j3d loads from files.

No public dataset is involved: the reference's README quotes a 28,055,742-
triangle scan; a displaced torus of 28,090,000 triangles stands in for it.
The generators live in libj3dgpu.so (host code, deterministic on x86 and Arm).

Seeds: 0x6A3D0000 + configuration index for the mesh; the cameras of a
configuration use that seed + 2**32.
  icosphere  level 6: 81,920 triangles, 40,962 vertices, radius
             1 + 0.05 sum_{k=1..8} a_k sin(f_k (d.u_k) + phi_k)
  torus      R = 1, r = 0.35, 5300 x 2650 periodic grid: 28,090,000 triangles,
             14,045,000 vertices, radial displacement 0.02 x sum of 16 sinusoids
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._ffi import fptr, lib, vptr

SEED_BASE = 0x6A3D0000


def icosphere(level: int = 6, seed: int = SEED_BASE, amp: float = 0.05) -> tuple[np.ndarray, np.ndarray]:
    nv = 10 * 4 ** level + 2
    nt = 20 * 4 ** level
    V = np.empty((nv, 3), np.float32)
    T = np.empty((nt, 3), np.uint32)
    st = lib().j3dg_synth_icosphere(level, seed, amp, vptr(V), vptr(T))
    if st:
        raise ValueError(f"icosphere(level={level}) failed: {st}")
    return V, T


def torus(nu: int = 5300, nv: int = 2650, R: float = 1.0, r: float = 0.35, seed: int = SEED_BASE + 1,
          amp: float = 0.02) -> tuple[np.ndarray, np.ndarray]:
    V = np.empty((nu * nv, 3), np.float32)
    T = np.empty((2 * nu * nv, 3), np.uint32)
    st = lib().j3dg_synth_torus(nu, nv, R, r, seed, amp, vptr(V), vptr(T))
    if st:
        raise ValueError(f"torus({nu}, {nv}) failed: {st}")
    return V, T


def torus_grid_for(n_tris: int, aspect: float = 2.0) -> tuple[int, int]:
    """(nu, nv) with nu / nv ~ aspect and 2 nu nv ~ n_tris."""
    nv = max(3, int(round((n_tris / (2.0 * aspect)) ** 0.5)))
    nu = max(3, int(round(n_tris / (2.0 * nv))))
    return nu, nv


def cameras(n: int, seed: int, r0: float, r1: float, target=(0.0, 0.0, 0.0)) -> np.ndarray:
    """n camera-to-world poses (column-major 4x4) looking at target."""
    cs = np.empty((n, 16), np.float32)
    t = np.asarray(target, np.float32)
    st = lib().j3dg_synth_cameras(n, seed, r0, r1, fptr(t), fptr(cs))
    if st:
        raise ValueError("cameras failed")
    return cs


def translation(x: float, y: float, z: float) -> np.ndarray:
    m = np.eye(4, dtype=np.float32)
    m[3, :3] = (x, y, z)  # column-major storage: translation in [12..14]
    return m.reshape(16).copy()


@dataclass
class Workload:
    name: str
    vertices: np.ndarray
    triangles: np.ndarray
    poses: np.ndarray           # (n_cameras, 16) camera-to-world
    width: int
    height: int
    vfov_deg: float = 60.0
    shadow: bool = True
    edges: bool = False
    extra: dict = field(default_factory=dict)


def config0(level: int = 6, width: int = 1024, height: int = 768) -> Workload:
    """Icosphere L6, camera at distance 3 on +z looking at the origin, 60 deg, shadow on."""
    V, T = icosphere(level, SEED_BASE + 0)
    return Workload("icosphere-L%d-%dx%d" % (level, width, height), V, T, translation(0.0, 0.0, 3.0)[None, :],
                    width, height)


def config1(n_cameras: int = 32, width: int = 1920, height: int = 1080, nu: int = 5300, nv: int = 2650) -> Workload:
    """Displaced torus (28.09M triangles at full size), cameras on radius 2.5..4 looking at the origin."""
    V, T = torus(nu, nv, seed=SEED_BASE + 1)
    poses = cameras(n_cameras, SEED_BASE + 1 + (1 << 32), 2.5, 4.0)
    return Workload("torus-%dx%d-%dtris-%dx%d-x%d" % (nu, nv, 2 * nu * nv, width, height, n_cameras), V, T, poses,
                    width, height)


@dataclass
class BatchWorkload:
    name: str
    meshes: list            # (V, T) per mesh
    poses: np.ndarray       # (n_meshes, n_cameras, 16)
    resolutions: list       # per (mesh, camera): (w, h)


def config2(n_meshes: int = 64, n_cameras: int = 16, t_min: float = 1e4, t_max: float = 2e6,
            seed: int = SEED_BASE + 2) -> BatchWorkload:
    """Batched frames: n_meshes meshes with triangle counts log-uniform in
    [t_min, t_max] (an icosphere level when one lands within 15 %, else a
    torus grid), n_cameras seeded cameras each, resolutions drawn from
    {256^2, 512^2, 768x512, 1024^2}. Draws: per mesh its count then kind; per
    frame its resolution index (numpy PCG64 seeded with `seed`)."""
    rng = np.random.default_rng(seed)
    meshes = []
    for i in range(n_meshes):
        t = float(np.exp(rng.uniform(np.log(t_min), np.log(t_max))))
        lvl = int(round(np.log(t / 20.0) / np.log(4.0)))
        if 0 <= lvl <= 9 and abs(20 * 4 ** lvl - t) <= 0.15 * t:
            meshes.append(icosphere(lvl, seed + 100 + i))
        else:
            nu, nv = torus_grid_for(int(t))
            meshes.append(torus(nu, nv, seed=seed + 100 + i))
    poses = np.stack([cameras(n_cameras, seed + 1000 + i, 2.5, 4.0) for i in range(n_meshes)])
    choices = [(256, 256), (512, 512), (768, 512), (1024, 1024)]
    res = [choices[int(rng.integers(0, 4))] for _ in range(n_meshes * n_cameras)]
    return BatchWorkload("batch-%dmeshes-x%dcams" % (n_meshes, n_cameras), meshes, poses, res)
