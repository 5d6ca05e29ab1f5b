"""Seeded synthetic workloads restated in numpy for the oracle side.

TEST INFRASTRUCTURE ONLY: used by tests/, tests/golden/ generators and
bench.py's reference (CPU) arm, so that the CPU path never loads the product
library. The product generates the same inputs in its own host code; a CPU
test asserts both give the same bytes.

The workloads themselves are the benchmark's stated constructions:
  icosphere  subdivided icosahedron, radius per vertex direction d
             1 + amp * sum_{k=1..8} a_k sin(f_k (d . u_k) + phi_k),
             a_k ~ U(0,1), f_k ~ U(2,12), u_k uniform unit, phi_k ~ U(0, 2 pi)
  torus      R = 1, r = 0.35 on an nu x nv periodic grid, two triangles per
             quad, radial displacement amp * sum of 16 sinusoids in (u, v)
             with integer frequencies (periodic on the grid)
  cameras    direction uniform on the sphere, radius ~ U(r0, r1), looking at
             the target, y up (z up near the poles)

Determinism: splitmix64 -> PCG32 (O'Neill 2014, XSH RR) draws, 24-bit
uniforms, rejection-sampled directions and a sine built only from IEEE
+ - * / and floor (Cody-Waite reduction by 2 pi, odd Taylor polynomial to
x^23), all in float64 with every operation rounded where it is written, so
x86 and Arm hosts and the product's C++ give the same bytes.
"""
from __future__ import annotations

import numpy as np

SEED_BASE = 0x6A3D0000
M64 = (1 << 64) - 1

PI = 3.141592653589793116
PI_LO = 1.2246467991473532e-16
TWO_PI = 6.283185307179586232
TWO_PI_LO = 2.4492935982947064e-16
_SIN_C = [1.0, -1.0 / 6.0, 1.0 / 120.0, -1.0 / 5040.0, 1.0 / 362880.0, -1.0 / 39916800.0, 1.0 / 6227020800.0,
          -1.0 / 1307674368000.0, 1.0 / 355687428096000.0, -1.0 / 121645100408832000.0,
          1.0 / 51090942171709440000.0, -1.0 / 25852016738884976640000.0]


def det_sin(x):
    """sin in float64 from IEEE basic operations only (error < 1e-16)."""
    x = np.asarray(x, np.float64)
    k = np.floor(x / TWO_PI + 0.5)
    r = (x - k * TWO_PI) - k * TWO_PI_LO
    r = np.where(r > 0.5 * PI, (PI - r) + PI_LO, np.where(r < -0.5 * PI, (-PI - r) - PI_LO, r))
    r2 = r * r
    p = np.full_like(r, _SIN_C[11])
    for j in range(10, -1, -1):
        p = p * r2 + _SIN_C[j]
    return r * p


def _splitmix64(s: int) -> tuple[int, int]:
    s = (s + 0x9E3779B97F4A7C15) & M64
    z = s
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return s, z ^ (z >> 31)


class Pcg32:
    """PCG32 XSH RR, state and stream seeded from splitmix64(seed)."""

    def __init__(self, seed: int):
        s, init_state = _splitmix64(seed & M64)
        s, init_seq = _splitmix64(s)
        self.inc = ((init_seq << 1) | 1) & M64
        self.state = 0
        self.next()
        self.state = (self.state + init_state) & M64
        self.next()

    def next(self) -> int:
        old = self.state
        self.state = (old * 6364136223846793005 + self.inc) & M64
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF

    def u01(self) -> float:
        return float(self.next() >> 8) * (1.0 / 16777216.0)

    def uniform(self, a: float, b: float) -> float:
        return a + (b - a) * self.u01()

    def unit3(self) -> tuple[float, float, float]:
        while True:
            x = self.uniform(-1.0, 1.0)
            y = self.uniform(-1.0, 1.0)
            z = self.uniform(-1.0, 1.0)
            n2 = x * x + y * y + z * z
            if 1e-6 < n2 <= 1.0:
                n = float(np.sqrt(n2))
                return x / n, y / n, z / n


def focal_for_vfov(vfov_deg: float, film_h_inch: float = 0.768) -> float:
    """Focal length (mm) giving vfov_deg over the film gate's height (Overscan fit)."""
    f32 = lambda x: float(np.float32(x))  # noqa: E731
    half = 0.5 * f32(vfov_deg) * (PI / 180.0)
    t = float(det_sin(half)) / float(det_sin(half + 0.5 * PI))
    return f32(((f32(film_h_inch) * 25.4) * 0.5) / t)


_ICO_P = [-1, "p", 0, 1, "p", 0, -1, "-p", 0, 1, "-p", 0, 0, -1, "p", 0, 1, "p",
          0, -1, "-p", 0, 1, "-p", "p", 0, -1, "p", 0, 1, "-p", 0, -1, "-p", 0, 1]
_ICO_F = [0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1, 8,
          3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1]


def _normalize_rows(P: np.ndarray) -> np.ndarray:
    n = np.sqrt(P[:, 0] * P[:, 0] + P[:, 1] * P[:, 1] + P[:, 2] * P[:, 2])
    return P / n[:, None]


def icosphere(level: int = 6, seed: int = SEED_BASE, amp: float = 0.05) -> tuple[np.ndarray, np.ndarray]:
    """Displaced icosphere: 20 * 4^level triangles, 10 * 4^level + 2 vertices.
    Each subdivision visits the faces in order and numbers a new edge midpoint
    when its edge is first met (ab, bc, ca per face); a face (a, b, c) becomes
    (a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)."""
    if not 0 <= level <= 11:
        raise ValueError(f"icosphere level {level} out of range")
    p = (1.0 + np.sqrt(5.0)) * 0.5
    P = np.array([p if v == "p" else -p if v == "-p" else float(v) for v in _ICO_P], np.float64).reshape(-1, 3)
    P = _normalize_rows(P)
    F = np.array(_ICO_F, np.int64).reshape(-1, 3)
    for _ in range(level):
        a, b, c = F[:, 0], F[:, 1], F[:, 2]
        e0 = np.stack([a, b, c], 1).reshape(-1)   # edge starts in visiting order: ab, bc, ca
        e1 = np.stack([b, c, a], 1).reshape(-1)
        key = np.minimum(e0, e1) << 32 | np.maximum(e0, e1)
        uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
        order = np.argsort(first, kind="stable")          # unique edges in order of first visit
        new_id = np.empty(len(uniq), np.int64)
        new_id[order] = len(P) + np.arange(len(uniq))
        mids = new_id[inv].reshape(-1, 3)                   # ab, bc, ca per face
        ea, eb = e0[first[order]], e1[first[order]]
        P = np.concatenate([P, _normalize_rows(P[ea] + P[eb])])
        ab, bc, ca = mids[:, 0], mids[:, 1], mids[:, 2]
        F = np.stack([a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca], 1).reshape(-1, 3)
    rng = Pcg32(seed)
    terms = []
    for _ in range(8):
        ak = rng.u01()
        fk = rng.uniform(2.0, 12.0)
        uk = rng.unit3()
        phk = rng.uniform(0.0, TWO_PI)
        terms.append((ak, fk, uk, phk))
    s = np.zeros(len(P))
    for ak, fk, uk, phk in terms:
        dot = P[:, 0] * uk[0] + P[:, 1] * uk[1] + P[:, 2] * uk[2]
        s = s + ak * det_sin(fk * dot + phk)
    rad = 1.0 + float(np.float32(amp)) * s
    V = (rad[:, None] * P).astype(np.float32)
    return V, F.astype(np.uint32)


def torus(nu: int = 5300, nv: int = 2650, R: float = 1.0, r: float = 0.35, seed: int = SEED_BASE + 1,
          amp: float = 0.02) -> tuple[np.ndarray, np.ndarray]:
    """Displaced torus on an nu x nv periodic grid: vertex (i, j) at
    index i nv + j; quad (i, j) gives triangles (q0, q1, q2), (q0, q2, q3)
    with q0 = (i, j), q1 = (i+1, j), q2 = (i+1, j+1), q3 = (i, j+1)."""
    if nu < 3 or nv < 3:
        raise ValueError("torus grid below 3 x 3")
    K = 16
    rng = Pcg32(seed)
    a, m, n, ps = [], [], [], []
    for _ in range(K):
        a.append(rng.u01())
        m.append(1 + rng.next() % 24)
        n.append(1 + rng.next() % 12)
        ps.append(rng.uniform(0.0, TWO_PI))
    th = TWO_PI * np.arange(nu, dtype=np.float64) / float(nu)
    ph = TWO_PI * np.arange(nv, dtype=np.float64) / float(nv)
    sth, cth = det_sin(th), det_sin(th + 0.5 * PI)
    sph, cph = det_sin(ph), det_sin(ph + 0.5 * PI)
    s = np.zeros((nu, nv))
    for k in range(K):
        A = float(m[k]) * th
        B = float(n[k]) * ph + ps[k]
        sA, cA = det_sin(A), det_sin(A + 0.5 * PI)
        sB, cB = det_sin(B), det_sin(B + 0.5 * PI)
        term = sA[:, None] * cB[None, :]
        term += cA[:, None] * sB[None, :]
        term *= a[k]
        s += term
        del term
    rr = s
    rr *= float(np.float32(amp))
    rr += float(np.float32(r))
    V = np.empty((nu, nv, 3), np.float32)
    V[:, :, 1] = rr * sph[None, :]
    ring = rr
    ring *= cph[None, :]
    ring += float(np.float32(R))
    V[:, :, 0] = ring * cth[:, None]
    V[:, :, 2] = ring * sth[:, None]
    del rr, ring, s
    i = np.arange(nu, dtype=np.uint32)[:, None]
    j = np.arange(nv, dtype=np.uint32)[None, :]
    i1 = np.where(i + 1 == nu, 0, i + 1).astype(np.uint32)
    j1 = np.where(j + 1 == nv, 0, j + 1).astype(np.uint32)
    q0 = i * nv + j
    q1 = i1 * nv + j
    q2 = i1 * nv + j1
    q3 = i * nv + j1
    T = np.empty((nu, nv, 6), np.uint32)
    T[:, :, 0] = q0
    T[:, :, 1] = q1
    T[:, :, 2] = q2
    T[:, :, 3] = q0
    T[:, :, 4] = q2
    T[:, :, 5] = q3
    return V.reshape(-1, 3), T.reshape(-1, 3)


def cameras(n: int, seed: int, r0: float, r1: float, target=(0.0, 0.0, 0.0)) -> np.ndarray:
    """n camera-to-world poses (column-major 4x4, float32) looking at target:
    column 0 right, 1 up, 2 back (= the drawn direction), 3 the position."""
    f32 = lambda x: float(np.float32(x))  # noqa: E731
    rng = Pcg32(seed)
    out = np.zeros((n, 16), np.float32)
    tg = [f32(t) for t in target]
    for c in range(n):
        d = rng.unit3()
        rad = rng.uniform(f32(r0), f32(r1))
        up0 = (0.0, 0.0, 1.0) if abs(d[1]) > 0.99 else (0.0, 1.0, 0.0)
        rt = [up0[1] * d[2] - up0[2] * d[1], up0[2] * d[0] - up0[0] * d[2], up0[0] * d[1] - up0[1] * d[0]]
        rn = float(np.sqrt(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2]))
        rt = [x / rn for x in rt]
        up = [d[1] * rt[2] - d[2] * rt[1], d[2] * rt[0] - d[0] * rt[2], d[0] * rt[1] - d[1] * rt[0]]
        M = out[c]
        for k in range(3):
            M[k] = rt[k]
            M[4 + k] = up[k]
            M[8 + k] = d[k]
            M[12 + k] = tg[k] + rad * d[k]
        M[15] = 1.0
    return out


def translation(x: float, y: float, z: float) -> np.ndarray:
    m = np.eye(4, dtype=np.float32)
    m[3, :3] = (x, y, z)
    return m.reshape(16).copy()


def config0():
    """Icosphere L6 at 1024x768, camera at distance 3 on +z: (V, T, poses, w, h)."""
    V, T = icosphere(6, SEED_BASE + 0)
    return V, T, translation(0.0, 0.0, 3.0)[None, :], 1024, 768


def config1(n_cameras: int = 32, width: int = 1920, height: int = 1080, nu: int = 5300, nv: int = 2650):
    """Displaced torus (28.09M triangles at full size) and its cameras: (V, T, poses, w, h)."""
    V, T = torus(nu, nv, seed=SEED_BASE + 1)
    poses = cameras(n_cameras, SEED_BASE + 1 + (1 << 32), 2.5, 4.0)
    return V, T, poses, width, height
