"""ctypes binding of the CPU oracle (oracle/_build/libj3doracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, always as the checker, never as the product.
Parity status of the oracle itself: "parity unpinned" (see j3d_oracle.cpp).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libj3doracle.so"

PIXEL_DTYPE = np.dtype([("mark", "u1"), ("r", "u1"), ("g", "u1"), ("b", "u1"), ("u", "<f4"), ("v", "<f4"),
                        ("depth", "<f4"), ("object_id", "<u4"), ("barycentric_u", "<f4"),
                        ("barycentric_v", "<f4"), ("db_id", "<u4")])
RAY_DTYPE = np.dtype([("orig", "<f4", 4), ("dir", "<f4", 4), ("t_near", "<f4"), ("t_far", "<f4")])
HIT_DTYPE = np.dtype([("found", "<u4"), ("distance", "<f4"), ("u", "<f4"), ("v", "<f4"), ("object_id", "<u4"),
                      ("two_level_index", "<u4")])
FLT_MAX = float(np.finfo(np.float32).max)


class Camera(C.Structure):
    _fields_ = [("focal_length", C.c_float), ("film_aperture_width_inch", C.c_float),
                ("film_aperture_height_inch", C.c_float), ("near_clipping_plane", C.c_float),
                ("far_clipping_plane", C.c_float), ("zoom", C.c_float), ("fit_film", C.c_int32)]


class Settings(C.Structure):
    _fields_ = [("one_bit", C.c_uint8), ("shadow", C.c_uint8), ("edges", C.c_uint8), ("wireframe", C.c_uint8),
                ("shading", C.c_uint8), ("textured", C.c_uint8), ("vertexcolors", C.c_uint8),
                ("reserved", C.c_uint8)]


class Instance(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("cs", C.c_float * 16), ("db_id", C.c_uint32), ("reserved", C.c_uint32)]


class View(C.Structure):
    _fields_ = [("coordinate_system", C.c_float * 16), ("coordinate_system_inv", C.c_float * 16),
                ("pivot", C.c_float * 3), ("diagonal", C.c_float), ("projection_inv", C.c_float * 16),
                ("near_clipping_plane", C.c_float)]


class Stats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64)]


_P, _I, _U, _F = C.c_void_p, C.c_int, C.c_uint32, C.c_float
_SIG = {
    "orc_make_default_camera": (None, [C.POINTER(Camera)]),
    "orc_render_pointclouds": (None, [_P, _P, _U, _U, _P, _P, _F, _U, _P, _P, _P, _P, _P, _I]),
    "orc_make_projection_matrix": (None, [C.POINTER(Camera), _I, _I, _P]),
    "orc_invert_projection_matrix": (None, [_P, _P]),
    "orc_invert_orthonormal": (None, [_P, _P]),
    "orc_matrix_vector_multiply": (None, [_P, _P, _P]),
    "orc_compute_bb": (None, [_P, _U, _P, _P]),
    "orc_compute_triangle_normals": (None, [_P, _P, _U, _P]),
    "orc_prepare_scene": (None, [_P, _P, _P, _U, _P, _P, _P]),
    "orc_unzoom": (None, [_P, _P, _F, _P, _P, _P]),
    "orc_mesh_build": (_P, [_P, _U, _P, _U, _U, _I, C.POINTER(C.c_double)]),
    "orc_mesh_free": (None, [_P]),
    "orc_mesh_node_count": (_U, [_P]),
    "orc_mesh_max_depth": (_U, [_P]),
    "orc_mesh_normals": (C.POINTER(C.c_float), [_P]),
    "orc_mesh_set_vertex_colors": (None, [_P, _P]),
    "orc_mesh_set_uv": (None, [_P, _P]),
    "orc_mesh_set_texture": (None, [_P, _P, _U, _U]),
    "orc_find_closest": (None, [C.POINTER(Instance), _U, _P, _U, _P, _I, _I, _I, C.POINTER(Stats)]),
    "orc_find_all": (_U, [_P, _P, _P, _U]),
    "orc_find_all_brute": (_U, [_P, _P, _P, _U]),
    "orc_get_world_position": (None, [_P, _P, _P, _P, _P]),
    "orc_voxelize": (C.c_uint64, [_P, _U, _P, _P, C.c_uint64]),
    "orc_fill_background": (None, [_P, _U, _U, _U, _U]),
    "orc_update_canvas": (None, [_P, _U, _U, _I, _I, _I, _I, C.POINTER(Instance), _U, C.POINTER(View),
                                 C.POINTER(Settings), _I, C.POINTER(Stats)]),
    "orc_canvas_to_image": (None, [_P, _U, _U, C.POINTER(View), C.POINTER(Settings), _P, _U, _U, _U, _P]),
    "orc_render_frame": (None, [_P, _P, _P, _U, _U, C.POINTER(Instance), _U, C.POINTER(View), C.POINTER(Settings),
                                _P, _U, _U, _U, _I, _P, C.POINTER(Stats)]),
    "orc_make_matcap": (None, [_I, _P, C.POINTER(_U)]),
    "orc_get_closest_vertex": (_U, [_P, _P, _P]),
}

_lib = None


def build() -> Path:
    """Compiles the oracle with its Makefile (g++, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        for k, (r, a) in _SIG.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _p(a: np.ndarray) -> int:
    assert a.flags.c_contiguous
    return a.ctypes.data


def threads(n: int | None = None) -> int:
    return n if n else (os.cpu_count() or 1)


# ----------------------------------------------------------------- camera

def make_default_camera() -> Camera:
    c = Camera()
    lib().orc_make_default_camera(C.byref(c))
    return c


def camera_with_focal(focal: float) -> Camera:
    c = make_default_camera()
    c.focal_length = focal
    return c


def make_projection_matrix(cam: Camera, w: int, h: int) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().orc_make_projection_matrix(C.byref(cam), w, h, _p(out))
    return out


def invert_projection_matrix(p: np.ndarray) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().orc_invert_projection_matrix(_p(np.ascontiguousarray(p, np.float32)), _p(out))
    return out


def invert_orthonormal(m: np.ndarray) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().orc_invert_orthonormal(_p(np.ascontiguousarray(m, np.float32).reshape(16)), _p(out))
    return out


def compute_bb(V: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    mn = np.zeros(3, np.float32)
    mx = np.zeros(3, np.float32)
    lib().orc_compute_bb(_p(V), V.shape[0], _p(mn), _p(mx))
    return mn, mx


def compute_triangle_normals(V: np.ndarray, T: np.ndarray) -> np.ndarray:
    out = np.zeros((T.shape[0], 3), np.float32)
    lib().orc_compute_triangle_normals(_p(V), _p(T), T.shape[0], _p(out))
    return out


def prepare_scene(bbs: list[tuple[np.ndarray, np.ndarray]], css: list[np.ndarray]):
    n = len(bbs)
    omin = np.ascontiguousarray(np.array([b[0] for b in bbs], np.float32).reshape(-1)) if n else np.zeros(3, np.float32)
    omax = np.ascontiguousarray(np.array([b[1] for b in bbs], np.float32).reshape(-1)) if n else np.zeros(3, np.float32)
    ocs = np.ascontiguousarray(np.array(css, np.float32).reshape(-1)) if n else np.zeros(16, np.float32)
    mn = np.zeros(3, np.float32)
    mx = np.zeros(3, np.float32)
    d = np.zeros(1, np.float32)
    lib().orc_prepare_scene(_p(omin), _p(omax), _p(ocs), n, _p(mn), _p(mx), _p(d))
    return mn, mx, np.float32(d[0])


def unzoom(mn: np.ndarray, mx: np.ndarray, diagonal: float):
    cs = np.zeros(16, np.float32)
    inv = np.zeros(16, np.float32)
    piv = np.zeros(3, np.float32)
    lib().orc_unzoom(_p(np.ascontiguousarray(mn, np.float32)), _p(np.ascontiguousarray(mx, np.float32)),
                     float(diagonal), _p(cs), _p(inv), _p(piv))
    return cs, inv, piv


def make_matcap(kind: int = 0) -> tuple[np.ndarray, int]:
    px = np.zeros((512, 512), np.uint32)
    cav = C.c_uint32()
    lib().orc_make_matcap(kind, _p(px), C.byref(cav))
    return px, int(cav.value)


def fill_background(w: int, h: int, top: int = 0xff000000, bottom: int = 0xff404040) -> np.ndarray:
    bg = np.zeros((h, w), np.uint32)
    lib().orc_fill_background(_p(bg), w, h, top, bottom)
    return bg


# ------------------------------------------------------------------ meshes

class Mesh:
    """scene_object + qbvh restated on the CPU (binned SAH, 4 wide)."""

    def __init__(self, V: np.ndarray, T: np.ndarray, leaf: int = 4, n_threads: int | None = None):
        self.V = np.ascontiguousarray(V, np.float32)
        self.T = np.ascontiguousarray(T, np.uint32)
        secs = C.c_double()
        self.h = lib().orc_mesh_build(_p(self.V), self.V.shape[0], _p(self.T), self.T.shape[0], leaf,
                                      threads(n_threads), C.byref(secs))
        self.build_seconds = secs.value
        self.min_bb, self.max_bb = compute_bb(self.V)
        self._keep = []

    def __del__(self):
        try:
            if self.h:
                lib().orc_mesh_free(self.h)
        except Exception:
            pass

    @property
    def n_nodes(self) -> int:
        return lib().orc_mesh_node_count(self.h)

    @property
    def max_depth(self) -> int:
        return lib().orc_mesh_max_depth(self.h)

    def normals(self) -> np.ndarray:
        p = lib().orc_mesh_normals(self.h)
        return np.ctypeslib.as_array(p, shape=(self.T.shape[0], 3)).copy()

    def set_vertex_colors(self, c: np.ndarray) -> None:
        c = np.ascontiguousarray(c, np.float32)
        self._keep.append(c)
        lib().orc_mesh_set_vertex_colors(self.h, _p(c))

    def set_uv(self, uv: np.ndarray) -> None:
        uv = np.ascontiguousarray(uv, np.float32)
        self._keep.append(uv)
        lib().orc_mesh_set_uv(self.h, _p(uv))

    def set_texture(self, tex: np.ndarray) -> None:
        tex = np.ascontiguousarray(tex, np.uint32)
        self._keep.append(tex)
        lib().orc_mesh_set_texture(self.h, _p(tex), tex.shape[1], tex.shape[0])


def instances(objs: list[tuple[Mesh, np.ndarray, int]]):
    arr = (Instance * max(1, len(objs)))()
    for i, (m, cs, db) in enumerate(objs):
        arr[i].mesh = m.h
        C.memmove(arr[i].cs, np.ascontiguousarray(cs, np.float32).ctypes.data, 64)
        arr[i].db_id = db
    return arr


def view(cs: np.ndarray, cs_inv: np.ndarray, pivot, diagonal: float, pinv: np.ndarray, near: float) -> View:
    v = View()
    C.memmove(v.coordinate_system, np.ascontiguousarray(cs, np.float32).ctypes.data, 64)
    C.memmove(v.coordinate_system_inv, np.ascontiguousarray(cs_inv, np.float32).ctypes.data, 64)
    C.memmove(v.pivot, np.ascontiguousarray(pivot, np.float32).ctypes.data, 12)
    v.diagonal = float(diagonal)
    C.memmove(v.projection_inv, np.ascontiguousarray(pinv, np.float32).ctypes.data, 64)
    v.near_clipping_plane = float(near)
    return v


def settings(one_bit=False, shadow=False, edges=True, wireframe=False, shading=True, textured=True,
             vertexcolors=True) -> Settings:
    return Settings(int(one_bit), int(shadow), int(edges), int(wireframe), int(shading), int(textured),
                    int(vertexcolors), 0)


def fresh_pixels(w: int, h: int) -> np.ndarray:
    """A canvas G-buffer after canvas::resize (pixel.h:13, canvas.cpp:126-130)."""
    p = np.zeros((h, w), PIXEL_DTYPE)
    p["object_id"] = 0xFFFFFFFF
    return p


def find_closest(objs, rays: np.ndarray, brute: bool = False, any_hit: bool = False,
                 n_threads: int | None = None) -> tuple[np.ndarray, Stats]:
    inst = instances(objs)
    hits = np.zeros(len(rays), HIT_DTYPE)
    st = Stats()
    lib().orc_find_closest(inst, len(objs), _p(rays), len(rays), _p(hits), 1 if brute else 0, 1 if any_hit else 0,
                           threads(n_threads), C.byref(st))
    return hits, st


def find_all(mesh: Mesh, ray: np.ndarray, cap: int = 4096, brute: bool = False) -> np.ndarray:
    """find_all_triangles (vox.cpp:333): hits sorted by (t, id)."""
    hits = np.zeros(cap, HIT_DTYPE)
    r = np.ascontiguousarray(np.asarray(ray).reshape(1), RAY_DTYPE)
    f = lib().orc_find_all_brute if brute else lib().orc_find_all
    n = f(mesh.h, _p(r), _p(hits), cap)
    return hits[:min(n, cap)]


def get_world_position(p: np.ndarray, V: np.ndarray, T: np.ndarray, cs: np.ndarray) -> np.ndarray:
    rec = np.ascontiguousarray(np.asarray(p).reshape(1), PIXEL_DTYPE)
    out = np.zeros(3, np.float32)
    lib().orc_get_world_position(_p(rec), _p(V), _p(T), _p(np.ascontiguousarray(cs, np.float32)), _p(out))
    return out


def voxelize(mesh: Mesh, max_dim: int) -> np.ndarray:
    """The voxel grid of write_vox (vox.cpp:284-380) as uint8[z, y, x]."""
    dims = np.zeros(3, np.uint32)
    total = lib().orc_voxelize(mesh.h, max_dim, _p(dims), None, 0)
    out = np.zeros(total, np.uint8)
    lib().orc_voxelize(mesh.h, max_dim, _p(dims), _p(out), total)
    return out.reshape(int(dims[2]), int(dims[1]), int(dims[0]))


def update_canvas(pix: np.ndarray, objs, v: View, s: Settings, rect=None, n_threads: int | None = None) -> Stats:
    h, w = pix.shape
    x0, y0, x1, y1 = rect if rect else (0, 0, w - 1, h - 1)
    inst = instances(objs)
    st = Stats()
    lib().orc_update_canvas(_p(pix), w, h, x0, y0, x1, y1, inst, len(objs), C.byref(v), C.byref(s),
                            threads(n_threads), C.byref(st))
    return st


def canvas_to_image(pix: np.ndarray, im: np.ndarray, v: View, s: Settings, matcap: np.ndarray, cavity: int) -> None:
    h, w = pix.shape
    lib().orc_canvas_to_image(_p(pix), w, h, C.byref(v), C.byref(s), _p(matcap), matcap.shape[1], matcap.shape[0],
                              cavity, _p(im))


def render_frame(pix: np.ndarray, im: np.ndarray, background: np.ndarray | None, objs, v: View, s: Settings,
                 matcap: np.ndarray, cavity: int, n_threads: int | None = None) -> tuple[float, float, Stats]:
    h, w = pix.shape
    inst = instances(objs)
    secs = (C.c_double * 2)()
    st = Stats()
    lib().orc_render_frame(_p(pix), _p(im), _p(background) if background is not None else None, w, h, inst,
                           len(objs), C.byref(v), C.byref(s), _p(matcap), matcap.shape[1], matcap.shape[0], cavity,
                           threads(n_threads), secs, C.byref(st))
    return secs[0], secs[1], st


def get_closest_vertex(p: np.ndarray, V: np.ndarray, T: np.ndarray) -> int:
    rec = np.ascontiguousarray(np.asarray(p).reshape(1), PIXEL_DTYPE)
    return lib().orc_get_closest_vertex(_p(rec), _p(V), _p(T))


def primary_rays(w: int, h: int, cs: np.ndarray, pinv: np.ndarray, near: float, t_near: float) -> np.ndarray:
    """Rays of canvas.cpp:773-782 computed with the oracle's mat x vec (for ray-batch tests)."""
    M = lib().orc_matrix_vector_multiply
    origin = np.zeros(4, np.float32)
    M(_p(np.ascontiguousarray(cs, np.float32)), _p(np.array([0, 0, 0, 1], np.float32)), _p(origin))
    rays = np.zeros(w * h, RAY_DTYPE)
    xs = np.arange(w, dtype=np.float32)
    ys = np.arange(h, dtype=np.float32)
    sx = np.float32(2) * ((xs + np.float32(0.5)) / np.float32(w)) - np.float32(1)
    sy = np.float32(2) * ((ys + np.float32(0.5)) / np.float32(h)) - np.float32(1)
    tmp = np.zeros(4, np.float32)
    out = np.zeros(4, np.float32)
    k = 0
    for y in range(h):
        for x in range(w):
            s = np.array([sx[x], sy[y], near, 1.0], np.float32)
            M(_p(np.ascontiguousarray(pinv, np.float32)), _p(s), _p(tmp))
            tmp[3] = 0
            M(_p(np.ascontiguousarray(cs, np.float32)), _p(tmp), _p(out))
            rays[k]["orig"] = origin
            rays[k]["dir"] = out
            rays[k]["t_near"] = t_near
            rays[k]["t_far"] = FLT_MAX
            k += 1
    return rays


def render_pointclouds(pix: np.ndarray, im: np.ndarray, projection: np.ndarray, cs_inv: np.ndarray,
                       near_plane: float, clouds, one_bit: bool = False) -> None:
    """canvas::render_pointclouds_on_image (canvas.cpp:952-1030) in place on
    the G-buffer `pix` and image `im`. clouds: [(vertices (n,3) f32, colors
    (n,) u32 or None, cs (16,) f32, db_id)]."""
    h, w = pix.shape
    k = len(clouds)
    keep = []
    vps = (C.c_void_p * max(1, k))()
    cps = (C.c_void_p * max(1, k))()
    counts = np.zeros(max(1, k), np.uint64)
    css = np.zeros((max(1, k), 16), np.float32)
    dbs = np.zeros(max(1, k), np.uint32)
    for i, (V, col, cs, db) in enumerate(clouds):
        V = np.ascontiguousarray(V, np.float32)
        keep.append(V)
        vps[i] = V.ctypes.data
        if col is not None:
            col = np.ascontiguousarray(col, np.uint32)
            keep.append(col)
            cps[i] = col.ctypes.data
        counts[i] = len(V)
        css[i] = np.asarray(cs, np.float32).reshape(16)
        dbs[i] = db
    lib().orc_render_pointclouds(_p(pix), _p(im), w, h, _p(np.ascontiguousarray(projection, np.float32)),
                                 _p(np.ascontiguousarray(cs_inv, np.float32)), float(near_plane), k,
                                 C.cast(vps, C.c_void_p), _p(counts), C.cast(cps, C.c_void_p), _p(css), _p(dbs),
                                 int(one_bit))

