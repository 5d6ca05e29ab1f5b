"""Host-side mirror of j3d's scene / canvas / camera / matcap API over the C-ABI.

Same names, argument meaning and error behaviour as the reference's classes:
  add_object (scene.cpp:8-38)        -> Scene.add_object (BVH built on the GPU)
  prepare_scene / unzoom (scene.cpp:50-110)
  canvas(w, h), resize, update_settings, set_background_color,
  update_canvas, render_scene, canvas_to_image, get_pixels, get_image
                                     (canvas.h:27-101)
  view::render_scene (view.cpp:421-430) -> Canvas.render_frame
Calls that the C-ABI rejects raise J3dgError.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _ffi
from ._ffi import (HIT_DTYPE, PIXEL_DTYPE, RAY_DTYPE, BuildOpts, Camera, CanvasSettings, Instance, J3dgError,
                   MeshInfo, fptr, lib, vptr)

IDENTITY = np.eye(4, dtype=np.float32).reshape(-1)  # column-major == row-major for identity


def _check(ctx_handle, status: int) -> None:
    if status != _ffi.J3DG_OK:
        msg = lib().j3dg_last_error(ctx_handle) if ctx_handle else b""
        raise J3dgError(status, (msg or b"").decode())


class Context:
    """One device, one CUDA stream (no reference counterpart)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        st = lib().j3dg_ctx_create(device, C.byref(h))
        if st != _ffi.J3DG_OK:
            raise J3dgError(st, f"j3dg_ctx_create(device={device})")
        self.h = h
        self._objs: dict = {}  # id -> weak reference, in creation order

    def _own(self, obj) -> None:
        """Registers an object made from this context; close() closes it first.
        The entry goes away with the object (a server makes many canvases)."""
        objs, key = self._objs, id(obj)
        objs[key] = weakref.ref(obj, lambda _r: objs.pop(key, None))

    def close(self) -> None:
        """Closes the meshes, canvases, ... made from this context (newest
        first), then the context itself."""
        if self.h:
            for r in reversed(list(self._objs.values())):
                o = r()
                if o is not None:
                    o.close()
            self._objs.clear()
            st = lib().j3dg_ctx_destroy(self.h)
            if st != _ffi.J3DG_OK:
                raise J3dgError(st, lib().j3dg_last_error(self.h).decode())
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self) -> None:
        _check(self.h, lib().j3dg_ctx_synchronize(self.h))

    def device_status(self) -> int:
        s = C.c_uint32()
        _check(self.h, lib().j3dg_ctx_device_status(self.h, C.byref(s)))
        return s.value

    def stream(self) -> int:
        return lib().j3dg_ctx_stream(self.h) or 0

    def set_counting(self, on: bool) -> None:
        _check(self.h, lib().j3dg_ctx_set_counting(self.h, 1 if on else 0))

    def set_batch_block(self, threads: int) -> None:
        _check(self.h, lib().j3dg_ctx_set_batch_block(self.h, threads))

    def set_primary_mode(self, mode: int) -> None:
        """How canvas frames find primary hits: PRIMARY_AUTO (default),
        PRIMARY_TRACE (BVH walk per pixel) or PRIMARY_RASTER (projected
        triangle boxes, the traversal's own ray / triangle test per covered
        pixel); the hits are the same."""
        _check(self.h, lib().j3dg_ctx_set_primary_mode(self.h, mode))

    def set_top_level(self, on: bool) -> None:
        """Walk scenes of several objects through a per-frame top-level BVH
        (default) or object after object (for measurement)."""
        _check(self.h, lib().j3dg_ctx_set_top_level(self.h, 1 if on else 0))

    def set_frame_overlap(self, on: bool) -> None:
        """Let a canvas's traced frame start while its previous frame
        finishes (default; the same results) or run frames strictly one
        after the other (for measurement)."""
        _check(self.h, lib().j3dg_ctx_set_frame_overlap(self.h, 1 if on else 0))

    def memory(self) -> dict:
        """Device free / total bytes and the reserved / used bytes of the
        context's canvas pool and of the device's default pool."""
        out = (C.c_uint64 * 6)()
        _check(self.h, lib().j3dg_ctx_memory(self.h, out))
        keys = ("device_free", "device_total", "canvas_pool_reserved", "canvas_pool_used",
                "default_pool_reserved", "default_pool_used")
        return {k: int(v) for k, v in zip(keys, out)}

    def read_counters(self, reset: bool = True) -> tuple[int, int]:
        out = (C.c_uint64 * 2)()
        _check(self.h, lib().j3dg_ctx_read_counters(self.h, out, 1 if reset else 0))
        return int(out[0]), int(out[1])


class Mesh:
    """scene_object's mesh + qbvh (scene.h:10-25), resident on the device."""

    BUILDERS = {"ploc": 0, "lbvh": 1}
    WIDTHS = {2: 0x2, 4: 0, 8: 0x4}  # J3DG_BUILD_WIDTH2 / (default) / J3DG_BUILD_WIDTH8
    REBUILDABLE = 0x8  # J3DG_BUILD_REBUILDABLE

    def __init__(self, ctx: Context, vertices, triangles, leaf_size: int = 2, build: str = "ploc", width: int = 4,
                 rebuildable: bool = False):
        """build: "ploc" (binned-SAH top levels over surface-area
        clustering, the default: fewer node visits per ray) or "lbvh" (Morton
        splits, 4-wide only, about a third of the build time);
        width: children per BVH node, 2, 4 (default) or 8; rebuildable: keep
        what a Batch(rebuild=True) rebuilds the BVH from, inside its graph."""
        self.ctx = ctx
        nv = int(vertices.shape[0]) if vertices.ndim > 1 else int(vertices.size // 3)
        nt = int(triangles.shape[0]) if triangles.ndim > 1 else int(triangles.size // 3)
        h = C.c_void_p()
        opts = BuildOpts(leaf_size, Mesh.BUILDERS[build] | Mesh.WIDTHS[width] | (Mesh.REBUILDABLE if rebuildable else 0))
        _check(ctx.h, lib().j3dg_mesh_build(ctx.h, vptr(vertices), nv, vptr(triangles), nt, C.byref(opts),
                                            C.byref(h)))
        self.h = h
        ctx._own(self)

    def close(self) -> None:
        if self.h:
            lib().j3dg_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> MeshInfo:
        i = MeshInfo()
        _check(self.ctx.h, lib().j3dg_mesh_get_info(self.h, C.byref(i)))
        return i

    def nodes(self) -> np.ndarray:
        """The BVH node array (n_nodes x 4 * width float32 words: planes
        [6][W], refs [W], padding) as host bytes."""
        i = self.info()
        words = {2: 16, 4: 32, 8: 64}[i.width]
        out = np.empty((i.n_nodes, words), np.float32)
        _check(self.ctx.h, lib().j3dg_mesh_get_nodes(self.h, vptr(out), out.nbytes))
        return out

    def triangle_normals(self) -> np.ndarray:
        i = self.info()
        out = np.empty((i.n_triangles, 3), np.float32)
        _check(self.ctx.h, lib().j3dg_mesh_get_triangle_normals(self.h, vptr(out)))
        return out

    def set_vertex_colors(self, colors) -> None:
        _check(self.ctx.h, lib().j3dg_mesh_set_vertex_colors(self.h, vptr(colors)))

    def set_uv(self, uv) -> None:
        _check(self.ctx.h, lib().j3dg_mesh_set_uv(self.h, vptr(uv)))

    def set_texture(self, tex: np.ndarray) -> None:
        h, w = tex.shape
        _check(self.ctx.h, lib().j3dg_mesh_set_texture(self.h, vptr(tex), w, h))


class Geometry:
    """Decoded mesh / point-cloud file resident on the device: the reader
    dispatch of read_from_file (mesh.cpp:76-176, pc.cpp:32-110)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.h = handle
        ctx._own(self)
        i = _ffi.GeometryInfo()
        _check(ctx.h, lib().j3dg_geometry_get_info(self.h, C.byref(i)))
        self.info = i

    @classmethod
    def read_file(cls, ctx: Context, path, fmt: str = "auto") -> "Geometry":
        h = C.c_void_p()
        _check(ctx.h, lib().j3dg_geometry_read_file(ctx.h, str(path).encode(), _ffi.FORMATS[fmt], C.byref(h)))
        return cls(ctx, h)

    @classmethod
    def read_memory(cls, ctx: Context, data: bytes, fmt: str = "auto") -> "Geometry":
        buf = np.frombuffer(data, np.uint8) if len(data) else np.zeros(1, np.uint8)
        h = C.c_void_p()
        _check(ctx.h, lib().j3dg_geometry_read_memory(ctx.h, buf.ctypes.data, len(data), _ffi.FORMATS[fmt],
                                                      C.byref(h)))
        return cls(ctx, h)

    def arrays(self) -> dict:
        """Host copies: vertices (V,3), triangles (T,3), and colors (V,),
        normals (V,3), uv (T,6) when present."""
        i = self.info
        out = {"vertices": np.empty((i.n_vertices, 3), np.float32),
               "triangles": np.empty((i.n_triangles, 3), np.uint32)}
        if i.has_colors:
            out["colors"] = np.empty(i.n_vertices, np.uint32)
        if i.has_normals:
            out["normals"] = np.empty((i.n_vertices, 3), np.float32)
        if i.has_uv:
            out["uv"] = np.empty((i.n_triangles, 6), np.float32)
        _check(self.ctx.h, lib().j3dg_geometry_get_arrays(
            self.h, vptr(out["vertices"]), vptr(out["triangles"]), vptr(out.get("colors")),
            vptr(out.get("normals")), vptr(out.get("uv"))))
        return out

    def close(self) -> None:
        if self.h:
            lib().j3dg_geometry_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PointCloud:
    """pc (pc.h:23-31): points and optional packed RGBA8 colours on the device."""

    def __init__(self, ctx: Context, vertices=None, colors=None, geometry: "Geometry | None" = None):
        self.ctx = ctx
        h = C.c_void_p()
        if geometry is not None:
            _check(ctx.h, lib().j3dg_pointcloud_from_geometry(ctx.h, geometry.h, C.byref(h)))
        else:
            n = int(vertices.shape[0]) if vertices.ndim > 1 else int(vertices.size // 3)
            _check(ctx.h, lib().j3dg_pointcloud_create(ctx.h, vptr(vertices), n, vptr(colors), C.byref(h)))
        self.h = h
        ctx._own(self)

    def bounds(self) -> tuple[np.ndarray, np.ndarray]:
        mn = np.zeros(3, np.float32)
        mx = np.zeros(3, np.float32)
        _check(self.ctx.h, lib().j3dg_pointcloud_get_bounds(self.h, fptr(mn), fptr(mx)))
        return mn, mx

    def close(self) -> None:
        if self.h:
            lib().j3dg_pointcloud_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ScenePointCloud:
    """scene_pointcloud (scene.h:27-38)."""

    def __init__(self, pc: PointCloud, cs=None, db_id: int = 2):
        self.pointcloud = pc
        self.cs = np.ascontiguousarray(IDENTITY if cs is None else np.asarray(cs, np.float32).reshape(16))
        self.db_id = db_id


def build_meshes(ctx: Context, meshes, leaf_sizes=None, width: int = 4, build: str = "ploc",
                 max_concurrent: int = 8, rebuildable: bool = False) -> list:
    """Many meshes built at once (j3dg_mesh_build_many): [(vertices,
    triangles)] -> [Mesh], up to max_concurrent builds in flight on their
    own streams. leaf_sizes: one per mesh, or None for 2; rebuildable: as
    for Mesh."""
    n = len(meshes)
    srcs = (_ffi.MeshSource * max(1, n))()
    keep = []
    for i, (V, T) in enumerate(meshes):
        V = np.ascontiguousarray(V, np.float32)
        T = np.ascontiguousarray(T, np.uint32)
        keep += [V, T]
        srcs[i].vertices = V.ctypes.data
        srcs[i].n_vertices = int(V.size // 3)
        srcs[i].triangles = T.ctypes.data
        srcs[i].n_triangles = int(T.size // 3)
    opts = (BuildOpts * max(1, n))()
    for i in range(n):
        opts[i] = BuildOpts(int(leaf_sizes[i]) if leaf_sizes is not None else 2,
                            Mesh.BUILDERS[build] | Mesh.WIDTHS[width] | (Mesh.REBUILDABLE if rebuildable else 0))
    hs = (C.c_void_p * max(1, n))()
    _check(ctx.h, lib().j3dg_mesh_build_many(ctx.h, n, C.cast(srcs, C.c_void_p), C.cast(opts, C.c_void_p),
                                             max_concurrent, C.cast(hs, C.c_void_p)))
    out = []
    for i in range(n):
        m = Mesh.__new__(Mesh)
        m.ctx = ctx
        m.h = C.c_void_p(hs[i])
        ctx._own(m)
        out.append(m)
    del keep
    return out


def mesh_from_geometry(ctx: Context, geom: Geometry, leaf_size: int = 2, build: str = "ploc",
                       width: int = 4) -> Mesh:
    """add_object's mesh built straight from device-resident geometry."""
    m = Mesh.__new__(Mesh)
    m.ctx = ctx
    h = C.c_void_p()
    opts = BuildOpts(leaf_size, Mesh.BUILDERS[build] | Mesh.WIDTHS[width])
    _check(ctx.h, lib().j3dg_mesh_build_geometry(ctx.h, geom.h, C.byref(opts), C.byref(h)))
    m.h = h
    ctx._own(m)
    return m


class SceneObject:
    def __init__(self, mesh: Mesh, cs=None, db_id: int = 1):
        self.mesh = mesh
        self.cs = np.ascontiguousarray(IDENTITY if cs is None else np.asarray(cs, np.float32).reshape(16))
        self.db_id = db_id


class Scene:
    """scene (scene.h:40-51): objects, coordinate_system(+inv), pivot, bbox, diagonal."""

    def __init__(self):
        self.objects: list[SceneObject] = []
        self.pointclouds: list[ScenePointCloud] = []
        self.coordinate_system = IDENTITY.copy()
        self.coordinate_system_inv = IDENTITY.copy()
        self.pivot = np.zeros(3, np.float32)
        self.min_bb = np.zeros(3, np.float32)
        self.max_bb = np.zeros(3, np.float32)
        self.diagonal = np.float32(0)

    def add_pointcloud(self, pc: PointCloud, cs=None, db_id: int = 2) -> ScenePointCloud:
        # scene.cpp:27-36
        o = ScenePointCloud(pc, cs, db_id)
        self.pointclouds.append(o)
        return o

    def _pc_instances(self):
        arr = (_ffi.PointCloudInstance * max(1, len(self.pointclouds)))()
        for i, o in enumerate(self.pointclouds):
            arr[i].pointcloud = o.pointcloud.h
            C.memmove(arr[i].cs, o.cs.ctypes.data, 64)
            arr[i].db_id = o.db_id
        return arr

    def add_object(self, mesh: Mesh, cs=None, db_id: int = 1) -> SceneObject:
        # scene.cpp:8-38 (the BVH was built when the Mesh was made)
        o = SceneObject(mesh, cs, db_id)
        self.objects.append(o)
        return o

    def remove_object(self, db_id: int) -> None:
        # scene.cpp:40-48
        for i, o in enumerate(self.objects):
            if o.db_id == db_id:
                del self.objects[i]
                break
        for i, o in enumerate(self.pointclouds):
            if o.db_id == db_id:
                del self.pointclouds[i]
                break

    def _instances(self):
        arr = (Instance * max(1, len(self.objects)))()
        for i, o in enumerate(self.objects):
            arr[i].mesh = o.mesh.h
            C.memmove(arr[i].cs, o.cs.ctypes.data, 64)
            arr[i].db_id = o.db_id
        return arr

    def prepare_scene(self) -> None:
        # scene.cpp:50-89
        inst = self._instances()
        mn = np.zeros(3, np.float32)
        mx = np.zeros(3, np.float32)
        d = np.zeros(1, np.float32)
        ctx = self.objects[0].mesh.ctx.h if self.objects else None
        if self.pointclouds:
            _check(ctx, lib().j3dg_prepare_scene_pointclouds(inst, len(self.objects), self._pc_instances(),
                                                             len(self.pointclouds), fptr(mn), fptr(mx), fptr(d)))
        else:
            _check(ctx, lib().j3dg_prepare_scene(inst, len(self.objects), fptr(mn), fptr(mx), fptr(d)))
        self.min_bb, self.max_bb, self.diagonal = mn, mx, np.float32(d[0])

    def unzoom(self) -> None:
        # scene.cpp:91-110
        cs = np.zeros(16, np.float32)
        inv = np.zeros(16, np.float32)
        piv = np.zeros(3, np.float32)
        lib().j3dg_unzoom(fptr(self.min_bb), fptr(self.max_bb), float(self.diagonal), fptr(cs), fptr(inv),
                          fptr(piv))
        self.coordinate_system, self.coordinate_system_inv, self.pivot = cs, inv, piv

    def set_pose(self, cs) -> None:
        """Sets coordinate_system (camera to world) and its orthonormal inverse."""
        self.coordinate_system = np.ascontiguousarray(np.asarray(cs, np.float32).reshape(16))
        self.coordinate_system_inv = invert_orthonormal(self.coordinate_system)

    def as_c(self):
        """(j3dg_scene, keep-alive) for the C-ABI."""
        inst = self._instances()
        s = _ffi.Scene()
        s.objects = C.cast(inst, C.POINTER(Instance))
        s.n_objects = len(self.objects)
        C.memmove(s.coordinate_system, self.coordinate_system.ctypes.data, 64)
        C.memmove(s.coordinate_system_inv, self.coordinate_system_inv.ctypes.data, 64)
        C.memmove(s.pivot, np.ascontiguousarray(self.pivot, np.float32).ctypes.data, 12)
        s.diagonal = float(self.diagonal)
        return s, inst


class Matcap:
    """matcap (matcap.h:18-24) uploaded to the device."""

    def __init__(self, ctx: Context, pixels: np.ndarray, cavity_clr: int):
        self.ctx = ctx
        self.pixels = np.ascontiguousarray(pixels, np.uint32)
        self.cavity_clr = int(cavity_clr)
        h = C.c_void_p()
        H, W = self.pixels.shape
        _check(ctx.h, lib().j3dg_matcap_create(ctx.h, vptr(self.pixels), W, H, self.cavity_clr, C.byref(h)))
        self.h = h
        ctx._own(self)

    @staticmethod
    def make(ctx: Context, kind: int = 0) -> "Matcap":
        px, cav = make_matcap(kind)
        return Matcap(ctx, px, cav)

    def close(self) -> None:
        if self.h:
            lib().j3dg_matcap_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def settings(one_bit=False, shadow=False, edges=True, wireframe=False, shading=True, textured=True,
             vertexcolors=True) -> CanvasSettings:
    """canvas_settings; defaults are j3d's (settings.cpp:5-25)."""
    return CanvasSettings(int(one_bit), int(shadow), int(edges), int(wireframe), int(shading), int(textured),
                          int(vertexcolors), 0)


class Canvas:
    """canvas (canvas.h:27-101) with device-resident G-buffer and image."""

    def __init__(self, ctx: Context, w: int, h: int):
        self.ctx = ctx
        hh = C.c_void_p()
        _check(ctx.h, lib().j3dg_canvas_create(ctx.h, w, h, C.byref(hh)))
        self.h = hh
        ctx._own(self)
        self.w, self.h_px = w, h

    def close(self) -> None:
        if self.h:
            lib().j3dg_canvas_destroy(self.h)
            self.h = None

    def expect_frame(self, seq: int) -> None:
        """Diagnostics: the next traced frame waits for every pixel to carry
        frame number seq (a number no frame wrote makes its waits run out)."""
        _check(self.ctx.h, lib().j3dg_canvas_expect_frame(self.h, seq))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def width(self) -> int:
        return self.w

    @property
    def height(self) -> int:
        return self.h_px

    def resize(self, w: int, h: int) -> None:
        _check(self.ctx.h, lib().j3dg_canvas_resize(self.h, w, h))
        self.w, self.h_px = w, h

    def set_camera(self, cam: Camera) -> None:
        _check(self.ctx.h, lib().j3dg_canvas_set_camera(self.h, C.byref(cam)))

    def get_projection(self) -> tuple[np.ndarray, np.ndarray]:
        p = np.zeros(16, np.float32)
        pi = np.zeros(16, np.float32)
        _check(self.ctx.h, lib().j3dg_canvas_get_projection(self.h, fptr(p), fptr(pi)))
        return p, pi

    def set_background_color(self, clr_top: int = 0xff000000, clr_bottom: int = 0xff404040) -> None:
        _check(self.ctx.h, lib().j3dg_canvas_set_background_color(self.h, clr_top, clr_bottom))

    def update_settings(self, s: CanvasSettings) -> None:
        _check(self.ctx.h, lib().j3dg_canvas_update_settings(self.h, C.byref(s)))

    def update_canvas(self, x0: int, y0: int, x1: int, y1: int, scene: Scene) -> None:
        s, keep = scene.as_c()
        _check(self.ctx.h, lib().j3dg_canvas_update_canvas(self.h, x0, y0, x1, y1, C.byref(s)))
        del keep

    def render_scene(self, scene: Scene | None) -> None:
        if scene is None:
            _check(self.ctx.h, lib().j3dg_canvas_render_scene(self.h, None))
            return
        s, keep = scene.as_c()
        _check(self.ctx.h, lib().j3dg_canvas_render_scene(self.h, C.byref(s)))
        del keep

    def canvas_to_image(self, matcap: Matcap, pixels=None) -> None:
        if pixels is None:
            _check(self.ctx.h, lib().j3dg_canvas_to_image(self.h, matcap.h))
        else:
            _check(self.ctx.h, lib().j3dg_canvas_to_image_from(self.h, vptr(pixels), matcap.h))

    def render_frame(self, scene: Scene | None, matcap: Matcap) -> None:
        """view::render_scene (view.cpp:421-430), asynchronous on the context stream."""
        if scene is None:
            _check(self.ctx.h, lib().j3dg_canvas_render_frame(self.h, None, matcap.h))
            return
        s, keep = scene.as_c()
        _check(self.ctx.h, lib().j3dg_canvas_render_frame(self.h, C.byref(s), matcap.h))
        del keep

    def render_pointclouds(self, scene: Scene) -> None:
        """canvas::render_pointclouds_on_image (canvas.cpp:952-1030) over the
        scene's point clouds, after a frame."""
        s, keep = scene.as_c()
        pcs = scene._pc_instances()
        _check(self.ctx.h, lib().j3dg_canvas_render_pointclouds(self.h, C.byref(s), pcs, len(scene.pointclouds)))

    def download_async(self, pixels=None, image=None) -> None:
        """Starts copying the G-buffer / image into `pixels` / `image` (pinned
        host or device buffers) on the copy stream; returns at once."""
        _check(self.ctx.h, lib().j3dg_canvas_download_async(self.h, vptr(pixels), vptr(image)))

    def download_wait(self) -> None:
        _check(self.ctx.h, lib().j3dg_canvas_download_wait(self.h))

    def get_pixels(self, out=None):
        if out is None:
            out = np.empty((self.h_px, self.w), PIXEL_DTYPE)
        _check(self.ctx.h, lib().j3dg_canvas_get_pixels(self.h, vptr(out)))
        return out

    def get_image(self, out=None):
        if out is None:
            out = np.empty((self.h_px, self.w), np.uint32)
        _check(self.ctx.h, lib().j3dg_canvas_get_image(self.h, vptr(out)))
        return out

    def set_pixels(self, px) -> None:
        _check(self.ctx.h, lib().j3dg_canvas_set_pixels(self.h, vptr(px)))

    def last_primary(self) -> int:
        """PRIMARY_TRACE or PRIMARY_RASTER: how the last frame found its primary hits."""
        return int(lib().j3dg_canvas_last_primary(self.h))

    def count_hits(self) -> tuple[int, int]:
        """(pixels with a hit, of which in shadow), counted on the device."""
        a, b = C.c_uint64(), C.c_uint64()
        _check(self.ctx.h, lib().j3dg_canvas_count_hits(self.h, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def device_buffers(self) -> tuple[int, int, int]:
        a, b, c = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(self.ctx.h, lib().j3dg_canvas_device_buffers(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value


# ----------------------------------------------------------------- batches

def _frames(frames):
    arr = (_ffi.Frame * max(1, len(frames)))()
    keep = []
    for i, (cv, sc, mc) in enumerate(frames):
        arr[i].canvas = cv.h
        arr[i].matcap = mc.h
        if sc is not None:
            s, k = sc.as_c()
            keep.append((s, k))
            arr[i].scene = C.pointer(s)
    return arr, keep


def render_batch(ctx: Context, frames) -> None:
    """Renders [(canvas, scene, matcap), ...] in one persistent launch (asynchronous)."""
    arr, keep = _frames(frames)
    _check(ctx.h, lib().j3dg_render_batch(ctx.h, arr, len(frames)))
    del keep


class Batch:
    """A fixed set of frames captured as a CUDA graph; set_scene() moves cameras.
    rebuild=True: every launch first rebuilds the BVHs of the scenes' meshes
    (built rebuildable) inside the same graph (J3DG_BATCH_REBUILD)."""

    def __init__(self, ctx: Context, frames, rebuild: bool = False):
        self.ctx = ctx
        self.frames = list(frames)
        arr, keep = _frames(self.frames)
        h = C.c_void_p()
        _check(ctx.h, lib().j3dg_batch_create2(ctx.h, arr, len(self.frames), 0x1 if rebuild else 0, C.byref(h)))
        self.h = h
        ctx._own(self)
        del keep

    def set_scene(self, i: int, scene: "Scene") -> None:
        s, keep = scene.as_c()
        _check(self.ctx.h, lib().j3dg_batch_set_scene(self.h, i, C.byref(s)))
        del keep

    def launch(self) -> None:
        _check(self.ctx.h, lib().j3dg_batch_launch(self.h))

    def close(self) -> None:
        if self.h:
            lib().j3dg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------- ray queries

def _instances(objs: list[SceneObject]):
    arr = (Instance * max(1, len(objs)))()
    for i, o in enumerate(objs):
        arr[i].mesh = o.mesh.h
        C.memmove(arr[i].cs, o.cs.ctypes.data, 64)
        arr[i].db_id = o.db_id
    return arr


def find_closest(ctx: Context, objs: list[SceneObject], rays, hits=None, any_hit: bool = False):
    """qbvh_two_level_with_transformations::find_closest_triangle over a ray batch."""
    n = len(rays)
    if hits is None:
        hits = np.empty(n, HIT_DTYPE)
    inst = _instances(objs)
    f = lib().j3dg_find_any if any_hit else lib().j3dg_find_closest
    _check(ctx.h, f(ctx.h, inst, len(objs), vptr(rays), n, vptr(hits)))
    return hits


def find_all(ctx: Context, mesh: Mesh, rays, cap: int = 64):
    """find_all_triangles (vox.cpp:333): (hits[n, cap] sorted by (t, id), counts[n])."""
    n = len(rays)
    hits = np.zeros((n, cap), HIT_DTYPE)
    counts = np.zeros(n, np.uint32)
    _check(ctx.h, lib().j3dg_find_all(ctx.h, mesh.h, vptr(rays), n, cap, vptr(hits) if cap else None, vptr(counts)))
    return hits, counts


def voxelize(ctx: Context, mesh: Mesh, max_dim: int = 100) -> np.ndarray:
    """The voxel grid of write_vox (vox.cpp:284-380) as uint8[z, y, x]."""
    dims = (C.c_uint32 * 3)()
    _check(ctx.h, lib().j3dg_voxelize(ctx.h, mesh.h, max_dim, dims, None, 0))
    out = np.zeros(int(dims[0]) * int(dims[1]) * int(dims[2]), np.uint8)
    _check(ctx.h, lib().j3dg_voxelize(ctx.h, mesh.h, max_dim, dims, vptr(out), out.size))
    return out.reshape(int(dims[2]), int(dims[1]), int(dims[0]))


def get_closest_vertex(p, V: np.ndarray, T: np.ndarray) -> int:
    """pixel.cpp:6-25"""
    rec = np.ascontiguousarray(np.asarray(p).reshape(1), PIXEL_DTYPE)
    return int(lib().j3dg_get_closest_vertex(vptr(rec), vptr(V), vptr(T)))


def get_world_position(p, V: np.ndarray, T: np.ndarray, cs) -> np.ndarray:
    """view.cpp:439-459 (mesh branch)"""
    rec = np.ascontiguousarray(np.asarray(p).reshape(1), PIXEL_DTYPE)
    out = np.zeros(3, np.float32)
    lib().j3dg_get_world_position(vptr(rec), vptr(V), vptr(T), fptr(np.ascontiguousarray(cs, np.float32)), fptr(out))
    return out


# --------------------------------------------------------- host j3d math

def make_default_camera() -> Camera:
    c = Camera()
    lib().j3dg_make_default_camera(C.byref(c))
    return c


def make_projection_matrix(cam: Camera, w: int, h: int) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().j3dg_make_projection_matrix(C.byref(cam), w, h, fptr(out))
    return out


def invert_projection_matrix(p: np.ndarray) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().j3dg_invert_projection_matrix(fptr(np.ascontiguousarray(p, np.float32)), fptr(out))
    return out


def invert_orthonormal(m: np.ndarray) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().j3dg_invert_orthonormal(fptr(np.ascontiguousarray(m, np.float32).reshape(16)), fptr(out))
    return out


def make_matcap(kind: int = 0) -> tuple[np.ndarray, int]:
    px = np.zeros((512, 512), np.uint32)
    w, h, cav = C.c_uint32(), C.c_uint32(), C.c_uint32()
    st = lib().j3dg_make_matcap(kind, vptr(px), C.byref(w), C.byref(h), C.byref(cav))
    if st:
        raise J3dgError(st, f"make_matcap({kind})")
    return px, int(cav.value)


def fill_background(w: int, h: int, top: int = 0xff000000, bottom: int = 0xff404040) -> np.ndarray:
    bg = np.zeros((h, w), np.uint32)
    lib().j3dg_fill_background(vptr(bg), w, h, top, bottom)
    return bg


def camera_for_vfov(vfov_deg: float) -> Camera:
    """Default film-gate camera (camera.cpp:5-16) with the focal length giving vfov_deg."""
    c = make_default_camera()
    c.focal_length = lib().j3dg_focal_for_vfov(vfov_deg, c.film_aperture_height_inch)
    return c


__all__ = ["Context", "Mesh", "Scene", "SceneObject", "Matcap", "Canvas", "settings", "find_closest", "find_all",
           "render_batch", "Batch",
           "voxelize", "get_closest_vertex", "get_world_position",
           "make_default_camera", "make_projection_matrix", "invert_projection_matrix", "invert_orthonormal",
           "make_matcap", "fill_background", "camera_for_vfov", "PIXEL_DTYPE", "RAY_DTYPE", "HIT_DTYPE",
           "J3dgError"]
