"""ctypes binding of libj3dgpu.so (include/j3dg.h).

Loads the in-tree library built by j3d_gb300/build.py. There is no fallback:
if the library is missing or has no usable GPU the calls raise.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libj3dgpu.so"

# ------------------------------------------------------------ record dtypes

# pixel.h:11-27 (32 bytes)
PIXEL_DTYPE = np.dtype([("mark", "u1"), ("r", "u1"), ("g", "u1"), ("b", "u1"), ("u", "<f4"), ("v", "<f4"),
                        ("depth", "<f4"), ("object_id", "<u4"), ("barycentric_u", "<f4"),
                        ("barycentric_v", "<f4"), ("db_id", "<u4")])
# jtk::ray (40 bytes)
RAY_DTYPE = np.dtype([("orig", "<f4", 4), ("dir", "<f4", 4), ("t_near", "<f4"), ("t_far", "<f4")])
# jtk::hit + find_closest_triangle out-params (24 bytes)
HIT_DTYPE = np.dtype([("found", "<u4"), ("distance", "<f4"), ("u", "<f4"), ("v", "<f4"), ("object_id", "<u4"),
                      ("two_level_index", "<u4")])
assert PIXEL_DTYPE.itemsize == 32 and RAY_DTYPE.itemsize == 40 and HIT_DTYPE.itemsize == 24

J3DG_OK = 0
J3DG_ERR_INVALID_ARGUMENT = 1
# how canvas frames find primary hits (j3dg_ctx_set_primary_mode)
PRIMARY_AUTO, PRIMARY_TRACE, PRIMARY_RASTER = 0, 1, 2
STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "no CUDA device",
                5: "device status raised", 6: "unsupported"}


class J3dgError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        super().__init__(f"j3dg status {status} ({STATUS_NAMES.get(status, '?')}): {msg}")
        self.status = status


class Instance(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("cs", C.c_float * 16), ("db_id", C.c_uint32), ("reserved", C.c_uint32)]


class Scene(C.Structure):
    _fields_ = [("objects", C.POINTER(Instance)), ("n_objects", C.c_uint32), ("reserved", C.c_uint32),
                ("coordinate_system", C.c_float * 16), ("coordinate_system_inv", C.c_float * 16),
                ("pivot", C.c_float * 3), ("diagonal", C.c_float)]


class Camera(C.Structure):
    _fields_ = [("focal_length", C.c_float), ("film_aperture_width_inch", C.c_float),
                ("film_aperture_height_inch", C.c_float), ("near_clipping_plane", C.c_float),
                ("far_clipping_plane", C.c_float), ("zoom", C.c_float), ("fit_film", C.c_int32)]


class CanvasSettings(C.Structure):
    _fields_ = [("one_bit", C.c_uint8), ("shadow", C.c_uint8), ("edges", C.c_uint8), ("wireframe", C.c_uint8),
                ("shading", C.c_uint8), ("textured", C.c_uint8), ("vertexcolors", C.c_uint8),
                ("reserved", C.c_uint8)]


class Frame(C.Structure):
    _fields_ = [("canvas", C.c_void_p), ("scene", C.POINTER(Scene)), ("matcap", C.c_void_p)]


class BuildOpts(C.Structure):
    _fields_ = [("leaf_size", C.c_uint32), ("flags", C.c_uint32)]


class MeshSource(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("n_vertices", C.c_uint32), ("n_triangles", C.c_uint32),
                ("triangles", C.c_void_p)]


class MeshInfo(C.Structure):
    _fields_ = [("n_vertices", C.c_uint32), ("n_triangles", C.c_uint32), ("min_bb", C.c_float * 3),
                ("max_bb", C.c_float * 3), ("n_nodes", C.c_uint32), ("max_depth", C.c_uint32),
                ("device_bytes", C.c_uint64), ("build_ms", C.c_float), ("width", C.c_uint32)]


class GeometryInfo(C.Structure):
    _fields_ = [("n_vertices", C.c_uint64), ("n_triangles", C.c_uint64), ("format", C.c_uint32),
                ("encoding", C.c_uint32), ("has_colors", C.c_uint32), ("has_normals", C.c_uint32),
                ("has_uv", C.c_uint32), ("device_decoded", C.c_uint32), ("file_bytes", C.c_uint64),
                ("read_ms", C.c_float), ("decode_ms", C.c_float), ("total_ms", C.c_float), ("reserved", C.c_float)]


class PointCloudInstance(C.Structure):
    _fields_ = [("pointcloud", C.c_void_p), ("cs", C.c_float * 16), ("db_id", C.c_uint32), ("reserved", C.c_uint32)]


FORMATS = {"auto": 0, "ply": 1, "stl": 2, "obj": 3, "off": 4, "xyz": 5, "pts": 6}

_P = C.c_void_p
_I = C.c_int
_U = C.c_uint32
_F = C.c_float
_FP = C.POINTER(C.c_float)

# name -> (restype, argtypes)
SIGNATURES = {
    "j3dg_abi_version": (_I, []),
    "j3dg_status_string": (C.c_char_p, [_I]),
    "j3dg_last_error": (C.c_char_p, [_P]),
    "j3dg_ctx_create": (_I, [_I, C.POINTER(_P)]),
    "j3dg_ctx_destroy": (_I, [_P]),
    "j3dg_ctx_synchronize": (_I, [_P]),
    "j3dg_ctx_device_status": (_I, [_P, C.POINTER(_U)]),
    "j3dg_ctx_stream": (_P, [_P]),
    "j3dg_ctx_set_counting": (_I, [_P, _I]),
    "j3dg_ctx_read_counters": (_I, [_P, C.POINTER(C.c_uint64), _I]),
    "j3dg_ctx_memory": (_I, [_P, C.POINTER(C.c_uint64)]),
    "j3dg_mesh_build_many": (_I, [_P, _U, _P, _P, _U, _P]),
    "j3dg_ctx_set_top_level": (_I, [_P, _I]),
    "j3dg_ctx_set_frame_overlap": (_I, [_P, _I]),
    "j3dg_canvas_expect_frame": (_I, [_P, _U]),
    "j3dg_mesh_build": (_I, [_P, _P, _U, _P, _U, C.POINTER(BuildOpts), C.POINTER(_P)]),
    "j3dg_mesh_destroy": (_I, [_P]),
    "j3dg_mesh_get_info": (_I, [_P, C.POINTER(MeshInfo)]),
    "j3dg_mesh_get_nodes": (_I, [_P, _P, C.c_uint64]),
    "j3dg_mesh_get_triangle_normals": (_I, [_P, _P]),
    "j3dg_mesh_set_vertex_colors": (_I, [_P, _P]),
    "j3dg_mesh_set_uv": (_I, [_P, _P]),
    "j3dg_mesh_set_texture": (_I, [_P, _P, _U, _U]),
    "j3dg_find_closest": (_I, [_P, C.POINTER(Instance), _U, _P, _U, _P]),
    "j3dg_find_any": (_I, [_P, C.POINTER(Instance), _U, _P, _U, _P]),
    "j3dg_find_all": (_I, [_P, _P, _P, _U, _U, _P, _P]),
    "j3dg_voxelize": (_I, [_P, _P, _U, C.POINTER(_U), _P, C.c_uint64]),
    "j3dg_voxelize_noalloc": (_I, [_P, _P, _U, C.POINTER(_U), _P, C.c_uint64]),
    "j3dg_get_closest_vertex": (_U, [_P, _P, _P]),
    "j3dg_get_world_position": (None, [_P, _P, _P, _FP, _FP]),
    "j3dg_geometry_read_file": (_I, [_P, C.c_char_p, _I, C.POINTER(_P)]),
    "j3dg_geometry_read_memory": (_I, [_P, _P, C.c_uint64, _I, C.POINTER(_P)]),
    "j3dg_geometry_get_info": (_I, [_P, C.POINTER(GeometryInfo)]),
    "j3dg_geometry_get_arrays": (_I, [_P, _P, _P, _P, _P, _P]),
    "j3dg_geometry_destroy": (_I, [_P]),
    "j3dg_mesh_build_geometry": (_I, [_P, _P, C.POINTER(BuildOpts), C.POINTER(_P)]),
    "j3dg_pointcloud_create": (_I, [_P, _P, C.c_uint64, _P, C.POINTER(_P)]),
    "j3dg_pointcloud_from_geometry": (_I, [_P, _P, C.POINTER(_P)]),
    "j3dg_pointcloud_destroy": (_I, [_P]),
    "j3dg_pointcloud_get_bounds": (_I, [_P, _FP, _FP]),
    "j3dg_prepare_scene_pointclouds": (_I, [C.POINTER(Instance), _U, C.POINTER(PointCloudInstance), _U, _FP, _FP,
                                            _FP]),
    "j3dg_canvas_render_pointclouds": (_I, [_P, C.POINTER(Scene), C.POINTER(PointCloudInstance), _U]),
    "j3dg_matcap_create": (_I, [_P, _P, _U, _U, _U, C.POINTER(_P)]),
    "j3dg_matcap_destroy": (_I, [_P]),
    "j3dg_canvas_create": (_I, [_P, _U, _U, C.POINTER(_P)]),
    "j3dg_canvas_destroy": (_I, [_P]),
    "j3dg_canvas_resize": (_I, [_P, _U, _U]),
    "j3dg_canvas_set_camera": (_I, [_P, C.POINTER(Camera)]),
    "j3dg_canvas_get_projection": (_I, [_P, _FP, _FP]),
    "j3dg_canvas_set_background_color": (_I, [_P, _U, _U]),
    "j3dg_canvas_update_settings": (_I, [_P, C.POINTER(CanvasSettings)]),
    "j3dg_canvas_update_canvas": (_I, [_P, _I, _I, _I, _I, C.POINTER(Scene)]),
    "j3dg_canvas_render_scene": (_I, [_P, C.POINTER(Scene)]),
    "j3dg_canvas_to_image": (_I, [_P, _P]),
    "j3dg_canvas_to_image_from": (_I, [_P, _P, _P]),
    "j3dg_canvas_render_frame": (_I, [_P, C.POINTER(Scene), _P]),
    "j3dg_canvas_get_pixels": (_I, [_P, _P]),
    "j3dg_canvas_get_image": (_I, [_P, _P]),
    "j3dg_canvas_set_pixels": (_I, [_P, _P]),
    "j3dg_canvas_download_async": (_I, [_P, _P, _P]),
    "j3dg_canvas_download_wait": (_I, [_P]),
    "j3dg_canvas_count_hits": (_I, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "j3dg_canvas_device_buffers": (_I, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    "j3dg_render_batch": (_I, [_P, C.POINTER(Frame), _U]),
    "j3dg_ctx_set_batch_block": (_I, [_P, _I]),
    "j3dg_ctx_set_primary_mode": (_I, [_P, _I]),
    "j3dg_canvas_last_primary": (_I, [_P]),
    "j3dg_batch_create": (_I, [_P, C.POINTER(Frame), _U, C.POINTER(_P)]),
    "j3dg_batch_create2": (_I, [_P, C.POINTER(Frame), _U, _U, C.POINTER(_P)]),
    "j3dg_batch_set_scene": (_I, [_P, _U, C.POINTER(Scene)]),
    "j3dg_batch_launch": (_I, [_P]),
    "j3dg_batch_destroy": (_I, [_P]),
    "j3dg_gemm_bf16": (_I, [_P, _P, _P, _P, _U, _U, _U, _I]),
    "j3dg_learned_create": (_I, [_P, _P, _P, C.POINTER(_P)]),
    "j3dg_learned_destroy": (_I, [_P]),
    "j3dg_learned_info": (_I, [_P, C.POINTER(_U), C.POINTER(C.c_uint64)]),
    "j3dg_learned_train": (_I, [_P, C.c_uint64, _F, _F, C.POINTER(_F), C.POINTER(_F), C.POINTER(_F)]),
    "j3dg_learned_predict": (_I, [_P, _P, _U, _P]),
    "j3dg_learned_predict_impl": (_I, [_P, _P, _U, _P, _I]),
    "j3dg_learned_find_closest": (_I, [_P, _P, _U, _P]),
    "j3dg_learned_find_closest_stats": (_I, [_P, _P, _U, _P, C.POINTER(C.c_uint64)]),
    "j3dg_learned_get_params": (_I, [_P, _P]),
    "j3dg_learned_set_params": (_I, [_P, _P]),
    "j3dg_learned_loss_grad": (_I, [_P, _P, _P, _U, C.POINTER(_F), _P]),
    "j3dg_learned_save": (_I, [_P, C.c_char_p]),
    "j3dg_learned_render_frame": (_I, [_P, _P, C.POINTER(Scene), _P]),
    "j3dg_learned_load": (_I, [_P, C.c_char_p]),
    "j3dg_make_default_camera": (None, [C.POINTER(Camera)]),
    "j3dg_make_projection_matrix": (None, [C.POINTER(Camera), _I, _I, _FP]),
    "j3dg_invert_projection_matrix": (None, [_FP, _FP]),
    "j3dg_invert_orthonormal": (None, [_FP, _FP]),
    "j3dg_prepare_scene": (_I, [C.POINTER(Instance), _U, _FP, _FP, _FP]),
    "j3dg_unzoom": (None, [_FP, _FP, _F, _FP, _FP, _FP]),
    "j3dg_make_matcap": (_I, [_I, _P, C.POINTER(_U), C.POINTER(_U), C.POINTER(_U)]),
    "j3dg_fill_background": (None, [_P, _U, _U, _U, _U]),
    "j3dg_synth_icosphere": (_I, [_U, C.c_uint64, _F, _P, _P]),
    "j3dg_synth_torus": (_I, [_U, _U, _F, _F, C.c_uint64, _F, _P, _P]),
    "j3dg_synth_cameras": (_I, [_U, C.c_uint64, _F, _F, _FP, _FP]),
    "j3dg_focal_for_vfov": (_F, [_F, _F]),
}

_lib = None


def lib() -> C.CDLL:
    """The loaded libj3dgpu.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run j3d_gb300.build.build() (there is no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_FP)


def vptr(a) -> int | None:
    """Address of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags.c_contiguous
        return a.ctypes.data
    return a.data_ptr()  # torch.Tensor
