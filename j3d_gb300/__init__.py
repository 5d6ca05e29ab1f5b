"""j3d_gb300: GB300 (sm_103a) implementation of j3d's ray-cast rendering hot path.

BVH build over a triangle mesh (jtk qbvh), per-pixel closest hit, shadow ray
and matcap shading into j3d's 32-byte pixel G-buffer and RGBA8 canvas, behind
the C-ABI of include/j3dg.h (libj3dgpu.so). This package is the host-side
mirror of the reference's scene/canvas interface over that C-ABI.
"""
from ._ffi import HIT_DTYPE, PIXEL_DTYPE, RAY_DTYPE, J3dgError, LIB_PATH, lib  # noqa: F401
from ._ffi import PRIMARY_AUTO, PRIMARY_RASTER, PRIMARY_TRACE  # noqa: F401
from .scene import (Batch, Canvas, Context, Geometry, Matcap, Mesh, PointCloud, build_meshes, mesh_from_geometry, Scene, SceneObject, camera_for_vfov, fill_background,  # noqa: F401
                    find_all, find_closest, get_closest_vertex, get_world_position, invert_orthonormal, voxelize, invert_projection_matrix, make_default_camera, make_matcap,
                    make_projection_matrix, render_batch, settings)
