"""Learned tmax: a ray -> cluster network that seeds exact closest-hit
traversal (wraps j3dg_learned_* of include/j3dg.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi
from ._ffi import HIT_DTYPE, lib, vptr
from .scene import Context, Mesh, _check

N_IN, N_HID, N_OUT = 256, 128, 4096


class LearnedOpts(C.Structure):
    _fields_ = [("cluster_depth", C.c_uint32), ("batch", C.c_uint32), ("lr", C.c_float), ("reserved", C.c_uint32),
                ("seed", C.c_uint64)]


def param_layout():
    """[(name, offset, shape)] of the flat parameter vector (W row-major [in][out])."""
    ins = [N_IN, N_HID, N_HID, N_HID, N_HID]
    outs = [N_HID, N_HID, N_HID, N_HID, N_OUT]
    out, o = [], 0
    for k in range(5):
        out.append((f"W{k + 1}", o, (ins[k], outs[k])))
        o += ins[k] * outs[k]
        out.append((f"b{k + 1}", o, (outs[k],)))
        o += outs[k]
    return out, o


class Learned:
    def __init__(self, ctx: Context, mesh: Mesh, cluster_depth: int = 6, batch: int = 16384, lr: float = 2e-3,
                 seed: int = 0x6A3D0003):
        self.ctx = ctx
        self.mesh = mesh
        h = C.c_void_p()
        o = LearnedOpts(cluster_depth, batch, lr, 0, seed)
        _check(ctx.h, lib().j3dg_learned_create(ctx.h, mesh.h, C.byref(o), C.byref(h)))
        self.h = h
        ctx._own(self)
        k, p = C.c_uint32(), C.c_uint64()
        _check(ctx.h, lib().j3dg_learned_info(self.h, C.byref(k), C.byref(p)))
        self.n_clusters, self.n_params = int(k.value), int(p.value)

    def close(self):
        if self.h:
            lib().j3dg_learned_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def train(self, n_rays: int, r0: float = 2.0, r1: float = 5.0):
        loss, acc, secs = C.c_float(), C.c_float(), C.c_float()
        _check(self.ctx.h, lib().j3dg_learned_train(self.h, n_rays, r0, r1, C.byref(loss), C.byref(acc), C.byref(secs)))
        return float(loss.value), float(acc.value), float(secs.value)

    def predict(self, rays, impl: int = 1) -> np.ndarray:
        """Top-2 clusters per ray: impl 1 the fused tcgen05 kernel, 0 the
        layer-by-layer tcgen05 GEMMs of training."""
        out = np.zeros((len(rays), 2), np.uint32)
        _check(self.ctx.h, lib().j3dg_learned_predict_impl(self.h, vptr(rays), len(rays), vptr(out), impl))
        return out

    def find_closest(self, rays, hits=None):
        if hits is None:
            hits = np.zeros(len(rays), HIT_DTYPE)
        _check(self.ctx.h, lib().j3dg_learned_find_closest(self.h, vptr(rays), len(rays), vptr(hits)))
        return hits

    def find_closest_stats(self, rays, hits=None):
        """(hits, {cluster_visits, cluster_tests, exact_visits, exact_tests})."""
        if hits is None:
            hits = np.zeros(len(rays), HIT_DTYPE)
        st = (C.c_uint64 * 4)()
        _check(self.ctx.h, lib().j3dg_learned_find_closest_stats(self.h, vptr(rays), len(rays), vptr(hits), st))
        return hits, dict(zip(("cluster_visits", "cluster_tests", "exact_visits", "exact_tests"), list(st)))

    def render_frame(self, canvas, scene, matcap) -> None:
        """A canvas frame whose primary hits come from the learned path
        (asynchronous on the context stream); equal to canvas.render_frame."""
        s, keep = scene.as_c()
        _check(self.ctx.h, lib().j3dg_learned_render_frame(self.h, canvas.h, C.byref(s), matcap.h))
        del keep

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        _check(self.ctx.h, lib().j3dg_learned_get_params(self.h, vptr(out)))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        _check(self.ctx.h, lib().j3dg_learned_set_params(self.h, vptr(p)))

    def loss_grad(self, feats: np.ndarray, labels: np.ndarray):
        feats = np.ascontiguousarray(feats, np.float32)
        labels = np.ascontiguousarray(labels, np.int32)
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_float()
        _check(self.ctx.h, lib().j3dg_learned_loss_grad(self.h, vptr(feats), vptr(labels), len(labels), C.byref(loss),
                                                        vptr(g)))
        return float(loss.value), g

    def save(self, path: str) -> None:
        _check(self.ctx.h, lib().j3dg_learned_save(self.h, str(path).encode()))

    def load(self, path: str) -> None:
        _check(self.ctx.h, lib().j3dg_learned_load(self.h, str(path).encode()))
