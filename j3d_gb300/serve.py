"""Render-request serving loop with continuous batching.

Meshes stay resident on the device (BVH, leaf triangles, normals) and are
admitted by their HBM footprint against a cap. Requests (mesh, camera pose,
resolution) arrive over time; whenever the device has room (at most
`max_in_flight` batches queued on the stream) every waiting request that fits
the free canvas slots and the memory cap is admitted and the admitted group
is rendered by one persistent launch (j3dg_render_batch). Requests that arrive
while a batch runs join the next one, without waiting for a full batch.
A frame's result is a pure function of (mesh, pose, resolution, settings): the
batch a request lands in does not change its bytes (tests check alone == in
the mix).

Latency = completion (a CUDA event after the request's batch) - arrival.

With learned networks attached (attach_learned), frames of those meshes find
their primary hits through the learned path (j3dg_learned_render_frame:
network, then the exact traversal it seeds); the admitted group is queued
frame by frame, and the images are the plain path's (tests check it).
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    rid: int
    mesh: str
    pose: np.ndarray          # camera-to-world, 16 floats column-major
    resolution: tuple         # (w, h)
    arrival: float            # seconds on the server clock
    admitted: float = -1.0
    done: float = -1.0
    slot: object = None


@dataclass
class ServeStats:
    requests: int
    frames_per_s: float
    p50_ms: float
    p99_ms: float
    mean_ms: float
    max_in_flight_frames: int
    batches: int
    mean_batch: float
    rejected_meshes: list = field(default_factory=list)
    peak_bytes: int = 0


class CanvasPool:
    """Canvases per resolution, reused across requests (no per-frame allocation)."""

    def __init__(self, ctx, camera):
        self.ctx = ctx
        self.camera = camera
        self.free: dict[tuple, list] = {}
        self.count = 0
        self.bytes = 0

    @staticmethod
    def canvas_bytes(w: int, h: int) -> int:
        # per pixel: G-buffer 32 B + image 4 B + background 4 B + frame scratch
        # 48 B; per canvas: 16 KB of scratch tables and 16 B of work counters
        return w * h * 88 + 16384 + 16

    def take(self, res, settings):
        from .scene import Canvas
        lst = self.free.get(res)
        if lst:
            cv = lst.pop()
        else:
            cv = Canvas(self.ctx, *res)
            cv.set_camera(self.camera)
            cv.set_background_color()
            self.count += 1
            self.bytes += self.canvas_bytes(*res)
        cv.update_settings(settings)
        return cv

    def give(self, res, cv) -> None:
        self.free.setdefault(res, []).append(cv)

    def evict(self, keep_res, nbytes: int, reserved: dict) -> int:
        """Frees idle canvases of other resolutions (not reserved for the
        group being formed) until nbytes are released; returns bytes freed."""
        freed = 0
        for res in list(self.free):
            if res == keep_res:
                continue
            lst = self.free[res]
            while lst and len(lst) > reserved.get(res, 0) and freed < nbytes:
                cv = lst.pop()
                cv.close()
                self.count -= 1
                b = self.canvas_bytes(*res)
                self.bytes -= b
                freed += b
            if freed >= nbytes:
                break
        return freed


class RenderServer:
    def __init__(self, ctx, hbm_cap_bytes: int, max_slots: int = 64, max_in_flight: int = 2, shadow: bool = True,
                 keep_images: bool = False):
        import torch

        from .scene import Matcap, camera_for_vfov, settings
        self.ctx = ctx
        self.cap = int(hbm_cap_bytes)
        self.max_slots = max_slots
        self.max_in_flight = max_in_flight
        self.meshes: dict[str, object] = {}
        self.mesh_bytes = 0
        self.matcap = Matcap.make(ctx, 0)
        self.settings = settings(shadow=shadow, edges=False)
        self.pool = CanvasPool(ctx, camera_for_vfov(60.0))
        self.stream = torch.cuda.ExternalStream(ctx.stream())
        self.in_flight: deque = deque()  # (event, [requests])
        self.busy_slots = 0
        self.peak_bytes = 0
        self.keep_images = keep_images
        self.images: dict[int, np.ndarray] = {}
        self.learned: dict[str, object] = {}

    # ------------------------------------------------------------- meshes
    def add_mesh(self, name: str, V, T, leaf_size: int = 2) -> bool:
        """Builds and keeps a mesh resident if its footprint fits the cap."""
        from .scene import Mesh
        est = int(len(T)) * (48 + 16 + 12 + 4 + 40) + int(len(V)) * 12
        if self.mesh_bytes + est > self.cap:
            return False
        m = Mesh(self.ctx, V, T, leaf_size)
        real = int(m.info().device_bytes)
        if self.mesh_bytes + real > self.cap:
            m.close()
            return False
        self.meshes[name] = m
        self.mesh_bytes += real
        return True

    def attach_learned(self, name: str, net) -> None:
        """Frames of mesh `name` go through the learned network `net`
        (a j3d_gb300.learned.Learned over that mesh)."""
        if net.mesh is not self.meshes[name]:
            raise ValueError("the network belongs to another mesh")
        self.learned[name] = net

    def footprint(self) -> int:
        return self.mesh_bytes + self.pool.bytes

    # ------------------------------------------------------------- frames
    def _scene(self, req: Request):
        from .scene import Scene
        sc = Scene()
        sc.add_object(self.meshes[req.mesh])
        sc.prepare_scene()
        sc.unzoom()
        sc.set_pose(req.pose)
        return sc

    def _fits(self, req: Request, reserved: dict, new_bytes: int) -> int:
        """Bytes a new canvas for req would add (0 if a pooled one is free), or -1 if it does not fit."""
        if self.busy_slots >= self.max_slots:
            return -1
        res = tuple(req.resolution)
        if len(self.pool.free.get(res, [])) > reserved.get(res, 0):
            return 0
        need = CanvasPool.canvas_bytes(*res)
        over = self.footprint() + new_bytes + need - self.cap
        if over > 0:
            self.pool.evict(res, over, reserved)
        return need if self.footprint() + new_bytes + need <= self.cap else -1

    def _launch(self, reqs: list) -> None:
        import torch

        from .scene import render_batch
        frames = []
        for r in reqs:
            cv = self.pool.take(tuple(r.resolution), self.settings)
            r.slot = cv
            if r.mesh in self.learned:
                self.learned[r.mesh].render_frame(cv, self._scene(r), self.matcap)
            else:
                frames.append((cv, self._scene(r), self.matcap))
        if frames:
            render_batch(self.ctx, frames)
        ev = torch.cuda.Event()
        ev.record(self.stream)
        self.in_flight.append((ev, reqs))
        self.busy_slots += len(reqs)
        self.peak_bytes = max(self.peak_bytes, self.footprint())

    def _retire(self, clock) -> int:
        n = 0
        while self.in_flight and self.in_flight[0][0].query():
            ev, reqs = self.in_flight.popleft()
            t = clock()
            for r in reqs:
                r.done = t
                if self.keep_images:
                    self.images[r.rid] = r.slot.get_image()
                self.pool.give(tuple(r.resolution), r.slot)
            self.busy_slots -= len(reqs)
            n += len(reqs)
        return n

    def run(self, requests: list, realtime: bool = True, on_done=None) -> ServeStats:
        """Serves requests in arrival order; with realtime, arrivals follow
        the wall clock (Poisson process replayed as recorded)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        t0 = time.perf_counter()
        clock = (lambda: time.perf_counter() - t0) if realtime else (lambda: float("inf"))
        waiting: deque = deque()
        i = 0
        batches = 0
        batch_sizes = []
        max_frames = 0
        while i < len(reqs) or waiting or self.in_flight:
            now = clock()
            while i < len(reqs) and reqs[i].arrival <= now:
                waiting.append(reqs[i])
                i += 1
            self._retire(clock)
            if waiting and len(self.in_flight) < self.max_in_flight:
                group = []
                reserved: dict = {}
                new_bytes = 0
                while waiting:
                    add = self._fits(waiting[0], reserved, new_bytes)
                    if add < 0:
                        break
                    r = waiting.popleft()
                    r.admitted = clock() if realtime else 0.0
                    group.append(r)
                    res = tuple(r.resolution)
                    reserved[res] = reserved.get(res, 0) + 1
                    new_bytes += add
                    self.busy_slots += 1  # reserve while grouping
                self.busy_slots -= len(group)
                if not group and not self.in_flight and waiting:
                    raise RuntimeError("a request does not fit the HBM cap even on an idle device")
                if group:
                    self._launch(group)
                    batches += 1
                    batch_sizes.append(len(group))
                    max_frames = max(max_frames, self.busy_slots)
                    continue
            if self.in_flight:
                if not waiting and i < len(reqs) and realtime:
                    # idle until the next arrival or the oldest batch completes
                    time.sleep(min(2e-4, max(0.0, reqs[i].arrival - clock())))
                else:
                    time.sleep(2e-5)
            elif i < len(reqs) and realtime:
                time.sleep(max(0.0, min(2e-4, reqs[i].arrival - clock())))
        self.ctx.synchronize()
        end = clock() if realtime else 0.0
        lat = np.array([(r.done - r.arrival) * 1e3 for r in reqs]) if realtime else np.zeros(len(reqs))
        span = max(end - reqs[0].arrival, 1e-9) if realtime and reqs else 1.0
        return ServeStats(len(reqs), len(reqs) / span, float(np.percentile(lat, 50)) if len(lat) else 0.0,
                          float(np.percentile(lat, 99)) if len(lat) else 0.0, float(lat.mean()) if len(lat) else 0.0,
                          max_frames, batches, float(np.mean(batch_sizes)) if batch_sizes else 0.0,
                          peak_bytes=self.peak_bytes)


def poisson_requests(n: int, rate: float, meshes: list, seed: int, resolutions=((512, 512), (1280, 720), (1920, 1080)),
                     r0: float = 2.5, r1: float = 4.0) -> list:
    """n requests with exponential inter-arrival times (mean 1/rate), a mesh,
    a camera and a resolution each, all from one seed."""
    from .workloads import cameras
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    poses = cameras(n, seed + 7, r0, r1)
    out = []
    for k in range(n):
        out.append(Request(k, meshes[int(rng.integers(0, len(meshes)))], poses[k],
                           tuple(resolutions[int(rng.integers(0, len(resolutions)))]), float(t[k])))
    return out
