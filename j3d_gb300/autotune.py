"""Autotuner for the batched renderer: picks, per mesh-size bucket, the BVH
width, the leaf size and the block shape of the persistent launch by timing
real frames.

Search space: BVH width (children per node) 2, 4, 8; leaf size (max
triangles per leaf) 1, 2, 4, 8; block shapes of 64, 128, 256 threads. A batch
shares one width and one block shape (the kernels are specialised on both):
the heaviest bucket's choice. Results are kept per bucket of log2(triangle
count) in a JSON cache.
"""
from __future__ import annotations

import json
import math
from dataclasses import asdict, dataclass
from pathlib import Path

import numpy as np

WIDTHS = (2, 4, 8)
LEAF_SIZES = (1, 2, 4, 8)
BLOCKS = (64, 128, 256)


@dataclass
class Choice:
    bucket: int
    leaf_size: int
    block_threads: int
    ms_per_frame: float
    width: int = 4


def bucket_of(n_triangles: int) -> int:
    return int(math.floor(math.log2(max(1, n_triangles))))


class Autotuner:
    def __init__(self, ctx, cache_path: str | Path | None = None):
        self.ctx = ctx
        self.cache_path = Path(cache_path) if cache_path else None
        self.table: dict[int, Choice] = {}
        if self.cache_path and self.cache_path.exists():
            for k, v in json.loads(self.cache_path.read_text()).items():
                self.table[int(k)] = Choice(**v)

    def save(self) -> None:
        if self.cache_path:
            self.cache_path.parent.mkdir(parents=True, exist_ok=True)
            self.cache_path.write_text(json.dumps({str(k): asdict(v) for k, v in self.table.items()}, indent=1))

    def lookup(self, n_triangles: int) -> Choice | None:
        return self.table.get(bucket_of(n_triangles))

    def tune(self, vertices, triangles, poses, resolution=(512, 512), repeats: int = 3, widths=WIDTHS,
             leaf_sizes=LEAF_SIZES, blocks=BLOCKS) -> Choice:
        """Times frames of this mesh for every (width, leaf size, block shape)."""
        import torch

        from .scene import Canvas, Matcap, Mesh, Scene, camera_for_vfov, render_batch, settings
        b = bucket_of(len(triangles))
        if b in self.table:
            return self.table[b]
        mc = Matcap.make(self.ctx, 0)
        stream = torch.cuda.ExternalStream(self.ctx.stream())
        best = None
        self.trials: list = []
        for width, leaf in [(w, lf) for w in widths for lf in leaf_sizes]:
            try:
                mesh = Mesh(self.ctx, vertices, triangles, leaf, "ploc", width)
            except Exception:  # noqa: BLE001  (a tree too deep for this width's stack is refused)
                continue
            frames = []
            for p in poses:
                sc = Scene()
                sc.add_object(mesh)
                sc.prepare_scene()
                sc.unzoom()
                sc.set_pose(p)
                cv = Canvas(self.ctx, *resolution)
                cv.set_camera(camera_for_vfov(60.0))
                cv.update_settings(settings(shadow=True, edges=False))
                frames.append((cv, sc, mc))
            for threads in blocks:
                self.ctx.set_batch_block(threads)
                render_batch(self.ctx, frames)  # warm-up
                self.ctx.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(repeats):
                    render_batch(self.ctx, frames)
                e1.record(stream)
                e1.synchronize()
                ms = e0.elapsed_time(e1) / (repeats * len(frames))
                self.trials.append((width, leaf, threads, float(ms)))
                if best is None or ms < best.ms_per_frame:
                    best = Choice(b, leaf, threads, float(ms), width)
            for cv, _, _ in frames:
                cv.close()
            mesh.close()
        self.ctx.set_batch_block(best.block_threads)
        self.table[b] = best
        self.save()
        return best


def choose_block(choices: list[Choice], weights: list[float]) -> int:
    """One block shape for a mixed batch: the choice of the heaviest bucket."""
    if not choices:
        return 128
    return choices[int(np.argmax(weights))].block_threads
