"""Benchmark: j3d ray-cast frames of the 28.09M-triangle torus at 1920x1080.

One step = one frame (primary ray + closest hit + G-buffer record + shadow ray
+ plain matcap shading, j3d's view::render_scene) for each of 32 seeded
cameras. `value` = Mrays/s (primary + shadow rays) with the mesh, BVH and
canvas resident in HBM; `e2e` = the same through the C-ABI per frame
including the device->host copies of the G-buffer and RGBA image into
pinned host memory (the arrays j3d's view reads back every frame).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl own|reference]

--impl reference times the CPU path on the host cores (the oracle port of
j3d's canvas + qbvh, all threads) on a bounded sample of the same frames.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

W_, H_ = 1920, 1080
N_CAMERAS = 32
NODE_BYTES = 128      # one BVH4 node: 4 child AABBs (96 B) + 4 refs, padded
TRI_BYTES = 48        # 12 B index triple + 36 B of vertices per tested triangle
RECORD_BYTES = 32 + 4  # G-buffer record + RGBA8 per primary ray
# DRAM and L2 bytes of one k_frame launch on this workload (leaf size 2),
# mean of two launches (cameras 8 and 9) from an ncu capture of
# dram__bytes_read.sum + dram__bytes_write.sum and lts__t_sectors.sum x 32 B
# (`ncu --set full -k regex:k_frame -s 40 -c 2 python bench.py --steps 2
# --warmup 1 --no-cpu --no-side`), per BVH builder:
#   ploc: DRAM 483.7 MB, L2 2401.3 MB (SAH top levels + PLOC below 64
#         triangles, cost-optimal collapse, depth-first node order, parked
#         finishes, 6 blocks per SM, next-node prefetch; captured before
#         frames overlapped, with the same traversal: on the overlapped
#         build that multi-pass capture ended in an Xid 31 during ncu's
#         memory save and restore, and it was not repeated)
#   lbvh: DRAM 533.9 MB, L2 1837.1 MB (level-order nodes, finishes in the
#         tracing loop, 5 blocks per SM; an older capture)
FRAME_TRAFFIC = {"ploc": (483_742_752, 2_401_349_440),
                 "lbvh": (463_159_392 + 70_692_880, 1_837_113_990)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        t0 = time.time()
        while not self.rows and time.time() - t0 < 5.0:  # nvidia-smi is up and sampling
            time.sleep(0.005)
        self.first = len(self.rows)  # samples from here on fall in the timed region

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)
        rows = self.rows[getattr(self, "first", 0):] or self.rows
        sm = [float(r[1]) for r in rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) > 8 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


class CpuRenderer:
    """The oracle (port of j3d's CPU path: canvas::render_scene's background
    copy, update_canvas and canvas_to_image over a 4-wide binned-SAH BVH) on
    the same mesh and cameras. Rows run on the oracle's persistent row pool
    over all host cores, like pooled_parallel_for (canvas.cpp:765); frames
    are whole 1920x1080 frames, timed as view.cpp:1263-1267 times them.
    Inputs come from the oracle's own generators: this process never loads
    the product library."""

    def __init__(self, n_threads: int):
        import oracle.oracle as O
        import oracle.workloads as OW
        self.O, self.n_threads = O, n_threads
        V, T, self.poses, self.w, self.h = OW.config1(N_CAMERAS, W_, H_)
        self.m = O.Mesh(V, T, 4, n_threads)
        del V, T
        self.I16 = np.eye(4, dtype=np.float32).reshape(16)
        mn, mx, diag = O.prepare_scene([(self.m.min_bb, self.m.max_bb)], [self.I16])
        _, _, piv = O.unzoom(mn, mx, diag)
        cam = O.camera_with_focal(OW.focal_for_vfov(60.0, 0.768))
        Pi = O.invert_projection_matrix(O.make_projection_matrix(cam, self.w, self.h))
        self.views = [O.view(p, O.invert_orthonormal(p), piv, diag, Pi, cam.near_clipping_plane) for p in self.poses]
        self.st = O.settings(shadow=True, edges=False)
        self.mc, self.cav = O.make_matcap(0)
        self.bg = O.fill_background(self.w, self.h)
        self.pix = O.fresh_pixels(self.w, self.h)
        self.im = np.zeros((self.h, self.w), np.uint32)

    def frame(self, cam: int):
        """One whole frame of camera `cam`: (rays, seconds, node visits, triangle tests)."""
        O = self.O
        self.pix[...] = O.fresh_pixels(self.w, self.h)
        t0 = time.perf_counter()
        _, _, s = O.render_frame(self.pix, self.im, self.bg, [(self.m, self.I16, 1)], self.views[cam], self.st,
                                 self.mc, self.cav, n_threads=self.n_threads)
        return s.rays, time.perf_counter() - t0, s.node_visits, s.tri_tests


CPU_FRAMES_PER_STEP = 8  # 4 steps cover the 32 cameras once


def run_reference(args):
    """CPU arm: the oracle port of j3d's renderer on all host cores, whole
    frames, CPU_FRAMES_PER_STEP cameras per step (step k renders cameras
    8k .. 8k+7 mod 32, warm-up steps included in the count)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle.oracle as O
    O.build()
    n_threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    cpu = CpuRenderer(n_threads)
    setup_s = time.perf_counter() - t0
    step_s, rays, visits, tests, frame_s = [], 0, 0, 0, []
    for i in range(args.warmup + args.steps):
        cams = [(i * CPU_FRAMES_PER_STEP + k) % N_CAMERAS for k in range(CPU_FRAMES_PER_STEP)]
        r = [cpu.frame(c) for c in cams]
        if i >= args.warmup:
            step_s.append(sum(x[1] for x in r))
            frame_s += [x[1] for x in r]
            rays += sum(x[0] for x in r)
            visits += sum(x[2] for x in r)
            tests += sum(x[3] for x in r)
    secs = float(np.sum(step_s))
    v = rays / secs / 1e6
    sample = (f"{CPU_FRAMES_PER_STEP} whole 1920x1080 frames per step (primary + shadow + plain shading, "
              f"background copy included), cameras cycled over the 32; {args.steps} timed steps, {rays} rays in "
              f"{secs:.2f} s on the oracle's persistent row pool over {n_threads} threads; the reference itself "
              "cannot be built (jtk absent, SSE-only canvas)")
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "Mrays/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(secs / max(1, args.steps) * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded displaced torus, no dataset)", "config": CONFIG,
            "cpu_baseline": {"value": round(v, 4), "unit": "Mrays/s", "cores": n_threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(v, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "details": {"step_ms": [round(x * 1e3, 1) for x in step_s],
                        "frame_ms_mean": round(float(np.mean(frame_s)) * 1e3, 2),
                        "frame_ms_p50": round(float(np.median(frame_s)) * 1e3, 2),
                        "oracle_bvh_build_s": round(cpu.m.build_seconds, 3),
                        "setup_s": round(setup_s, 2),
                        "oracle_node_visits_per_ray": round(visits / max(1, rays), 4),
                        "oracle_tri_tests_per_ray": round(tests / max(1, rays), 4)}}
    print(json.dumps(line), flush=True)
    return 0


METRIC = "Mrays/s & frame ms, 28M-tri mesh @1080p, 1 GB300, learned vs plain vs CPU qbvh (plain GPU path)"
CONFIG = {"workload": "torus R=1 r=0.35 5300x2650 grid, 28,090,000 tris / 14,045,000 verts, 32 cameras r 2.5-4, "
                      "1920x1080, primary + shadow, plain red-wax matcap", "cameras": N_CAMERAS,
          "resolution": [W_, H_], "l2": "inputs larger than L2 (BVH + leaf triangles ~1.9 GB)"}


def side_workloads(ctx, mesh, wl, args) -> dict:
    """Short runs of the other configurations in the same process, so that one
    bench run measures them beside the headline (each guarded: a failure is
    reported in its entry and does not stop the headline line)."""
    import torch

    from j3d_gb300 import (Batch, Canvas, Matcap, Mesh, Scene, camera_for_vfov, settings, workloads as Wk)
    stream = torch.cuda.ExternalStream(ctx.stream())
    out = {}

    def ev_ms(fn, reps):
        fn()
        ctx.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    # batched frames: 64 meshes (10k-2M tris) x 16 cameras, mixed resolutions,
    # all 1024 frames in one graph-captured persistent launch
    try:
        from j3d_gb300 import build_meshes
        b = Wk.config2()
        t0 = time.perf_counter()
        meshes = build_meshes(ctx, b.meshes, rebuildable=True)  # concurrently, 8 builds in flight
        ctx.synchronize()
        build_s = time.perf_counter() - t0
        mc = Matcap.make(ctx, 0)
        frames, k = [], 0
        for i, m in enumerate(meshes):
            for c in range(16):
                sc = Scene()
                sc.add_object(m, db_id=i + 1)
                sc.prepare_scene()
                sc.unzoom()
                sc.set_pose(b.poses[i][c])
                cv = Canvas(ctx, *b.resolutions[k])
                cv.set_camera(camera_for_vfov(60.0))
                cv.set_background_color()
                cv.update_settings(settings(shadow=True, edges=False))
                frames.append((cv, sc, mc))
                k += 1
        g = Batch(ctx, frames)
        ms = ev_ms(g.launch, 3)
        prim = sum(cv.width * cv.height for cv, _, _ in frames)
        rays = prim + sum(cv.count_hits()[0] for cv, _, _ in frames)
        g.close()
        # all 64 builds, then all 1024 frames, in one graph launch
        g = Batch(ctx, frames, rebuild=True)
        ms_rb = ev_ms(g.launch, 3)
        out["batch_config2"] = {"frames": len(frames), "ms_per_launch": round(ms, 3),
                                "mrays_s": round(rays / ms / 1e3, 1), "rays": rays,
                                "triangles": int(sum(len(T) for _, T in b.meshes)),
                                "builds_64_wall_s": round(build_s, 3),
                                "builds_and_frames_one_graph_ms": round(ms_rb, 3),
                                "builds_in_graph_ms": round(ms_rb - ms, 3)}
        g.close()
        for cv, _, _ in frames:
            cv.close()
        for m in meshes:
            m.close()
    except Exception as e:  # noqa: BLE001
        out["batch_config2"] = {"error": repr(e)[:300]}

    # serving: 8 resident tori 200k..28.09M tris (the headline mesh is the
    # 28M one), Poisson arrivals at 400/s, plain path
    try:
        from j3d_gb300.serve import RenderServer, poisson_requests
        srv = RenderServer(ctx, 150 << 30, max_slots=64, max_in_flight=2)
        for i, t in enumerate([200_000, 500_000, 1_000_000, 2_000_000, 5_000_000, 10_000_000, 20_000_000]):
            assert srv.add_mesh(f"torus{t}", *Wk.torus(*Wk.torus_grid_for(t), seed=Wk.SEED_BASE + 4 + i))
        srv.meshes["torus28090000"] = mesh  # resident already
        srv.mesh_bytes += int(mesh.info().device_bytes)
        names = list(srv.meshes)
        srv.run(poisson_requests(64, 1600.0, names, seed=Wk.SEED_BASE + 40), realtime=True)
        # this process holds the headline's multi-GB arrays and their Python
        # objects: collect once and freeze the heap, as a server process
        # would, so that a collection pausing the host loop does not land in
        # the latency tail (the dedicated serving run measures p99 1.8 ms;
        # here, with the heap unfrozen, 8.6-26.9 ms)
        gc.collect()
        gc.freeze()
        st = srv.run(poisson_requests(600, 400.0, names, seed=Wk.SEED_BASE + 41), realtime=True)
        gc.unfreeze()
        out["serve_config4_plain"] = {"requests": st.requests, "rate_per_s": 400, "p50_ms": round(st.p50_ms, 3),
                                      "p99_ms": round(st.p99_ms, 3), "frames_per_s": round(st.frames_per_s, 1),
                                      "mean_batch": round(st.mean_batch, 2),
                                      "peak_hbm_gb": round(st.peak_bytes / 2**30, 2)}
        for c in list(srv.pool.free.values()):
            for cv in c:
                cv.close()
        for name, m in srv.meshes.items():
            if m is not mesh:
                m.close()
    except Exception as e:  # noqa: BLE001
        out["serve_config4_plain"] = {"error": repr(e)[:300]}

    # learned tmax on the headline mesh: a 4096-cluster network trained on
    # 16M rays, then one 1080p frame with learned vs plain primary hits
    try:
        from j3d_gb300.learned import Learned
        net = Learned(ctx, mesh, cluster_depth=6, batch=16384, seed=Wk.SEED_BASE + 3)
        loss, acc, train_s = net.train(16_000_000, 2.0, 5.0)
        sc = Scene()
        sc.add_object(mesh)
        sc.prepare_scene()
        sc.unzoom()
        sc.set_pose(wl.poses[0])
        mc = Matcap.make(ctx, 0)
        cvs = []
        for _ in range(2):
            cv = Canvas(ctx, W_, H_)
            cv.set_camera(camera_for_vfov(60.0))
            cv.set_background_color()
            cv.update_settings(settings(shadow=True, edges=False))
            cvs.append(cv)
        ms_plain = ev_ms(lambda: cvs[0].render_frame(sc, mc), 5)
        ms_learned = ev_ms(lambda: net.render_frame(cvs[1], sc, mc), 3)
        same = bool(np.array_equal(cvs[0].get_pixels().view(np.uint8), cvs[1].get_pixels().view(np.uint8)))
        out["learned_config3"] = {"train_rays": 16_000_000, "train_s": round(train_s, 2),
                                  "train_loss": round(loss, 4), "train_top1": round(acc, 4),
                                  "frame_ms_plain": round(ms_plain, 3), "frame_ms_learned": round(ms_learned, 3),
                                  "learned_over_plain": round(ms_plain / ms_learned, 4),
                                  "frames_identical": same}
        for cv in cvs:
            cv.close()
        net.close()
    except Exception as e:  # noqa: BLE001
        out["learned_config3"] = {"error": repr(e)[:300]}
    return out


def run_own(args):
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from j3d_gb300 import (Canvas, Context, Matcap, Mesh, Scene, build as B, camera_for_vfov, settings,
                           workloads as Wk)
    B.build()
    wl = Wk.config1(N_CAMERAS, W_, H_)
    ctx = Context(local)
    t0 = time.perf_counter()
    mesh = Mesh(ctx, wl.vertices, wl.triangles, args.leaf, args.build, args.width)
    build_wall = time.perf_counter() - t0
    info = mesh.info()
    # three more builds give the steady build time (their median: the level
    # loops synchronise with the host, so one build can catch host noise)
    build_samples = []
    for _ in range(3):
        mesh2 = Mesh(ctx, wl.vertices, wl.triangles, args.leaf, args.build, args.width)
        build_samples.append(mesh2.info().build_ms)
        mesh2.close()
    build_ms = float(np.median(build_samples))
    sc = Scene()
    sc.add_object(mesh)
    sc.prepare_scene()
    sc.unzoom()
    cv = Canvas(ctx, W_, H_)
    cv.set_camera(camera_for_vfov(60.0))
    cv.set_background_color()
    cv.update_settings(settings(shadow=True, edges=False))
    mc = Matcap.make(ctx, 0)
    stream = torch.cuda.ExternalStream(ctx.stream())

    # rays per frame (primary + shadow) and the GPU's own traversal counters
    prim = W_ * H_
    shadow_rays = []
    ctx.set_counting(True)
    for p in wl.poses:
        sc.set_pose(p)
        cv.render_frame(sc, mc)
        px = cv.get_pixels()
        shadow_rays.append(int((px["object_id"] != 0xFFFFFFFF).sum()))
    gvis, gtests = ctx.read_counters(reset=True)
    ctx.set_counting(False)
    rays_per_step = prim * N_CAMERAS + sum(shadow_rays)

    def step():
        for p in wl.poses:
            sc.set_pose(p)
            cv.render_frame(sc, mc)

    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    ctx.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    from j3d_gb300.multi import reduce_timing
    if ws > 1:
        torch.distributed.barrier()
    ms, total_rays = reduce_timing(ms, rays_per_step)
    value = total_rays / (ms / 1e3) / 1e6

    # the same step with every frame run after the previous one has ended
    # (no overlapped frames), outside the timed region above
    ctx.set_frame_overlap(False)
    step()
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    step()
    s1.record(stream)
    s1.synchronize()
    serial_frame_ms = s0.elapsed_time(s1) / N_CAMERAS
    ctx.set_frame_overlap(True)

    # per-frame kernel time (one k_render launch per frame in plain mode)
    fe0 = [torch.cuda.Event(enable_timing=True) for _ in wl.poses]
    fe1 = [torch.cuda.Event(enable_timing=True) for _ in wl.poses]
    for i, p in enumerate(wl.poses):
        sc.set_pose(p)
        fe0[i].record(stream)
        cv.render_frame(sc, mc)
        fe1[i].record(stream)
    ctx.synchronize()
    frame_ms = [a.elapsed_time(b) for a, b in zip(fe0, fe1)]

    # the same frames with the opt-in rasterised primary hits (identical
    # images; the default traces because this measures slower): one warm-up
    # step and one timed step, outside the timed region above
    from j3d_gb300 import PRIMARY_AUTO, PRIMARY_RASTER
    ctx.set_primary_mode(PRIMARY_RASTER)
    step()
    r0 = torch.cuda.Event(enable_timing=True)
    r1 = torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    step()
    r1.record(stream)
    r1.synchronize()
    raster_frame_ms = r0.elapsed_time(r1) / N_CAMERAS if cv.last_primary() == PRIMARY_RASTER else None
    ctx.set_primary_mode(PRIMARY_AUTO)

    # end to end through the C-ABI: render + G-buffer and image into pinned
    # host memory; four canvases (and host buffers) rotate, so that frame k's
    # download (copy stream, 0.42 ms for 74.6 MB) overlaps the next frames'
    # renders (context stream) and the host never waits on a copy that the
    # next frame needs to be queued behind (with two, that wait left the GPU
    # a gap per frame: 0.72-0.74 ms per frame against 0.61)
    n_rot = 4
    canv = [cv]
    for _ in range(n_rot - 1):
        c2 = Canvas(ctx, W_, H_)
        c2.set_camera(camera_for_vfov(60.0))
        c2.set_background_color()
        c2.update_settings(settings(shadow=True, edges=False))
        canv.append(c2)
    hp = [torch.empty(H_ * W_ * 32, dtype=torch.uint8, pin_memory=True) for _ in range(n_rot)]
    hi = [torch.empty(H_ * W_ * 4, dtype=torch.uint8, pin_memory=True) for _ in range(n_rot)]

    def e2e_step():
        for k, p in enumerate(wl.poses):
            c = canv[k % n_rot]
            c.download_wait()  # the host buffers of this canvas are free again
            sc.set_pose(p)
            c.render_frame(sc, mc)
            c.download_async(hp[k % n_rot], hi[k % n_rot])
        for c in canv:
            c.download_wait()
        ctx.synchronize()

    e2e_step()
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_value = rays_per_step / e2e_s / 1e6
    # host -> device per frame: the FrameParams kernel argument block (the
    # instance table is unchanged between frames and not re-sent)
    h2d = N_CAMERAS * 512
    d2h = N_CAMERAS * (H_ * W_ * 36)

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return 0

    side = {} if args.no_side else side_workloads(ctx, mesh, wl, args)

    # CPU baseline: the reference arm's own routine (the oracle port, whole
    # frames on all host cores) in a fresh process, so that no CUDA context,
    # torch threads or product library share the host with it; four warm-up
    # steps cover the 32 cameras once, eight timed steps twice
    cpu = None
    if not args.no_cpu:
        env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
        rr = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "8",
                             "--warmup", "4"], capture_output=True, text=True, env=env)
        ref = json.loads(rr.stdout.strip().splitlines()[-1]) if rr.returncode == 0 else None
        if ref and "value" in ref:
            cpu = ref
    peak, peak_kind = peaks()
    # per-ray counts of the reference algorithm (the oracle's 4-wide SAH BVH)
    # over every full frame of this workload, from tests/golden/traffic.json
    # (tests/golden/make_traffic.py); the GPU tree's own counts if it is absent
    traffic_file = ROOT / "tests" / "golden" / "traffic.json"
    ref_counts = json.loads(traffic_file.read_text()).get("config1") if traffic_file.exists() else None
    if ref_counts and args.leaf == 2 and ref_counts["frames"] == N_CAMERAS:
        node_per_ray = ref_counts["node_visits_per_ray"]
        tri_per_ray = ref_counts["tri_tests_per_ray"]
        model_src = "oracle BVH4 SAH counts over all 32 frames, tests/golden/traffic.json"
    else:
        node_per_ray = gvis / rays_per_step
        tri_per_ray = gtests / rays_per_step
        model_src = "GPU BVH counts"
    alg_bytes = prim * N_CAMERAS * RECORD_BYTES + rays_per_step * (node_per_ray * NODE_BYTES + tri_per_ray * TRI_BYTES)
    # k_frame's time per launch: the timed region's time per frame (a frame's
    # kernel overlaps the tail of the one before it)
    achieved = alg_bytes / (ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded displaced torus, no dataset)",
        "config": CONFIG,
        "details": dict(parallelism="replicas" if ws > 1 else "single GPU",
                       frame_ms_mean=round(ms / N_CAMERAS, 4), frame_ms_p50=round(float(np.median(frame_ms)), 4),
                       frame_ms_p50_note="per-frame timing events between the frames keep them from overlapping",
                       frame_ms_without_overlap=round(serial_frame_ms, 4),
                       raster_primary_frame_ms_mean=None if raster_frame_ms is None else round(raster_frame_ms, 4),
                       rays_per_step=rays_per_step, shadow_ray_fraction=round(sum(shadow_rays) / (prim * N_CAMERAS), 4),
                       bvh_build_ms=round(build_ms, 3), bvh_build_ms_samples=[round(b, 2) for b in build_samples],
                       bvh_first_build_wall_s=round(build_wall, 3),
                       bvh_nodes=info.n_nodes, bvh_depth=info.max_depth, leaf_size=args.leaf,
                       bvh_builder=args.build, bvh_width=args.width,
                       mesh_device_bytes=int(info.device_bytes),
                       bvh_build_mtris_per_s=round(28_090_000 / (build_ms / 1e3) / 1e6, 1),
                       # T (12 + 36) B read + T 24 B boxes + nodes x 128 B written, per build ms
                       bvh_build_alg_gbs=round((28_090_000 * (48 + 24) + info.n_nodes * 128) / (build_ms / 1e3) / 1e9, 1),
                       gpu_node_visits_per_ray=round(gvis / rays_per_step, 3),
                       gpu_tri_tests_per_ray=round(gtests / rays_per_step, 3)),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": FRAME_TRAFFIC[args.build][0] if args.leaf == 2 and args.width == 4 else None,
                     "traffic_l2": FRAME_TRAFFIC[args.build][1] if args.leaf == 2 and args.width == 4 else None,
                     "traffic_note": "DRAM (and L2) bytes per k_frame launch: mean of two launches (cameras 8 "
                                     "and 9) of one ncu capture; the algorithmic bytes per launch are bytes_per_ray "
                                     "x rays_per_step / 32; achieved divides them by the timed region's time per "
                                     "frame (each frame's kernel overlaps the tail of the one before)",
                     "kernel": "k_frame (primary + shadow + shading, one launch per frame)", "peak_kind": peak_kind,
                     "bytes_per_ray": round(alg_bytes / rays_per_step, 1),
                     "node_visits_per_ray": round(node_per_ray, 3), "tri_tests_per_ray": round(tri_per_ray, 3),
                     "per_ray_model": "36 B per primary ray + node_visits*128 B + tri_tests*48 B (" + model_src + ")"},
        "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "other_configs": side,
        "gpu_launches": N_CAMERAS * args.steps,  # one k_frame per frame
        "clocks": clk,
    }
    if cpu:
        line["cpu_baseline"] = dict(cpu["cpu_baseline"])
        line["cpu_baseline"]["sample"] = ("separate process: " + cpu["cpu_baseline"]["sample"] +
                                          f"; oracle BVH build {cpu['details']['oracle_bvh_build_s']:.2f} s")
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_batch(args):
    """Batched frames (64 meshes of uneven size x 16 cameras, mixed resolutions):
    per-frame launches vs one persistent launch vs a replayed CUDA graph, with
    leaf size and block shape from the autotuner."""
    import torch

    from j3d_gb300 import (Batch, Canvas, Context, Matcap, Mesh, Scene, build as B, camera_for_vfov,
                           render_batch, settings, workloads as Wk)
    from j3d_gb300.autotune import Autotuner, bucket_of
    B.build()
    wl = Wk.config2(args.batch_meshes, args.batch_cameras)
    ctx = Context(0)
    tuner = Autotuner(ctx)
    t0 = time.perf_counter()
    buckets = {}
    for V, T in wl.meshes:
        buckets.setdefault(bucket_of(len(T)), (V, T))
    for b, (V, T) in sorted(buckets.items()):
        tuner.tune(V, T, wl.poses[0][:4], resolution=(384, 384), repeats=2)
    tune_s = time.perf_counter() - t0
    weights = {b: 0.0 for b in buckets}
    for V, T in wl.meshes:
        weights[bucket_of(len(T))] += len(T)
    heavy = max(weights, key=weights.get)
    ctx.set_batch_block(tuner.table[heavy].block_threads)
    width = tuner.table[heavy].width  # one width per batch: the heaviest bucket's
    from j3d_gb300 import build_meshes
    t0 = time.perf_counter()
    serial = [Mesh(ctx, V, T, tuner.table[bucket_of(len(T))].leaf_size, "ploc", width) for V, T in wl.meshes]
    ctx.synchronize()
    serial_s = time.perf_counter() - t0
    for m in serial:
        m.close()
    t0 = time.perf_counter()
    meshes = build_meshes(ctx, wl.meshes, [tuner.table[bucket_of(len(T))].leaf_size for _, T in wl.meshes], width,
                          rebuildable=True)
    ctx.synchronize()
    build_s = time.perf_counter() - t0
    build_ms = sum(m.info().build_ms for m in meshes)
    mc = Matcap.make(ctx, 0)
    cam = camera_for_vfov(60.0)
    frames = []
    k = 0
    for i, m in enumerate(meshes):
        for c in range(args.batch_cameras):
            sc = Scene()
            sc.add_object(m, db_id=i + 1)
            sc.prepare_scene()
            sc.unzoom()
            sc.set_pose(wl.poses[i][c])
            cv = Canvas(ctx, *wl.resolutions[k])
            cv.set_camera(cam)
            cv.set_background_color()
            cv.update_settings(settings(shadow=True, edges=False))
            frames.append((cv, sc, mc))
            k += 1
    stream = torch.cuda.ExternalStream(ctx.stream())
    render_batch(ctx, frames)
    ctx.synchronize()
    prim = sum(cv.width * cv.height for cv, _, _ in frames)
    shadow = sum(cv.count_hits()[0] for cv, _, _ in frames)
    rays = prim + shadow

    def timed(fn, reps):
        for _ in range(args.warmup):
            fn()
        ctx.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    ms_single = timed(lambda: [cv.render_frame(sc, m) for cv, sc, m in frames], args.steps)
    ms_batch = timed(lambda: render_batch(ctx, frames), args.steps)
    g = Batch(ctx, frames)
    ms_graph = timed(g.launch, args.steps)
    g.close()
    # the configuration as specified: all builds, then all frames, one graph launch
    g = Batch(ctx, frames, rebuild=True)
    ms_rebuild = timed(g.launch, args.steps)
    g.close()
    line = {"metric": "Mrays/s, batched frames (config 2)", "value": round(rays / (ms_graph / 1e3) / 1e6, 3),
            "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms_graph, 3), "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded icospheres and tori)",
            "config": {"workload": wl.name, "frames": len(frames), "triangles_total": int(sum(len(T) for _, T in wl.meshes)),
                       "rays_per_step": rays, "pixels_per_step": prim,
                       "per_frame_launches_ms": round(ms_single, 3), "one_launch_ms": round(ms_batch, 3),
                       "graph_ms": round(ms_graph, 3), "per_frame_launches_mrays_s": round(rays / ms_single / 1e3, 3),
                       "one_launch_mrays_s": round(rays / ms_batch / 1e3, 3),
                       "builds_ms_device": round(build_ms, 2), "builds_wall_s": round(build_s, 3),
                       "builds_and_frames_one_graph_ms": round(ms_rebuild, 3),
                       "builds_in_graph_ms": round(ms_rebuild - ms_graph, 3),
                       "builds_one_by_one_wall_s": round(serial_s, 3),
                       "autotune_s": round(tune_s, 2),
                       "autotune": {str(b): {"width": c.width, "leaf": c.leaf_size, "block": c.block_threads,
                                             "ms_per_frame": round(c.ms_per_frame, 4)}
                                    for b, c in sorted(tuner.table.items())},
                       "block_threads": tuner.table[heavy].block_threads, "bvh_width": width}}
    print(json.dumps(line), flush=True)
    return 0


def run_serve(args):
    """Serving (config 4): 8 resident tori (200k .. 28M triangles), Poisson
    render requests at 400/s, resolutions {512^2, 1280x720, 1920x1080},
    admission by HBM footprint (150 GB, then a cap that binds)."""
    from j3d_gb300 import Context, build as B, workloads as Wk
    from j3d_gb300.serve import CanvasPool, RenderServer, poisson_requests
    from j3d_gb300.learned import Learned
    B.build()
    ctx = Context(0)
    sizes = [200_000, 500_000, 1_000_000, 2_000_000, 5_000_000, 10_000_000, 20_000_000, 28_090_000]
    out = {}
    meshes = []
    for i, t in enumerate(sizes):
        nu, nv = (5300, 2650) if t == 28_090_000 else Wk.torus_grid_for(t)
        meshes.append((f"torus{t}", Wk.torus(nu, nv, seed=Wk.SEED_BASE + 4 + i)))
    nets = {}
    train_s = 0.0
    for cap_name, mode in (("150GB", "plain"), ("binding", "plain"), ("150GB", "learned")):
        srv = RenderServer(ctx, 150 << 30, max_slots=64, max_in_flight=2)
        for name, (V, T) in meshes:
            assert srv.add_mesh(name, V, T)
        if mode == "learned":
            # one 4096-cluster network per mesh, trained on the GPU on rays of
            # seeded cameras (the serving cameras' radius range)
            for name in srv.meshes:
                net = Learned(ctx, srv.meshes[name], cluster_depth=6, batch=16384, seed=Wk.SEED_BASE + 3)
                _, _, secs = net.train(args.serve_train_rays, 2.5, 4.0)
                train_s += secs
                srv.attach_learned(name, net)
                nets[name] = net
        if cap_name == "binding":
            srv.cap = srv.mesh_bytes + 3 * CanvasPool.canvas_bytes(1920, 1080)
        names = list(srv.meshes)
        warm = poisson_requests(64, args.serve_rate * 4, names, seed=Wk.SEED_BASE + 40)
        srv.run(warm, realtime=True)
        reqs = poisson_requests(args.serve_requests, args.serve_rate, names, seed=Wk.SEED_BASE + 41)
        st = srv.run(reqs, realtime=True)
        out[f"{mode}_{cap_name}"] = {
            "p50_ms": round(st.p50_ms, 3), "p99_ms": round(st.p99_ms, 3), "mean_ms": round(st.mean_ms, 3),
            "frames_per_s": round(st.frames_per_s, 1), "batches": st.batches, "mean_batch": round(st.mean_batch, 2),
            "peak_hbm_gb": round(st.peak_bytes / 2**30, 2), "cap_gb": round(srv.cap / 2**30, 2),
            "canvases": srv.pool.count, "resident_mesh_gb": round(srv.mesh_bytes / 2**30, 2)}
        for net in nets.values():
            net.close()
        nets.clear()
        for c in list(srv.pool.free.values()):
            for cv in c:
                cv.close()
        for m in srv.meshes.values():
            m.close()
    out["learned_training_s_total"] = round(train_s, 1)
    line = {"metric": "serving p50/p99 frame latency (ms) and frames/s (config 4)",
            "value": out["plain_150GB"]["p99_ms"], "unit": "ms (p99)", "n_gpus": 1, "higher_is_better": False,
            "dtype": "f32", "data": "synthetic (seeded tori, Poisson arrivals)",
            "config": {"workload": "8 tori 200k..28.09M tris, Poisson %.0f req/s, %d requests, "
                                   "512^2 / 1280x720 / 1920x1080, primary + shadow" % (args.serve_rate, args.serve_requests),
                       "runs": out}}
    print(json.dumps(line), flush=True)
    return 0


def primary_rays(pose, pinv, w, h, near, t_near):
    """j3d primary rays (canvas.cpp:773-782) of one camera, float32 numpy."""
    cs = np.asarray(pose, np.float32).reshape(4, 4)  # column-major storage: rows are columns
    P = np.asarray(pinv, np.float32).reshape(4, 4)
    xs = (np.float32(2) * ((np.arange(w, dtype=np.float32) + np.float32(0.5)) / np.float32(w)) - np.float32(1))
    ys = (np.float32(2) * ((np.arange(h, dtype=np.float32) + np.float32(0.5)) / np.float32(h)) - np.float32(1))
    sx, sy = np.meshgrid(xs, ys)
    s = np.stack([sx, sy, np.full_like(sx, near), np.ones_like(sx)], -1).reshape(-1, 4)
    d = s @ P
    d[:, 3] = 0
    d = d @ cs
    rays = np.zeros(len(d), [("orig", "<f4", 4), ("dir", "<f4", 4), ("t_near", "<f4"), ("t_far", "<f4")])
    rays["orig"][:] = cs[3]
    rays["dir"][:] = d
    rays["t_near"] = t_near
    rays["t_far"] = np.finfo(np.float32).max
    return rays


def run_build(args):
    """The config-1 mesh's BVH builds alone: warm builds of the 28.09M-triangle
    torus with the default builder (one CUDA graph with device-driven level
    loops) and with the LBVH builder, CUDA-event times from the library."""
    from j3d_gb300 import Context, Mesh, build as B, workloads as Wk
    B.build()
    wl = Wk.config1(N_CAMERAS, W_, H_)
    ctx = Context(0)
    out = {}
    for name in ("ploc", "lbvh"):
        ms = []
        for k in range(args.warmup + args.steps):
            m = Mesh(ctx, wl.vertices, wl.triangles, args.leaf, name, args.width)
            if k >= args.warmup:
                ms.append(m.info().build_ms)
            info = m.info()
            m.close()
        out[name] = {"ms_median": round(float(np.median(ms)), 3), "ms": [round(x, 2) for x in ms],
                     "nodes": int(info.n_nodes), "depth": int(info.max_depth)}
    nt = len(wl.triangles)
    med = out["ploc"]["ms_median"]
    line = {"metric": "BVH build ms, 28.09M-triangle torus (config 1)", "value": med, "unit": "ms", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": med, "higher_is_better": False,
            "dtype": "f32", "data": "synthetic (seeded displaced torus)",
            "config": {"workload": "torus R=1 r=0.35 5300x2650 grid, 28,090,000 tris", "leaf": args.leaf,
                       "width": args.width, "default_builder": out["ploc"], "lbvh_builder": out["lbvh"],
                       "mtris_per_s": round(nt / (med / 1e3) / 1e6, 1),
                       "alg_gbs": round((nt * (48 + 24) + out["ploc"]["nodes"] * 128) / (med / 1e3) / 1e9, 1)}}
    print(json.dumps(line), flush=True)
    return 0


def run_learned(args):
    """Learned tmax (config 3): the 4096-cluster network trained on 50M rays
    of the 28.09M-triangle torus, then learned vs plain closest hit on the
    primary rays of 4 cameras at 1920x1080 (hit ids must be identical)."""
    import torch

    from j3d_gb300 import (Context, Mesh, SceneObject, build as B, camera_for_vfov, find_closest,
                           invert_projection_matrix, make_projection_matrix, workloads as Wk)
    from j3d_gb300.learned import Learned
    B.build()
    wl = Wk.config1(N_CAMERAS, W_, H_)
    if args.learned_mesh == "icosphere":  # a small case of the same kernels (profiling)
        wl.vertices, wl.triangles = Wk.icosphere(7, Wk.SEED_BASE + 76)
    ctx = Context(0)
    # the LBVH: its depth-6 subtrees are Morton-ordered ranges of the mesh,
    # the "4096 spatial clusters (Morton order)" of this configuration
    mesh = Mesh(ctx, wl.vertices, wl.triangles, args.leaf, "lbvh")
    net = Learned(ctx, mesh, cluster_depth=6, batch=16384, lr=2e-3, seed=Wk.SEED_BASE + 3)
    loss, acc, train_s = net.train(args.learned_rays, 2.0, 5.0)
    info = mesh.info()
    diag = max(info.max_bb[k] - info.min_bb[k] for k in range(3))
    cam = camera_for_vfov(60.0)
    pinv = invert_projection_matrix(make_projection_matrix(cam, W_, H_))
    host = np.concatenate([primary_rays(p, pinv, W_, H_, cam.near_clipping_plane, np.float32(diag) / np.float32(100))
                           for p in wl.poses[:4]])
    n = len(host)
    d_rays = torch.from_numpy(host.view(np.uint8)).cuda()
    d_plain = torch.zeros(n * 24, dtype=torch.uint8, device="cuda")
    d_learn = torch.zeros(n * 24, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream())
    objs = [SceneObject(mesh, None, 1)]

    def timed(fn, reps=3):
        fn()
        ctx.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    from j3d_gb300 import _ffi
    from j3d_gb300.scene import _instances
    L = _ffi.lib()
    inst = _instances(objs)

    def plain():
        assert L.j3dg_find_closest(ctx.h, inst, 1, d_rays.data_ptr(), n, d_plain.data_ptr()) == 0

    def learned():
        assert L.j3dg_learned_find_closest(net.h, d_rays.data_ptr(), n, d_learn.data_ptr()) == 0

    ms_plain = timed(plain)
    ms_learned = timed(learned)
    ctx.set_counting(True)
    ctx.read_counters(reset=True)
    plain()
    ctx.synchronize()
    pv, pt = ctx.read_counters(reset=True)
    learned()
    ctx.synchronize()
    lv, lt = ctx.read_counters(reset=True)
    ctx.set_counting(False)
    _, phase = net.find_closest_stats(host[:n])
    hp = d_plain.cpu().numpy().view(_ffi.HIT_DTYPE)
    hl = d_learn.cpu().numpy().view(_ffi.HIT_DTYPE)
    same = bool(all(np.array_equal(hp[f], hl[f]) for f in ("found", "distance", "u", "v", "object_id")))
    # the network alone: top-2 prediction time on the same rays
    d_top2 = torch.zeros(2 * n, dtype=torch.int32, device="cuda")
    d_top2_layered = torch.zeros(2 * n, dtype=torch.int32, device="cuda")
    ms_predict = timed(lambda: L.j3dg_learned_predict_impl(net.h, d_rays.data_ptr(), n, d_top2.data_ptr(), 1))
    ms_layered = timed(lambda: L.j3dg_learned_predict_impl(net.h, d_rays.data_ptr(), n, d_top2_layered.data_ptr(), 0))
    agree = float((d_top2.view(-1, 2)[:, 0] == d_top2_layered.view(-1, 2)[:, 0]).float().mean())
    flops = 2.0 * (256 * 128 + 3 * 128 * 128 + 128 * 4096) * n
    pk = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak_tf, peak_kind = (float(pk["bf16_tflops"]), "measured") if "bf16_tflops" in pk else (1900.0, "fallback")
    tf_fused = flops / (ms_predict / 1e3) / 1e12
    line = {"metric": "learned vs plain closest-hit Mrays/s (config 3)", "value": round(n / ms_learned / 1e3, 3),
            "unit": "Mrays/s", "n_gpus": 1, "higher_is_better": True, "dtype": "bf16 network / f32 traversal",
            "data": "synthetic (seeded displaced torus; training rays from cameras at radius 2-5)",
            "config": {"workload": "torus 28.09M tris, primary rays of 4 cameras at 1920x1080 (%d rays)" % n,
                       "clusters": net.n_clusters, "params": net.n_params, "train_rays": args.learned_rays,
                       "train_seconds": round(train_s, 2), "train_final_loss": round(loss, 4),
                       "train_top1_accuracy": round(acc, 4),
                       "plain_ms": round(ms_plain, 3), "learned_ms": round(ms_learned, 3),
                       "network_predict_ms": round(ms_predict, 3),
                       "network_tflops": round(tf_fused, 2),
                       "network_layered_tcgen05_ms": round(ms_layered, 3),
                       "network_layered_tflops": round(flops / (ms_layered / 1e3) / 1e12, 2),
                       "fused_vs_layered_top1_agreement": round(agree, 5),
                       "plain_mrays_s": round(n / ms_plain / 1e3, 3),
                       "learned_over_plain": round(ms_plain / ms_learned, 4),
                       "hits_identical": same, "hit_fraction": round(float(hp["found"].mean()), 4),
                       "plain_node_visits_per_ray": round(pv / n, 3), "learned_node_visits_per_ray": round(lv / n, 3),
                       "plain_tri_tests_per_ray": round(pt / n, 3), "learned_tri_tests_per_ray": round(lt / n, 3),
                       "learned_cluster_phase_visits_per_ray": round(phase["cluster_visits"] / n, 3),
                       "learned_exact_phase_visits_per_ray": round(phase["exact_visits"] / n, 3),
                       "exact_phase_visit_saving_vs_plain": round(1 - phase["exact_visits"] / max(1, pv), 4)},
            "roofline": {"bound": "tensor", "achieved": round(tf_fused, 1), "peak": peak_tf, "unit": "TFLOP/s",
                         "frac": round(tf_fused / peak_tf, 4), "traffic": None, "peak_kind": peak_kind,
                         "kernel": "k_learned_fused (features, 5 tcgen05 layers, running top-2; 1.196 MFLOP per ray)"}}
    print(json.dumps(line), flush=True)
    return 0


def run_ingest(args):
    """Mesh ingest: the 28.09M-triangle torus written as a binary PLY (the
    Stanford scan layout: float xyz, uchar count + int indices) and as a
    binary STL, read from the file straight into a device mesh with its BVH
    (j3dg_geometry_read_file + j3dg_mesh_build_geometry), wall clock per
    load. The file is in the page cache (written just before). An OBJ of
    2.1M triangles times the host-threaded text path. The CPU baseline
    parses the same PLY with numpy and builds the oracle's BVH on the host
    cores."""
    import shutil
    import tempfile

    from j3d_gb300 import Context, Geometry, mesh_from_geometry, workloads as W
    from oracle import formats as F

    ctx = Context(0)
    V, T = W.torus()
    tmp = Path(tempfile.mkdtemp(prefix="j3dg_ingest_"))
    out = {}
    try:
        files = {"ply": tmp / "torus.ply", "stl": tmp / "torus.stl"}
        files["ply"].write_bytes(F.write_ply_triangles_fast(V, T))
        files["stl"].write_bytes(F.write_stl_binary(V, T))
        Vo, To = W.torus(1030, 1030, seed=W.SEED_BASE + 75)
        files["obj"] = tmp / "torus2M.obj"
        with open(files["obj"], "w") as f:
            f.write("".join(f"v {a!r} {b!r} {c!r}\n" for a, b, c in Vo.astype(np.float64).tolist()))
            f.write("".join(f"f {a + 1} {b + 1} {c + 1}\n" for a, b, c in To.tolist()))
        for fmt, path in files.items():
            times, infos, builds = [], [], []
            for rep in range(args.warmup + args.steps):
                t0 = time.perf_counter()
                g = Geometry.read_file(ctx, path)
                m = mesh_from_geometry(ctx, g, args.leaf)
                dt = time.perf_counter() - t0
                if rep >= args.warmup:
                    times.append(dt)
                    infos.append(g.info)
                    builds.append(m.info().build_ms)
                m.close()
                g.close()
            i = infos[-1]
            size = path.stat().st_size
            out[fmt] = {"file_mb": round(size / 1e6, 1), "triangles": int(i.n_triangles),
                        "vertices": int(i.n_vertices), "load_and_build_ms": round(1e3 * float(np.median(times)), 1),
                        "read_ms": round(float(np.median([x.read_ms for x in infos])), 1),
                        "decode_ms": round(float(np.median([x.decode_ms for x in infos])), 1),
                        "bvh_build_ms_device": round(float(np.median(builds)), 2),
                        "device_decoded": bool(i.device_decoded),
                        "file_gb_per_s": round(size / float(np.median(times)) / 1e9, 2)}
        cpu = None
        if not args.no_cpu:
            import oracle.oracle as O
            O.build()
            t0 = time.perf_counter()
            data = files["ply"].read_bytes()
            enc, elements, at = F.parse_ply_header(data)
            nv, nf = elements[0]["count"], elements[1]["count"]
            Vc = np.frombuffer(data, "<f4", 3 * nv, at).reshape(-1, 3)
            fr = np.frombuffer(data, np.dtype([("n", "u1"), ("i", "<i4", 3)]), nf, at + 12 * nv)
            assert (fr["n"] == 3).all()
            Tc = fr["i"].astype(np.uint32)
            t_parse = time.perf_counter() - t0
            m = O.Mesh(np.ascontiguousarray(Vc), Tc, 4, os.cpu_count() or 1)
            cpu = {"value": round(1e3 * (t_parse + m.build_seconds), 1), "unit": "ms",
                   "cores": os.cpu_count() or 1, "kind": "port",
                   "sample": f"numpy parse of the same PLY ({1e3 * t_parse:.0f} ms) + the oracle's binned-SAH "
                             f"BVH4 build on all host threads ({1e3 * m.build_seconds:.0f} ms), one load"}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    line = {"metric": "mesh ingest: file -> device mesh + BVH (load + build ms, 28.09M-tri binary PLY)",
            "value": out["ply"]["load_and_build_ms"], "unit": "ms", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": False, "dtype": "f32",
            "data": "synthetic (seeded displaced torus written to a local file, page cache warm)",
            "config": {"workload": "torus 28,090,000 tris as binary PLY (532 MB) and binary STL (1.4 GB); "
                                   "torus 2.12M tris as OBJ", "formats": out,
                       "reference_published": "README.md:37-45 (Lucy, 28.06M tris, other hardware): PLY load "
                                              "2.52 s, STL 4.53 s, OBJ 34 s; BVH build 3.6 s"},
            "gpu_launches": None}
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    return 0


def run_objects(args):
    """Scenes of many objects (the two-level structure of canvas.cpp:762):
    n instances of four meshes (icosphere L5, tori of 200k and 50k triangles,
    icosphere L4) under seeded rigid transforms, 1920x1080 primary + shadow
    + plain shading from 16 cameras, walked through the per-frame top-level
    BVH and object after object (the same context, switched)."""
    import torch

    from j3d_gb300 import Canvas, Context, Matcap, Mesh, Scene, build as B, camera_for_vfov, settings, workloads as Wk
    B.build()
    ctx = Context(0)
    rng = np.random.default_rng(Wk.SEED_BASE + 9)
    meshes = [Mesh(ctx, *Wk.icosphere(5, Wk.SEED_BASE + 90)), Mesh(ctx, *Wk.torus(448, 224, seed=Wk.SEED_BASE + 91)),
              Mesh(ctx, *Wk.torus(224, 112, seed=Wk.SEED_BASE + 92)), Mesh(ctx, *Wk.icosphere(4, Wk.SEED_BASE + 93))]
    stream = torch.cuda.ExternalStream(ctx.stream())
    out = {}
    for n in (16, 256, 1024):
        sc = Scene()
        spread = 1.5 * n ** (1 / 3)
        for k in range(n):
            q = rng.normal(size=4)
            q /= np.linalg.norm(q)
            w, x, y, z = q
            M = np.eye(4)
            M[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                         [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                         [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
            M[:3, 3] = rng.uniform(-spread, spread, size=3)
            sc.add_object(meshes[k % 4], M.T.reshape(16).astype(np.float32), 1 + k)
        sc.prepare_scene()
        sc.unzoom()
        poses = Wk.cameras(16, Wk.SEED_BASE + 94, 2.2 * spread, 3.0 * spread)
        cv = Canvas(ctx, W_, H_)
        cv.set_camera(camera_for_vfov(60.0))
        cv.set_background_color()
        cv.update_settings(settings(shadow=True, edges=False))
        mc = Matcap.make(ctx, 0)
        res = {}
        for top in (True, False):
            ctx.set_top_level(top)
            for p in poses[:4]:
                sc.set_pose(p)
                cv.render_frame(sc, mc)
            ctx.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for p in poses:
                sc.set_pose(p)
                cv.render_frame(sc, mc)
            e1.record(stream)
            e1.synchronize()
            ctx.synchronize()
            res["top_level" if top else "object_loop"] = round(e0.elapsed_time(e1) / len(poses), 3)
        ctx.set_top_level(True)
        hits = int((cv.get_pixels()["object_id"] != 0xFFFFFFFF).sum())
        out[n] = dict(res, last_frame_hit_pixels=hits)
        cv.close()
    print(json.dumps({"workload": "objects", "metric": "frame ms, 1920x1080 primary + shadow + shading",
                      "frames_per_point": 16, "by_instances": out}), flush=True)
    return 0


def run_config0(args):
    """The small configuration: icosphere level 6 (81,920 triangles) at
    1024x768, camera at distance 3, primary + shadow + plain shading; GPU
    build and frame beside the CPU oracle's build and frame (all host
    cores, persistent row pool), in one process (the CPU leg runs after the
    GPU leg has finished)."""
    import torch

    import oracle.oracle as O
    import oracle.workloads as OW
    from j3d_gb300 import Canvas, Context, Matcap, Mesh, Scene, build as B, camera_for_vfov, settings
    B.build()
    O.build()
    V, T, poses, w, h = OW.config0()
    ctx = Context(0)
    builds = []
    for _ in range(4):
        m = Mesh(ctx, V, T)
        builds.append(m.info().build_ms)
    sc = Scene()
    sc.add_object(m)
    sc.prepare_scene()
    sc.unzoom()
    sc.set_pose(poses[0])
    cv = Canvas(ctx, w, h)
    cv.set_camera(camera_for_vfov(60.0))
    cv.set_background_color()
    cv.update_settings(settings(shadow=True, edges=False))
    mc = Matcap.make(ctx, 0)
    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(args.warmup):
        cv.render_frame(sc, mc)
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        cv.render_frame(sc, mc)
    e1.record(stream)
    e1.synchronize()
    gpu_ms = e0.elapsed_time(e1) / args.steps
    hits = int((cv.get_pixels()["object_id"] != 0xFFFFFFFF).sum())
    rays = w * h + hits
    n_threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    om = O.Mesh(V, T, 4, n_threads)
    cpu_build_s = time.perf_counter() - t0
    mn, mx, diag = O.prepare_scene([(om.min_bb, om.max_bb)], [np.eye(4, dtype=np.float32).reshape(16)])
    _, _, piv = O.unzoom(mn, mx, diag)
    cam = O.camera_with_focal(OW.focal_for_vfov(60.0, 0.768))
    Pi = O.invert_projection_matrix(O.make_projection_matrix(cam, w, h))
    v = O.view(poses[0], O.invert_orthonormal(poses[0]), piv, diag, Pi, cam.near_clipping_plane)
    st = O.settings(shadow=True, edges=False)
    omc, cav = O.make_matcap(0)
    bg = O.fill_background(w, h)
    cpu_ms = []
    for k in range(8):
        pix = O.fresh_pixels(w, h)
        im = np.zeros((h, w), np.uint32)
        t0 = time.perf_counter()
        O.render_frame(pix, im, bg, [(om, np.eye(4, dtype=np.float32).reshape(16), 1)], v, st, omc, cav,
                       n_threads=n_threads)
        if k >= 2:
            cpu_ms.append((time.perf_counter() - t0) * 1e3)
    same = bool(np.array_equal(pix.view(np.uint8), cv.get_pixels().view(np.uint8)))
    line = {"workload": "config0", "metric": "Mrays/s & frame ms, icosphere L6 81,920 tris @1024x768, primary + shadow",
            "gpu": {"frame_ms": round(gpu_ms, 4), "mrays_s": round(rays / gpu_ms / 1e3, 1),
                    "build_ms_median_warm": round(float(np.median(builds[1:])), 3)},
            "cpu_oracle": {"frame_ms": round(float(np.median(cpu_ms)), 2),
                           "mrays_s": round(rays / float(np.median(cpu_ms)) / 1e3, 2),
                           "build_s": round(cpu_build_s, 3), "cores": n_threads},
            "rays_per_frame": rays, "gbuffer_identical": same}
    print(json.dumps(line), flush=True)
    return 0


def run_pointcloud(args):
    """Point-cloud splat after each headline frame: the 28.09M-triangle torus
    frame at 1920x1080 for each of the 32 cameras, then its 14.045M vertices
    pushed 1 % outward as a coloured point cloud drawn by
    j3dg_canvas_render_pointclouds. `value` = Mpoints/s of the splat pass
    alone (CUDA events around it); the CPU baseline runs the oracle's
    sequential splat on one camera."""
    import torch

    from j3d_gb300 import (Canvas, Context, Matcap, Mesh, PointCloud, Scene, camera_for_vfov, settings,
                           workloads as Wk)
    wl = Wk.config1(N_CAMERAS, W_, H_)
    ctx = Context(0)
    mesh = Mesh(ctx, wl.vertices, wl.triangles, args.leaf)
    Vp = (wl.vertices * np.float32(1.01)).astype(np.float32)
    rng = np.random.default_rng(0x6A3D0005)
    colors = rng.integers(0, 2 ** 32, len(Vp), dtype=np.uint64).astype(np.uint32)
    pc = PointCloud(ctx, Vp, colors)
    sc = Scene()
    sc.add_object(mesh)
    sc.add_pointcloud(pc, None, 2)
    sc.prepare_scene()
    sc.unzoom()
    cv = Canvas(ctx, W_, H_)
    cv.set_camera(camera_for_vfov(60.0))
    cv.set_background_color()
    cv.update_settings(settings(shadow=True, edges=False))
    mc = Matcap.make(ctx, 0)
    stream = torch.cuda.ExternalStream(ctx.stream())
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in wl.poses]
    splat_ms = []
    drawn = 0
    for rep in range(args.warmup + args.steps):
        for i, p in enumerate(wl.poses):
            sc.set_pose(p)
            cv.render_frame(sc, mc)
            ev[i][0].record(stream)
            cv.render_pointclouds(sc)
            ev[i][1].record(stream)
        ctx.synchronize()
        if rep >= args.warmup:
            splat_ms += [a.elapsed_time(b) for a, b in ev]
    px = cv.get_pixels()
    drawn = int((px["db_id"] == 2).sum())
    ms = float(np.mean(splat_ms))
    value = len(Vp) / (ms / 1e3) / 1e6
    line = {"metric": "point-cloud splat Mpoints/s (14.05M points over the 28M-tri frame, 1920x1080)",
            "value": round(value, 1), "unit": "Mpoints/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms * N_CAMERAS, 3), "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (torus vertices scaled by 1.01, seeded colours)",
            "config": {"workload": "torus 28.09M tris frame + 14,045,000-point cloud, 32 cameras, 1920x1080",
                       "splat_ms_mean": round(ms, 4), "splat_ms_p50": round(float(np.median(splat_ms)), 4),
                       "points_drawn_last_camera": drawn,
                       "kernels_per_cloud": "k_splat (one 64-bit atomicMax per visible point) + k_resolve; "
                                            "k_zinit once per call"},
            "gpu_launches": 3 * N_CAMERAS * args.steps}
    if not args.no_cpu:
        import oracle.oracle as O
        O.build()
        P, _ = cv.get_projection()
        sc.set_pose(wl.poses[-1])
        cv.render_frame(sc, mc)
        pix = cv.get_pixels().reshape(H_, W_).copy()
        im = cv.get_image().reshape(H_, W_).copy()
        t0 = time.perf_counter()
        O.render_pointclouds(pix, im, P, sc.coordinate_system_inv, 0.1, [(Vp, colors, np.eye(4, dtype=np.float32).reshape(16), 2)])
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": round(len(Vp) / dt / 1e6, 2), "unit": "Mpoints/s", "cores": 1, "kind": "port",
                                "sample": f"oracle sequential splat of the 14.05M points over one camera's frame ({dt:.2f} s)"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="own", choices=["own", "reference"])
    ap.add_argument("--leaf", type=int, default=2)
    ap.add_argument("--width", type=int, default=4, choices=[2, 4, 8], help="BVH width of the headline mesh")
    ap.add_argument("--build", default="ploc", choices=["ploc", "lbvh"], help="BVH builder of the headline mesh")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-side", action="store_true", help="skip the short runs of the other configurations")
    ap.add_argument("--workload", default="torus",
                    choices=["torus", "batch", "serve", "learned", "ingest", "pointcloud", "objects", "config0", "build"],
                    help="torus: the headline 28M-triangle frames; batch: config-2 batched frames; "
                         "serve: config-4 request serving")
    ap.add_argument("--serve-rate", type=float, default=400.0)
    ap.add_argument("--serve-requests", type=int, default=1200)
    ap.add_argument("--serve-train-rays", type=int, default=4_000_000, help="training rays per mesh (learned serving)")
    ap.add_argument("--learned-rays", type=int, default=50_000_000)
    ap.add_argument("--learned-mesh", default="torus", choices=["torus", "icosphere"],
                    help="icosphere: a 327,680-triangle mesh instead of the 28M torus (a small case of the same "
                         "kernels, for profiling)")
    ap.add_argument("--batch-meshes", type=int, default=64)
    ap.add_argument("--batch-cameras", type=int, default=16)
    args = ap.parse_args()
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "learned":
        return run_learned(args)
    if args.workload == "ingest":
        return run_ingest(args)
    if args.workload == "pointcloud":
        return run_pointcloud(args)
    if args.workload == "objects":
        return run_objects(args)
    if args.workload == "config0":
        return run_config0(args)
    if args.workload == "build":
        return run_build(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_own(args)


if __name__ == "__main__":
    sys.exit(main())
