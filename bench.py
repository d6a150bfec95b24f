#!/usr/bin/env python3
"""Benchmark of the GB300 render core: Mrays/s and ms/frame at 1920x1080, 1 spp.

Workload (one step = one frame): 64 distinct 32,000-triangle noise-displaced spheres with random affine
transforms over a 2-triangle 1000x1000 ground (2,048,002 triangles, 66 instances), 16 quad lights + 4 point
lights, 20 materials (4 with 1024^2 RGBA8 textures, 5 MIP levels), sky dome; max depth 8, Russian roulette after
depth 3, next-event estimation; frames follow a seeded 8-pose camera path. Seeded synthetic data.

  value     Mrays/s = (primary + extension + shadow rays) / device time of K frames, scene and path state
            resident in HBM, CUDA events on the core's own stream bracketing the K frames.
  e2e       the same metric through the C ABI with a host round trip per frame: camera in, frame (W*H float4)
            read back into pinned host memory.
  roofline  the kernel with the largest share of the frame: algorithmic bytes per launch / measured launch
            duration against the measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle (a restatement of the reference's path tracer) on all host cores.
  svgf      filter-core frames of the same scene and camera path with SVGF + TAA: device time of the six filter
            launches per frame against the measured HBM bandwidth.
  serving   the serving loop on seeded job lists over 4 resident scenes against sequential plain-core renders of
            the same jobs: saturated throughput, and p50 / p99 latency under Poisson arrivals swept over rates.
  ray_queries  closest-hit and any-hit queries of 16M incoherent and 16M secondary-like rays on the same BVH.
  radiance_cache  the cache estimator against the plain one on the same scene and frame size, RMSE and relative MSE
            against a 4096-spp FP64-accumulated plain render, at equal device time and at equal sample count.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun each rank renders its own frames on its own GPU (replicas, weak scaling); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
import zlib

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W_DEFAULT, H_DEFAULT = 1920, 1080
MAX_DEPTH, RR_START = 8, 4
WAVE_TAIL = 5          # path lengths >= 5 run in the persistent tail kernel (setting "waveTail")
LANES = 6              # frames in flight (setting "pipelineFrames")
# ncu dram__bytes_read.sum + dram__bytes_write.sum of three k_extend launches of this workload (waves 1, 2 and 3
# of camera pose 1): 197.65 MB + 197.72 MB + 74.47 MB (profiles/k_extend_spheres_2m_1080p.md)
EXTEND_CAPTURE = {"pose": 1, "waves": (1, 2, 3), "dram_bytes": (150.159872e6 + 39.314432e6) + (146.592e6 + 33.778688e6) + (61.080832e6 + 6.445824e6)}
WORKLOAD = "spheres_2m: 64 x 32k-tri displaced spheres + ground (2,048,002 tris, 66 instances), 16 quad + 4 point lights, " \
           "20 materials (4 textured), sky; 1920x1080 1spp, max depth 8, RR after depth 3, NEE"
METRIC = "Mrays/s @1080p 1spp"
VIEW_BYTES, PARAMS_BYTES = 68, 56     # lh2g_view and lh2g_render_params copied host -> device per frame


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms during the timed region."""
    Q = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
        "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def frame_params(k, W, H):
    from lighthouse2_gb300 import scenes as S
    from lighthouse2_gb300.core import make_params, camera_r0, RP_NEE, RP_DEPTH_W
    view = S.spheres_view(W, H, frame=k % 8)
    p = make_params(W, H, 1, max_depth=MAX_DEPTH, rr_start=RR_START, samples_taken=0, camera_r0=camera_r0(0),
                    flags=RP_NEE | RP_DEPTH_W)
    return view, p


def cpu_baseline(sc, W, H, seconds, threads, core=None, compare=3):
    """The oracle on the host cores; one full frame at a time until `seconds` have elapsed. With `core`, the first
    `compare` oracle frames are checked against the GPU core's frames of the same poses (outside any timed region):
    per path length the extension and connection counts exactly, per-pixel radiance within 1e-4 relative."""
    import numpy as np
    from oracle import bind
    o = bind.Oracle()
    t0 = time.time()
    o.set_scene(sc)
    build_s = time.time() - t0
    rays, elapsed, frames = 0, 0.0, 0
    parity = {"frames_compared": 0, "counters_equal": True, "max_rel_radiance": 0.0}
    while frames == 0 or elapsed < seconds:
        view, p = frame_params(frames, W, H)
        t = time.time()
        r = o.render(view, p, nthreads=threads)
        elapsed += time.time() - t
        c = r["counters"]
        rays += W * H + int(c[:, 0].sum()) + int(c[:, 1].sum())
        if core is not None and frames < compare:
            g = core.render_ex(view, p, counters=True)["counters"]
            acc = core.read_accumulator()
            rel = np.abs(acc - r["accum"]) / np.maximum(np.abs(r["accum"]), 1e-6)
            parity["frames_compared"] += 1
            parity["counters_equal"] &= bool(np.array_equal(g, c))
            parity["max_rel_radiance"] = max(parity["max_rel_radiance"], float(rel.max()))
        frames += 1
    out = {"value": rays / elapsed / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
           "sample": f"{frames} full 1920x1080 1spp frame(s) of the same scene and estimator ({elapsed:.1f} s; oracle BVH build "
                     f"{build_s:.1f} s not timed)", "ms_per_frame": elapsed / frames * 1e3}
    if core is not None:
        parity["ok"] = parity["counters_equal"] and parity["max_rel_radiance"] <= 1e-4
        out["parity_vs_gpu"] = parity
    return out


def bench_config(W, H):
    """The workload both arms run (the same keys in both lines)."""
    return {"workload": WORKLOAD, "width": W, "height": H, "spp": 1, "max_depth": MAX_DEPTH, "rr_start_depth": RR_START,
            "nee": True, "scene_seed": 7, "camera_path": "8 seeded poses, frame k uses pose k % 8",
            "l2": "inputs larger than L2 (scene ~0.6 GB + path state ~0.36 GB resident), no flush"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from lighthouse2_gb300 import scenes as S
    W, H = args.width, args.height
    sc = S.spheres_2m(seed=7)
    threads = os.cpu_count() or 1
    from oracle import bind
    o = bind.Oracle()
    o.set_scene(sc)
    for k in range(args.warmup):
        view, p = frame_params(k, W, H)
        o.render(view, p, nthreads=threads)
    rays, t_total = 0, 0.0
    for k in range(args.steps):
        view, p = frame_params(k, W, H)
        t = time.time()
        r = o.render(view, p, nthreads=threads)
        t_total += time.time() - t
        c = r["counters"]
        rays += W * H + int(c[:, 0].sum()) + int(c[:, 1].sum())
    value = rays / t_total / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(W, H),
            "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} full frames after {args.warmup} warm-up frames"},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def algorithmic_bytes(kind, n_in, n_ext, n_shadow):
    """Bytes a stage must move per launch (path-state and queue traffic; scene data counted per access):
    extend: ray 32 B in + hit 16 B out; shade: the partition's hit record read (16 B) and order written (4 B), then
    the order read back (4 B), path state 48 B + hit 16 B + 5 triangle float4 (80 B) + 2 material float4 (32 B) per
    path, 48 B per extension ray and per connection written; connect: ray 32 B + contribution 16 B."""
    if kind == "extend":
        return n_in * 48
    if kind == "shade":
        return n_in * (16 + 4 + 4 + 48 + 16 + 80 + 32) + 48 * n_ext + 48 * n_shadow
    return n_in * 48


# SVGF bytes per pixel and frame (own-pixel buffers; neighbourhood taps hit L1/L2): prepare reads accumulator
# halves 32, features 16, world position 16, previous world position 16, previous moments 16 and writes shading 16,
# motion 8, moments 16, features 16; a-trous phase 1 reads features, packed light, depth derivatives, moments
# (4 x 16), motion 8, world positions 2 x 16, history 16 and writes 16; phases 2 and 3 read 4 x 16 and write 16;
# TAA reads 16 + 8 + 16 and writes 16; unsharpen reads 16 and writes 16.
SVGF_BYTES_PER_PIXEL = (96 + 56) + (64 + 56 + 16) + 2 * (64 + 16) + (40 + 16) + (16 + 16)


def reduce_replicas(dist, ms, units, device):
    """Replicas (one process per GPU, no collective on the data path): the job's time is the slowest rank's, its
    work the sum over ranks. Returns (max ms, total units)."""
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(u)
    return float(t.item()), int(u.item())


def ray_query_leg(core, sc, n, cpu, name):
    """The ray-query microbenchmark on a scene's BVH: n incoherent rays (origins uniform in the scene box,
    directions uniform on the sphere) and n secondary-like rays (origins on area-weighted surface points,
    cosine-weighted directions), tmax ~ U[0.1, scene diagonal], closest hit and any hit. Rays and results stay in
    device memory (lh2g_trace); CUDA events on the core's stream. The CPU oracle traces 2^20 of the same rays."""
    import numpy as np
    import torch
    from lighthouse2_gb300 import scenes as S
    from oracle import bind
    peak, _ = peaks()
    out = {"workload": f"{name} BVH ({sc.triangle_count:,} triangles, {len(sc.instances)} instances), {n} rays per kind, rays and hits "
                       f"resident on the device"}
    o = None
    if cpu:
        o = bind.Oracle()
        o.set_scene(sc)
    stream = torch.cuda.ExternalStream(core.stream_ptr())
    for kind, seed in (("incoherent", 21), ("secondary", 22)):
        rays = S.random_rays(sc, n, seed=seed, kind=kind)
        d_rays = torch.from_numpy(rays.view(np.uint8).reshape(-1)).cuda()
        for mode, name, bytes_per_ray in ((0, "closest", 48), (1, "any", 36)):
            d_out = torch.empty(n * (16 if mode == 0 else 4), dtype=torch.uint8, device="cuda")
            for _ in range(2):
                core.trace(d_rays.data_ptr(), d_out.data_ptr(), n, mode, core.stream_ptr())
            core.stream_ptr()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps = 5
            with torch.cuda.stream(stream):
                e0.record()
            for _ in range(reps):
                core.trace(d_rays.data_ptr(), d_out.data_ptr(), n, mode, core.stream_ptr())
            with torch.cuda.stream(stream):
                e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            res = d_out.cpu().numpy()
            hits = float((res.view(S.HIT_DTYPE)["prim"] >= 0).mean()) if mode == 0 else float((res.view(np.uint32) != 0).mean())
            gbps = n * bytes_per_ray / (ms / 1e3) / 1e9
            row = {"Mrays_per_s": n / (ms / 1e3) / 1e6, "ms": ms, "hit_fraction": hits, "algorithmic_GBps": gbps, "frac_of_hbm": gbps / peak}
            if o is not None:
                m = 1 << 20
                t = time.time()
                o.trace(rays[:m], mode=mode, nthreads=os.cpu_count() or 1)
                row["cpu_Mrays_per_s"] = m / (time.time() - t) / 1e6
                row["cpu_cores"] = os.cpu_count() or 1
            out[f"{kind}_{name}"] = row
        del d_rays
    return out


def decode_launches(lt_all, frames, counts, waves, W, H):
    """Per stage kind: [summed launch ms, algorithmic bytes, launches] over `frames` frames whose per-launch device
    times are lt_all (per frame: generate, (extend, shade, connect) x waves, tail if used, finalize; a shade slot
    spans the partition of the queue into hits and misses and the shading) and whose per-depth queue sizes are
    counts[frame % 8]."""
    per_frame = 2 + 3 * waves + (1 if waves < MAX_DEPTH else 0)
    per_kind = {k: [0.0, 0, 0] for k in ("extend", "shade", "connect", "tail", "generate", "finalize")}
    for k in range(frames):
        c = counts[k % 8]
        lt = lt_all[k * per_frame:(k + 1) * per_frame]
        n_in = [W * H] + [int(x) for x in c[:-1, 0]]
        per_kind["generate"][0] += lt[0]
        per_kind["finalize"][0] += lt[-1]
        for d in range(waves):
            te, ts, tc = lt[1 + 3 * d], lt[2 + 3 * d], lt[3 + 3 * d]
            for kind, t, b in (("extend", te, algorithmic_bytes("extend", n_in[d], 0, 0)),
                               ("shade", ts, algorithmic_bytes("shade", n_in[d], int(c[d, 0]), int(c[d, 1]))),
                               ("connect", tc, algorithmic_bytes("connect", int(c[d, 1]), 0, 0))):
                per_kind[kind][0] += t
                per_kind[kind][1] += b
                per_kind[kind][2] += 1
        if waves < MAX_DEPTH:   # the tail kernel: every remaining path vertex is traced, shaded and connected
            b = sum(algorithmic_bytes("extend", n_in[d], 0, 0) + algorithmic_bytes("shade", n_in[d], int(c[d, 0]), int(c[d, 1])) +
                    algorithmic_bytes("connect", int(c[d, 1]), 0, 0) for d in range(waves, MAX_DEPTH))
            per_kind["tail"][0] += lt[1 + 3 * waves]
            per_kind["tail"][1] += b
            per_kind["tail"][2] += 1
    return per_kind


def estimators_leg(core, sc, W, H, steps):
    """The OptiX 7 core's estimator (LH2G_RP_OPTIX7: MIS, blue noise for the first 64 samples, one diffuse bounce),
    the same with its light tree (LH2G_RP_LIGHTTREE) on this scene and on a room of 2,144 lights, and PrimeAdaptive
    frames (variance-driven second wave) on the same scene and frame size, seeded synthetic blue-noise tables; device
    time per frame from CUDA events on the core's stream, rays from the frames' counters."""
    import numpy as np
    import torch
    from lighthouse2_gb300 import scenes as S
    from lighthouse2_gb300.core import RenderCore, make_params, camera_r0, RP_NEE, RP_OPTIX7, RP_LIGHTTREE
    core.set_blue_noise(S.synthetic_blue_noise(7))
    stream = torch.cuda.ExternalStream(core.stream_ptr())
    out = {"workload": f"the same scene and camera path, {W}x{H} 1 spp, max depth {MAX_DEPTH}; synthetic blue-noise tables"}

    def timed(render, n):
        core.WaitForRender()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record()
        for k in range(n):
            render(k)
        core.stream_ptr()
        with torch.cuda.stream(stream):
            e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    def o7(k, counters=False):
        p = make_params(W, H, 1, max_depth=MAX_DEPTH, samples_taken=k, camera_r0=camera_r0(k), flags=RP_NEE | RP_OPTIX7,
                        shift=(0x11331445 * (k + 1)) & 0xFFFFFFFF)
        return core.render_ex(S.spheres_view(W, H, frame=k % 8), p, accumulate=k > 0, counters=counters)

    rays = [W * H + int(c[:, 0].sum()) + int(c[:, 1].sum()) for c in (o7(k, True)["counters"] for k in range(8))]
    ms = timed(o7, steps)
    out["optix7"] = {"ms_per_frame": ms, "Mrays_per_s": float(np.mean(rays)) / (ms / 1e3) / 1e6, "rays_per_frame": float(np.mean(rays))}

    def o7t(k, counters=False, c=core, view=lambda k: S.spheres_view(W, H, frame=k % 8)):
        p = make_params(W, H, 1, max_depth=MAX_DEPTH, samples_taken=k, camera_r0=camera_r0(k), flags=RP_NEE | RP_OPTIX7 | RP_LIGHTTREE,
                        shift=(0x11331445 * (k + 1)) & 0xFFFFFFFF)
        return c.render_ex(view(k), p, accumulate=k > 0, counters=counters)

    rays = [W * H + int(c[:, 0].sum()) + int(c[:, 1].sum()) for c in (o7t(k, True)["counters"] for k in range(8))]
    ms = timed(o7t, steps)
    out["optix7_light_tree"] = {"ms_per_frame": ms, "Mrays_per_s": float(np.mean(rays)) / (ms / 1e3) / 1e6, "rays_per_frame": float(np.mean(rays)),
                                "lights": len(sc.tri_lights) + len(sc.point_lights) + len(sc.spot_lights)}
    # a room of 2,144 lights (2,048 area, 64 point, 32 spot): only the light tree renders it
    room = S.lit_room(seed=29, grid=32, n_points=64, n_spots=32)
    rc = RenderCore(0)
    rc.set_scene(room)
    rc.SetTarget(W, H, 1)
    rc.set_blue_noise(S.synthetic_blue_noise(7))
    rstream = torch.cuda.ExternalStream(rc.stream_ptr())
    room_view = lambda k: S.cornell_view(W, H, frame=k % 4)
    rays = [W * H + int(c[:, 0].sum()) + int(c[:, 1].sum()) for c in (o7t(k, True, rc, room_view)["counters"] for k in range(4))]
    rc.WaitForRender()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(rstream):
        e0.record()
    n_room = max(4, steps // 4)
    for k in range(n_room):
        o7t(k, False, rc, room_view)
    rc.stream_ptr()   # joins the frames in flight into the core's stream
    with torch.cuda.stream(rstream):
        e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n_room
    out["light_tree_2144_lights"] = {"workload": f"lit_room(grid=32): Cornell room + 2,048 area, 64 point and 32 spot lights, {W}x{H} 1 spp, "
                                                 f"max depth {MAX_DEPTH}; OptiX 7 estimator with the light tree",
                                     "ms_per_frame": ms, "Mrays_per_s": float(np.mean(rays)) / (ms / 1e3) / 1e6, "rays_per_frame": float(np.mean(rays))}
    rc.close()
    core.set_adaptive_scale(10.0)

    def ad(k):
        p = make_params(W, H, 1, max_depth=MAX_DEPTH, samples_taken=k, camera_r0=camera_r0(2 * k), frame_seed=camera_r0(2 * k + 1), flags=RP_NEE,
                        shift=(0x11331445 * (k + 1)) & 0xFFFFFFFF)
        return core.render_adaptive(S.spheres_view(W, H, frame=0), p, accumulate=k > 0)

    hist = [ad(k) for k in range(24)]   # devScale settles towards the 91-98 % budget band
    t = []
    for k in range(24, 24 + max(4, steps // 4)):
        core.WaitForRender()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record()
        r = ad(k)
        with torch.cuda.stream(stream):
            e1.record()
        torch.cuda.synchronize()
        t.append(e0.elapsed_time(e1))
        hist.append(r)
    last = hist[-1]
    rays_ad = [W * H + r["adaptive_paths"] + int(r["counters"][:, 0].sum()) + int(r["counters"][:, 1].sum()) for r in hist[-len(t):]]
    out["adaptive"] = {"ms_per_frame": float(np.median(t)), "Mrays_per_s": float(np.mean(rays_ad)) / (float(np.median(t)) / 1e3) / 1e6,
                       "second_wave_paths": last["adaptive_paths"], "requested": last["requested"], "budget": W * H,
                       "dev_scale": last["dev_scale"], "frames_before_timing": 24,
                       "note": "one frame at a time (the frame waits for its statistics); rays: both waves' primary, extension and shadow rays"}
    core.set_blue_noise(None)
    return out


def raster_leg(core, sc, W, H, steps, cpu, device):
    """The SoftRasterizer core (lh2g_raster_render) on the path tracer's scenes: the 2M-triangle sphere field at
    W x H (8 camera poses; the core already holds the scene and the target) and the closed room at 512 x 512. Device
    time per frame by CUDA events on the core's stream (no host copies); e2e with every frame's pixels copied to host
    memory; parity: pixels and z-buffer of two poses equal the oracle's bit for bit (outside the timed regions); CPU
    baseline: the oracle's single-threaded restatement (the reference rasterizer is single-threaded) on a few frames."""
    import numpy as np
    import torch
    from lighthouse2_gb300 import scenes as S
    from lighthouse2_gb300.core import RenderCore
    peak, peak_kind = peaks()

    def one(core, views, W, H, sc, label):
        stream = torch.cuda.ExternalStream(core.stream_ptr())
        for k in range(3):
            core.raster(views[k % len(views)], pixels=False)
        st = core.raster(views[0], pixels=False, stats=True)["stats"]
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record()
        for k in range(steps):
            core.raster(views[k % len(views)], pixels=False)
        with torch.cuda.stream(stream):
            e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        t = time.perf_counter()
        for k in range(steps):
            core.raster(views[k % len(views)])
        ms_e2e = (time.perf_counter() - t) / steps * 1e3
        out = {"workload": label, "ms_per_frame": ms, "frames_per_s": 1e3 / ms, "Mtriangles_per_s": st["triangles"] / (ms / 1e3) / 1e6,
               "e2e": {"ms_per_frame": ms_e2e, "Mtriangles_per_s": st["triangles"] / (ms_e2e / 1e3) / 1e6, "d2h_bytes_per_frame": 4 * W * H},
               "stats_pose0": st}
        # bytes a frame must move: every kept triangle's vertices and face normal (60 B), the pixels written (4 B)
        alg = st["triangles"] * 60 + 4 * W * H
        out["roofline"] = {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                           "frac": alg / (ms / 1e3) / 1e9 / peak, "peak_source": peak_kind, "algorithmic_bytes_per_frame": alg,
                           "note": "two passes (depth keys, then colour) and per-triangle setup; issue- and latency-bound, not HBM-bound"}
        if cpu:
            from oracle.bind import Oracle
            o = Oracle()
            o.set_scene(sc)
            same = True
            for k in (0, len(views) // 2):
                r = o.raster(views[k], W, H)
                g = core.raster(views[k], depth=True)
                same = same and np.array_equal(r["pixels"], g["pixels"]) and np.array_equal(r["zbuffer"].view(np.uint32), g["zbuffer"].view(np.uint32))
            n = 3
            t = time.perf_counter()
            for k in range(n):
                o.raster(views[k % len(views)], W, H)
            cms = (time.perf_counter() - t) / n * 1e3
            out["parity_vs_oracle"] = same
            out["cpu_baseline"] = {"value": st["triangles"] / (cms / 1e3) / 1e6, "unit": "Mtriangles/s", "ms_per_frame": cms, "cores": 1,
                                   "kind": "port", "sample": f"{n} frames of the same poses, single-threaded like the reference"}
        return out

    res = {"spheres_2m": one(core, [S.spheres_view(W, H, frame=k) for k in range(8)], W, H, sc,
                             f"spheres_2m (2,048,002 triangles) {W}x{H}, 8 camera poses")}
    cb = S.cornell_sphere(subdiv=6)
    core_c = RenderCore(device)
    core_c.set_scene(cb)
    core_c.SetTarget(512, 512, 1)
    res["cornell"] = one(core_c, [S.cornell_view(512, 512, frame=k) for k in range(8)], 512, 512, cb, "cornell_sphere subdiv 6 (81,932 triangles) 512x512")
    core_c.close()
    return res


def svgf_leg(core, W, H, steps, warmup):
    """Filter-core frames with SVGF + TAA over the 8-pose camera path (Restart every frame, as a moving camera
    does); the filter passes are timed by the core's own events (coreStats.filterTime)."""
    from lighthouse2_gb300 import scenes as S
    core.Setting("maxDepth", MAX_DEPTH)
    core.Setting("rrStartDepth", RR_START)
    core.Setting("filter", 1)
    core.Setting("TAA", 1)
    for k in range(warmup):
        core.Render(S.spheres_view(W, H, frame=k % 8), converge=1)
        core.GetCoreStats()
    filt, rend = [], []
    for k in range(steps):
        core.Render(S.spheres_view(W, H, frame=k % 8), converge=1)
        st = core.GetCoreStats()
        filt.append(st["filterTime"])
        rend.append(st["renderTime"])
    core.Setting("filter", 0)
    ms = statistics.median(filt)
    peak, peak_kind = peaks()
    achieved = SVGF_BYTES_PER_PIXEL * W * H / (ms / 1e3) / 1e9
    return {"workload": f"filter-core frames of the same scene, {W}x{H}, 8-pose camera path, Halton jitter, TAA + unsharpen",
            "filter_ms_per_frame": ms, "filter_ms_min": min(filt), "render_ms_per_frame": statistics.median(rend),
            "launches_per_frame": 6, "algorithmic_bytes_per_pixel": SVGF_BYTES_PER_PIXEL, "achieved_GBps": achieved,
            "peak_GBps": peak, "frac": achieved / peak, "peak_source": peak_kind}


# serving loop queue capacity in paths when the mix's largest job needs less: 8M paths hold about 1.4 GB of queues (164 B per path)
# (well inside a 40 GB path-memory budget at 64 B per path) and let ticks carry several small jobs at once
SERVING_CAPACITY = 1 << 23
SERVING_MIXES = {
    # the serving workload's job distribution: resolution in {256^2, 512^2, 1024^2, 1920x1080}, spp in {1, 4, 16}
    "full": {"res": [(256, 256), (512, 512), (1024, 1024), (1920, 1080)], "spp": [1, 4, 16], "rates": [10, 20, 30, 40, 50, 60, 100, 200]},
    # small interactive requests only, where one job alone leaves most of the GPU idle
    "small": {"res": [(256, 256), (512, 512)], "spp": [1, 4], "rates": [100, 200, 300, 400, 500, 700, 1000, 2000]},
}


def serving_jobs(n, n_scenes, mix, seed=11):
    """Seeded job list: scene, resolution and spp drawn from the mix, depth 4..8, a camera pose per job."""
    import numpy as np
    rng = np.random.default_rng(seed)
    res, spp = SERVING_MIXES[mix]["res"], SERVING_MIXES[mix]["spp"]
    jobs = []
    for k in range(n):
        W, H = res[int(rng.integers(0, len(res)))]
        jobs.append({"scene": int(rng.integers(0, n_scenes)), "W": W, "H": H, "spp": int(rng.choice(spp)),
                     "depth": int(rng.integers(4, 9)), "frame": int(rng.integers(0, 64))})
    return jobs


def serving_leg(args):
    """The serving loop against sequential plain-core renders of the same job lists (one per mix): saturated
    throughput (every job submitted at once), then latency under Poisson arrivals swept over rates. The sequential
    arm is replayed in real time at each rate (first come, first served; one plain core per scene and resolution,
    each holding its target, so a job never waits for a buffer reallocation); the latencies its measured per-job
    service times imply are reported beside. The serving loop runs the sweep with its default admission (smallest
    pending job first, the oldest once one has waited 0.2 s) and first come, first served (setting
    maxWaitSeconds 0). For each arm, the highest tested rate whose p99 latency stays within 2x the p99 of the jobs'
    standalone latencies."""
    import numpy as np
    import torch
    from lighthouse2_gb300 import scenes as S
    from lighthouse2_gb300.core import RenderCore, make_params, camera_r0, RP_NEE, RP_DEPTH_W
    from lighthouse2_gb300.server import RenderServer
    t0 = time.time()
    scene_defs = [("cornell 82k", lambda: S.cornell_sphere(subdiv=6)),
                  ("spheres 16 (512k)", lambda: S.spheres_2m(seed=3, n_spheres=16)),
                  ("spheres 64 (2M)", lambda: S.spheres_2m(seed=7)),
                  ("spheres 128 (4M)", lambda: S.spheres_2m(seed=9, n_spheres=128))]
    cores, scene_objs = [], []
    for name, make in scene_defs:
        core = RenderCore(0)
        sc = make()
        core.set_scene(sc)
        cores.append(core)
        scene_objs.append(sc)
    # the sequential replay's cores: one per (scene, resolution), target set once at the mix's largest spp
    seq_cores = {}

    def seq_core(scene, W, H, spp_max):
        key = (scene, W, H)
        if key not in seq_cores:
            c = RenderCore(0)
            c.set_scene(scene_objs[scene])
            c.SetTarget(W, H, spp_max)
            seq_cores[key] = c
        return seq_cores[key]
    setup_s = time.time() - t0
    pct = lambda a, q: float(np.percentile(a, q) * 1e3)

    def inputs(j):
        view = S.cornell_view(j["W"], j["H"], frame=j["frame"] % 4) if j["scene"] == 0 else S.spheres_view(j["W"], j["H"], frame=j["frame"])
        p = make_params(j["W"], j["H"], j["spp"], max_depth=j["depth"], rr_start=min(4, j["depth"]), camera_r0=camera_r0(0),
                        flags=RP_NEE | RP_DEPTH_W)
        return view, p

    def run_mix(mix, n_jobs):
        jobs = serving_jobs(n_jobs, len(cores), mix)
        # pinned host images for both arms (copies back are part of each job's latency)
        pinned = [torch.empty((j["W"] * j["H"], 4), dtype=torch.float32, pin_memory=True).numpy() for j in jobs]
        for j in jobs[:4]:   # warm-up
            view, p = inputs(j)
            cores[j["scene"]].SetTarget(j["W"], j["H"], j["spp"])
            cores[j["scene"]].render_ex(view, p, counters=False)
            cores[j["scene"]].read_accumulator()
        # sequential plain-core renders: service time of every job alone (render + image read back). SetTarget,
        # which reallocates when the resolution changes, stays outside: a plain-core deployment would keep a
        # target per resolution.
        service, seq_rays = [], 0
        for k, j in enumerate(jobs):
            view, p = inputs(j)
            c = cores[j["scene"]]
            c.SetTarget(j["W"], j["H"], j["spp"])
            c.WaitForRender()
            t = time.perf_counter()
            out = c.render_ex(view, p, counters=True)
            c.read_accumulator_into(pinned[k])
            service.append(time.perf_counter() - t)
            cnt = out["counters"]
            seq_rays += j["W"] * j["H"] * j["spp"] + int(cnt[:, 0].sum()) + int(cnt[:, 1].sum())
        service = np.array(service)
        t_seq = float(service.sum())
        seq_sums = [zlib.crc32(pinned[k]) for k in range(len(jobs))]   # each sequential image's checksum
        cap = max(max(j["W"] * j["H"] * j["spp"] for j in jobs) * 2, args.serving_capacity)
        opts = {"tickBudget": args.serving_tick_budget} if args.serving_tick_budget else {}
        if args.serving_device_loop >= 0:
            opts["deviceLoop"] = args.serving_device_loop
        srv = RenderServer(path_capacity=cap, **opts)
        sids = [srv.add_scene(c) for c in cores]
        for j in jobs[:4]:   # warm-up
            view, p = inputs(j)
            jid = srv.submit_render(sids[j["scene"]], view, p)
            srv.wait(jid)
            srv.release(jid)
        r0 = srv.stats()["raysTraced"]
        t = time.perf_counter()
        ids = []
        for k, j in enumerate(jobs):
            view, p = inputs(j)
            ids.append(srv.submit_render(sids[j["scene"]], view, p, out=pinned[k]))
        for i in ids:
            srv.wait(i)
        t_sat = time.perf_counter() - t
        sat_rays = srv.stats()["raysTraced"] - r0
        same_images = sum(zlib.crc32(pinned[k]) == seq_sums[k] for k in range(len(jobs)))
        for i in ids:
            srv.release(i)
        bound = 2.0 * np.percentile(service, 99)
        spp_max = max(SERVING_MIXES[mix]["spp"])
        for j in jobs:
            seq_core(j["scene"], j["W"], j["H"], spp_max)

        def served(arrivals):
            t_start = time.perf_counter()
            ids = []
            for k, j in enumerate(jobs):
                delay = arrivals[k] - (time.perf_counter() - t_start)
                if delay > 0:
                    time.sleep(delay)
                view, p = inputs(j)
                ids.append(srv.submit_render(sids[j["scene"]], view, p, out=pinned[k]))
            lat = []
            for i in ids:
                ts, ta, td = srv.wait(i)
                lat.append(td - ts)
                srv.release(i)
            return np.array(lat)

        def sequential_replay(arrivals):
            """the plain cores in real time: each job starts at its arrival or when the previous one is done"""
            t_start = time.perf_counter()
            lat = []
            for k, j in enumerate(jobs):
                delay = arrivals[k] - (time.perf_counter() - t_start)
                if delay > 0:
                    time.sleep(delay)
                c = seq_core(j["scene"], j["W"], j["H"], spp_max)
                c.SetTarget(j["W"], j["H"], j["spp"])   # same pixel count: no reallocation
                view, p = inputs(j)
                c.render_ex(view, p, counters=False)
                c.read_accumulator_into(pinned[k])
                lat.append(time.perf_counter() - t_start - arrivals[k])
            return np.array(lat)

        sweep = []
        for rate in SERVING_MIXES[mix]["rates"]:
            arrivals = np.cumsum(np.random.default_rng(5).exponential(1.0 / rate, len(jobs)))
            lat = served(arrivals)
            srv.setting("maxWaitSeconds", 0.0)
            lat_fcfs = served(arrivals)
            srv.setting("maxWaitSeconds", 0.2)
            seq_lat = sequential_replay(arrivals)
            seq_model, free_at = [], 0.0
            for k in range(len(jobs)):
                start = max(arrivals[k], free_at)
                free_at = start + service[k]
                seq_model.append(free_at - arrivals[k])
            seq_model = np.array(seq_model)
            sweep.append({"rate_jobs_per_s": rate, "server_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99)},
                          "server_fcfs_ms": {"p50": pct(lat_fcfs, 50), "p99": pct(lat_fcfs, 99)},
                          "sequential_measured_ms": {"p50": pct(seq_lat, 50), "p99": pct(seq_lat, 99)},
                          "sequential_from_service_times_ms": {"p50": pct(seq_model, 50), "p99": pct(seq_model, 99)},
                          "server_p99_within_bound": bool(np.percentile(lat, 99) <= bound),
                          "server_fcfs_p99_within_bound": bool(np.percentile(lat_fcfs, 99) <= bound),
                          "sequential_p99_within_bound": bool(np.percentile(seq_lat, 99) <= bound),
                          "slowdown_vs_standalone": {"p50": float(np.percentile(lat / service, 50)), "p99": float(np.percentile(lat / service, 99))}})
        sst = srv.stats()
        srv.close()
        ok_srv = [r["rate_jobs_per_s"] for r in sweep if r["server_p99_within_bound"]]
        ok_fcfs = [r["rate_jobs_per_s"] for r in sweep if r["server_fcfs_p99_within_bound"]]
        ok_seq = [r["rate_jobs_per_s"] for r in sweep if r["sequential_p99_within_bound"]]
        return {"jobs": len(jobs), "resolutions": [f"{w}x{h}" for w, h in SERVING_MIXES[mix]["res"]], "spp": SERVING_MIXES[mix]["spp"],
                "path_capacity": cap,
                "standalone_ms": {"p50": pct(service, 50), "p99": pct(service, 99)},
                "sequential": {"jobs_per_s": len(jobs) / t_seq, "Mrays_per_s": seq_rays / t_seq / 1e6, "seconds": t_seq},
                "saturated": {"jobs_per_s": len(jobs) / t_sat, "Mrays_per_s": sat_rays / t_sat / 1e6, "seconds": t_sat,
                              "throughput_vs_sequential": t_seq / t_sat},
                # the served images equal the sequential ones bit for bit (CRC32 of each image), so both arms are
                # compared at the same RMSE: that of the plain estimator at each job's spp
                "images_equal_to_sequential": f"{same_images}/{len(jobs)}",
                "ticks": int(sst["ticks"]), "device_loop_launches": int(sst["loopLaunches"]),
                "poisson_sweep": sweep,
                "rate_at_p99_bound": {"bound_ms": bound * 1e3, "server": max(ok_srv) if ok_srv else None,
                                      "server_fcfs": max(ok_fcfs) if ok_fcfs else None,
                                      "sequential": max(ok_seq) if ok_seq else None}}

    out = {"workload": f"seeded job lists over 4 resident scenes ({', '.join(n for n, _ in scene_defs)}), depth 4..8, one camera pose "
                       f"per job; scenes built once ({setup_s:.0f} s); latency = submit to image in pinned host memory",
           "full": run_mix("full", args.serving_jobs), "small": run_mix("small", 4 * args.serving_jobs)}
    for c in cores + list(seq_cores.values()):
        c.close()
    return out


NRC_FIELD_BOUNDS = ((-100.0, -2.0, -100.0), (100.0, 48.0, 100.0))   # the sphere field and its lights, with margin


def nrc_leg(args, core, name, view, bounds, W, H):
    """Radiance cache against the plain estimator on the core's scene at W x H, measured against a plain render of
    args.nrc_ref_spp samples per pixel accumulated in FP64: RMSE and relative MSE at equal device time (frame counts
    from measured frame times) and at equal sample count, after the cache has trained online for some frames.
    Both estimators run on the same core, scene and camera pose."""
    import numpy as np
    from lighthouse2_gb300.core import make_params, camera_r0, RP_NEE, RP_DEPTH_W
    from lighthouse2_gb300.nrc import RadianceCache

    def P(k, spp=1):
        return make_params(W, H, spp, max_depth=MAX_DEPTH, rr_start=RR_START, samples_taken=k, camera_r0=camera_r0(k), flags=RP_NEE | RP_DEPTH_W)

    t0 = time.time()
    batch = 16
    core.SetTarget(W, H, batch)
    ref = np.zeros((W * H, 3), np.float64)
    for k in range(args.nrc_ref_spp // batch):
        p = P(batch * k, batch)
        p["cameraR0"] = (0x9E3779B9 * (k + 7)) & 0xFFFFFFFF
        core.render_ex(view, p, accumulate=False, counters=False)
        ref += core.read_accumulator()[:, :3]
    ref /= float(args.nrc_ref_spp // batch * batch)
    ref_s = time.time() - t0
    core.SetTarget(W, H, 1)
    cache = RadianceCache(bounds[0], bounds[1], learning_rate=args.nrc_lr, seed=5)
    stats = [core.render_nrc(cache, view, P(100000 + k)) for k in range(args.nrc_warmup)]

    def timed(fn, n=16):
        for k in range(3):
            fn(k)
        core.WaitForRender()
        t = time.perf_counter()
        for k in range(n):
            fn(k)
        core.WaitForRender()
        return (time.perf_counter() - t) / n

    plain = lambda k: core.render_ex(view, P(k), accumulate=k > 0, counters=False)
    cached = lambda k: core.render_nrc(cache, view, P(k), accumulate=k > 0, stats=False)
    t_plain, t_cache = timed(plain), timed(cached)

    def image(fn, n):
        for k in range(n):
            fn(k)
        return core.read_accumulator()[:, :3].astype(np.float64) / n

    def errors(img):
        return {"rmse": float(np.sqrt(np.mean((img - ref) ** 2))), "relmse": float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))}

    box = [[round(float(x), 3) for x in b] for b in bounds]
    out = {"workload": f"{name}, {W}x{H}, depth {MAX_DEPTH}, RR after depth {RR_START - 1}, NEE; reference {args.nrc_ref_spp} spp plain, "
                       f"FP64 sums ({ref_s:.0f} s); cache box {box}, Adam lr {args.nrc_lr}; trained over {args.nrc_warmup} frames "
                       f"first, then online (1/16 of the cached paths, at most 65,536 per frame); relmse = mean of err^2 / (ref^2 + 0.01)",
           "plain_ms_per_frame": t_plain * 1e3, "cache_ms_per_frame": t_cache * 1e3,
           "cache_queries_per_frame": stats[-1][0], "train_samples_per_frame": stats[-1][1],
           "loss_first": float(np.mean([x[2] for x in stats[:5]])), "loss_last": float(np.mean([x[2] for x in stats[-5:]])), "equal_time": {}}
    for n_plain in (4, 16, 64):
        n_cache = max(1, int(round(n_plain * t_plain / t_cache)))
        e_p, e_c = errors(image(plain, n_plain)), errors(image(cached, n_cache))
        out["equal_time"][f"{n_plain}_plain_frames"] = {"cache_frames": n_cache, "plain": e_p, "cache": e_c,
                                                        "rmse_reduction": 1.0 - e_c["rmse"] / e_p["rmse"],
                                                        "relmse_reduction": 1.0 - e_c["relmse"] / e_p["relmse"]}
    e_p, e_c = errors(image(plain, 16)), errors(image(cached, 16))
    out["equal_spp_16"] = {"plain": e_p, "cache": e_c, "rmse_reduction": 1.0 - e_c["rmse"] / e_p["rmse"]}
    # where the plain estimator's error lives: the direct part (emission seen by the camera and light connected at the
    # first vertex: the same estimator at depth 1), which the cache cannot touch (it replaces paths from their second
    # diffuse-led vertex on), against the whole; both against references of args.nrc_ref_spp samples
    def P1(k, spp=1):
        return make_params(W, H, spp, max_depth=1, rr_start=RR_START, samples_taken=k, camera_r0=camera_r0(k), flags=RP_NEE | RP_DEPTH_W)
    core.SetTarget(W, H, batch)
    ref1 = np.zeros((W * H, 3), np.float64)
    for k in range(args.nrc_ref_spp // batch):
        p = P1(batch * k, batch)
        p["cameraR0"] = (0x9E3779B9 * (k + 7)) & 0xFFFFFFFF
        core.render_ex(view, p, accumulate=False, counters=False)
        ref1 += core.read_accumulator()[:, :3]
    ref1 /= float(args.nrc_ref_spp // batch * batch)
    core.SetTarget(W, H, 1)
    direct = lambda k: core.render_ex(view, P1(k), accumulate=k > 0, counters=False)
    img1 = image(direct, 16)
    mse_direct = float(np.mean((img1 - ref1) ** 2))
    out["error_budget_16_frames"] = {"mse_all": e_p["rmse"] ** 2, "mse_direct": mse_direct, "direct_share": mse_direct / max(e_p["rmse"] ** 2, 1e-30),
                                     "note": "direct = the depth-1 estimator (primary emission + one light connection); the cache acts on the rest"}
    cache.close()
    return out


def run_gb300(args):
    import numpy as np
    import torch
    from lighthouse2_gb300 import scenes as S
    from lighthouse2_gb300.core import RenderCore
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    W, H = args.width, args.height
    t0 = time.time()
    sc = S.spheres_2m(seed=7)
    gen_s = time.time() - t0
    core = RenderCore(local)
    core.set_scene(sc)
    build_ms = core.GetCoreStats()["bvhBuildTime"]
    split = world > 1 and args.partition == "rows"
    band = None
    if split:   # each rank renders its band of every frame's rows (lighthouse2_gb300.sharding)
        from lighthouse2_gb300 import sharding
        band = sharding.row_bands(H, world)[rank]
        core.SetTarget(W, band[1], 1)
    else:
        core.SetTarget(W, H, 1)
    core.Setting("waveTail", args.wave_tail)
    core.Setting("pipelineFrames", args.lanes)
    if args.wave_occupancy < 1.0:
        core.Setting("waveOccupancy", args.wave_occupancy)
    core.Setting("sortConnections", args.sort_connections)
    core.Setting("sortRays", args.sort_rays)
    waves = min(MAX_DEPTH, args.wave_tail - 1) if args.wave_tail > 0 else MAX_DEPTH
    stream = torch.cuda.ExternalStream(core.stream_ptr())
    frames = [frame_params(k, W, H) for k in range(8)]
    if split:
        frames = [(v, sharding.band_params(p, rank, world)) for v, p in frames]
    pix = W * (band[1] if split else H)   # primary rays per frame on this rank
    for k in range(args.warmup):
        core.render_ex(*frames[k % 8], counters=False)
    # per-pose queue sizes and traversal work: a frame is a deterministic function of its view and parameters, so
    # the timed frames below have exactly these (checked again after the timed region)
    counts, trav_pose = [], []
    core.enable_launch_timing(True)
    for k in range(8):
        counts.append(core.render_ex(*frames[k], counters=True)["counters"].copy())
        trav_pose.append(np.asarray(core.traversal_stats(), np.float64))
    lt_iso = [float(x) for x in core.launch_times()]   # the counting frames run one at a time: isolated kernels
    core.WaitForRender()
    per_frame = 2 + 3 * waves + (1 if waves < MAX_DEPTH else 0)
    # ---- device-timed region: K frames back to back, scene and path state resident, no host synchronisation ----
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    core.WaitForRender()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record()
    for k in range(args.steps):
        core.render_ex(*frames[k % 8], counters=False)
    core.stream_ptr()   # orders the core's stream after the frames (consecutive frames overlap on internal lanes)
    with torch.cuda.stream(stream):
        e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    lt_all = [float(x) for x in core.launch_times()]
    core.enable_launch_timing(False)
    assert np.array_equal(core.render_ex(*frames[0], counters=True)["counters"], counts[0]), "frame counters are not deterministic"
    assert len(lt_all) == per_frame * args.steps, (len(lt_all), per_frame, args.steps)
    assert len(lt_iso) == per_frame * 8, (len(lt_iso), per_frame)
    per_kind = decode_launches(lt_all, args.steps, counts, waves, W, H)
    per_kind_iso = decode_launches(lt_iso, 8, counts, waves, W, H)
    launches = len(lt_all) + args.steps * waves   # each shading slot launches k_partition and k_shade
    rays, trav, ext_rays, shadow_rays = 0, np.zeros(4, np.float64), 0, 0
    for k in range(args.steps):
        c = counts[k % 8]
        rays += pix + int(c[:, 0].sum()) + int(c[:, 1].sum())
        trav += trav_pose[k % 8]
        ext_rays += pix + int(c[:-1, 0].sum())
        shadow_rays += int(c[:, 1].sum())
    if dist:
        ms, rays = reduce_replicas(dist, ms, rays, "cuda")
        if split:   # the one gather of the partition, after the timed region: the last frame's bands into the whole frame
            whole = sharding.gather_frame(dist, core.read_accumulator(), frames[(args.steps - 1) % 8][1], rank, world, device="cuda")
            assert whole.shape == (W * H, 4)
    value = rays / (ms / 1e3) / 1e6
    # ---- end-to-end through the C ABI: camera and parameters in from host memory, every frame copied back into
    # pinned host memory (lh2g_render_to_host; consecutive frames and their copies overlap), timed on the host ----
    hosts = [torch.empty((pix, 4), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    core.WaitForRender()
    e2e_rays = 0
    t = time.perf_counter()
    for k in range(args.steps):
        core.render_to_host(*frames[k % 8], hosts[k % 2].data_ptr())
        c = counts[k % 8]
        e2e_rays += pix + int(c[:, 0].sum()) + int(c[:, 1].sum())
    core.WaitForRender()
    t_e2e = time.perf_counter() - t
    last = core.read_framebuffer()
    assert np.array_equal(hosts[(args.steps - 1) % 2].numpy(), last), "the last copied frame differs from the device frame"
    e2e_value = e2e_rays * world / t_e2e / 1e6
    rq = None
    if not args.no_rays and rank == 0:
        # the large scene's BVH (most incoherent and secondary-like rays leave the open sphere field) and the small
        # scene's (a room: most rays hit)
        rq = {"spheres_2m": ray_query_leg(core, sc, args.rays, world == 1 and not args.no_cpu_baseline, "spheres_2m")}
        cb = S.cornell_sphere(subdiv=6)
        core_c = RenderCore(local)
        core_c.set_scene(cb)
        rq["cornell"] = ray_query_leg(core_c, cb, args.rays, world == 1 and not args.no_cpu_baseline, "cornell 82k")
        core_c.close()
    svgf = svgf_leg(core, W, H, max(args.steps, 8), args.warmup) if not args.no_svgf else None
    estimators = estimators_leg(core, sc, W, H, max(args.steps, 8)) if not args.no_estimators and rank == 0 else None
    raster = raster_leg(core, sc, W, H, max(args.steps, 8), world == 1 and not args.no_cpu_baseline, local) if not args.no_raster and rank == 0 else None
    serving = serving_leg(args) if (not args.no_serving and rank == 0) else None
    nrc = None
    if not args.no_nrc and rank == 0:
        # the large scene at the bench's frame size; paths there are short (most bounces leave the sphere field for
        # the sky), so the cache also runs on the closed Cornell room, where every path is long
        nrc = {}
        scenes_nrc = args.nrc_scenes.split(",")
        if "spheres_2m" in scenes_nrc:
            nrc["spheres_2m"] = nrc_leg(args, core, "spheres_2m", S.spheres_view(W, H, frame=0), NRC_FIELD_BOUNDS, W, H)
        if "cornell" in scenes_nrc:
            cb = S.cornell_sphere(subdiv=6)
            core_c = RenderCore(local)
            core_c.set_scene(cb)
            core_c.Setting("waveTail", args.wave_tail)
            nrc["cornell"] = nrc_leg(args, core_c, "cornell 82k", S.cornell_view(1024, 1024), cb.bounds, 1024, 1024)
            core_c.close()
    if rank != 0:
        return 0
    frame_ms = sum(v[0] for v in per_kind.values())
    frame_ms_iso = sum(v[0] for v in per_kind_iso.values())
    # the dominant kernel by isolated device time (in the timed region consecutive frames overlap, so launch
    # durations there include time shared with the other frames' kernels)
    dom = max(("extend", "shade", "connect", "tail"), key=lambda k: per_kind_iso[k][0])
    t_dom, b_dom, n_dom = per_kind[dom]
    peak, peak_kind = peaks()
    achieved = (b_dom / n_dom) / ((t_dom / n_dom) / 1e3) / 1e9 if t_dom > 0 else 0.0
    ti, bi, ni = per_kind_iso[dom]
    achieved_iso = (bi / ni) / ((ti / ni) / 1e3) / 1e9 if ti > 0 else 0.0
    traffic = None
    if dom == "extend":
        # DRAM bytes per ray from the ncu capture of the same workload, scaled to this run's mean launch
        rays_captured = sum(W * H if w == 1 else int(counts[EXTEND_CAPTURE["pose"]][w - 2, 0]) for w in EXTEND_CAPTURE["waves"])
        traffic = EXTEND_CAPTURE["dram_bytes"] / rays_captured * (b_dom / n_dom) / algorithmic_bytes("extend", 1, 0, 0)
    line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "strong" if split else "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": bench_config(W, H),
            "details": {"wave_tail": args.wave_tail, "frames_in_flight": args.lanes,
                       "bvh_build_ms": round(build_ms, 2), "scene_generation_s": round(gen_s, 1),
                       "rays_per_frame": rays / args.steps / world,
                       "kernel_ms_per_frame": {k: round(v[0] / args.steps, 4) for k, v in per_kind.items()},
                       "kernel_share": {k: round(v[0] / frame_ms, 4) for k, v in per_kind.items()},
                       "kernel_ms_per_frame_isolated": {k: round(v[0] / 8, 4) for k, v in per_kind_iso.items()},
                       "kernel_share_isolated": {k: round(v[0] / frame_ms_iso, 4) for k, v in per_kind_iso.items()},
                       "queue_sizes_pose1": counts[1].tolist(),
                       "traversal": {"closest_nodes_per_ray": trav[0] / max(ext_rays, 1), "closest_tris_per_ray": trav[1] / max(ext_rays, 1),
                                     "any_nodes_per_ray": trav[2] / max(shadow_rays, 1), "any_tris_per_ray": trav[3] / max(shadow_rays, 1),
                                     "traversal_bytes_per_closest_ray": (trav[0] * 80 + trav[1] * 48) / max(ext_rays, 1),
                                     "extend_traversal_GBps": (trav[0] * 80 + trav[1] * 48) / max(per_kind["extend"][0], 1e-9) / 1e6}},
            "roofline": {"kernel": "k_" + dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                         "achieved_isolated": achieved_iso, "frac_isolated": achieved_iso / peak,
                         "note": "traversal/shading are ALU-issue bound; algorithmic bytes count queue traffic only (48 B per ray); "
                                 "achieved from launches in the timed region, where frames overlap; achieved_isolated from the same "
                                 "kernels of frames rendered one at a time; traffic = ncu DRAM bytes per ray x rays per launch"},
            "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": VIEW_BYTES + PARAMS_BYTES, "d2h_bytes_per_step": pix * 16},
            "gpu_launches": launches * world,
            "clocks": clk}
    if rq is not None:
        line["ray_queries"] = rq
    if svgf is not None:
        line["svgf"] = svgf
    if estimators is not None:
        line["estimators"] = estimators
    if raster is not None:
        line["rasterizer"] = raster
    if serving is not None:
        line["serving"] = serving
    if nrc is not None:
        line["radiance_cache"] = nrc
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sc, W, H, args.cpu_seconds, os.cpu_count() or 1, core=core)
    print(json.dumps(line, default=float), flush=True)
    core.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--width", type=int, default=W_DEFAULT)
    ap.add_argument("--height", type=int, default=H_DEFAULT)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-svgf", action="store_true")
    ap.add_argument("--no-estimators", action="store_true", help="skip the OptiX 7 estimator and adaptive-frame leg")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-nrc", action="store_true")
    ap.add_argument("--no-rays", action="store_true")
    ap.add_argument("--rays", type=int, default=1 << 24, help="rays per kind of the ray-query leg")
    ap.add_argument("--nrc-lr", type=float, default=1e-3)
    ap.add_argument("--nrc-scenes", default="spheres_2m,cornell", help="comma list of spheres_2m, cornell")
    ap.add_argument("--nrc-ref-spp", type=int, default=4096)
    ap.add_argument("--nrc-warmup", type=int, default=200)
    ap.add_argument("--serving-jobs", type=int, default=120)
    ap.add_argument("--serving-capacity", type=int, default=SERVING_CAPACITY,
                    help="queue capacity of the serving loop in paths (at least twice the largest job)")
    ap.add_argument("--serving-tick-budget", type=int, default=0, help="new paths per tick of the serving loop (0: the loop's default)")
    ap.add_argument("--serving-device-loop", type=int, default=-1,
                    help="1: the serving loop's ticks run in a device-side graph loop (its default), 0: host-driven ticks")
    ap.add_argument("--lanes", type=int, default=LANES, help="frames in flight (0 or 1: one at a time)")
    ap.add_argument("--wave-occupancy", type=float, default=1.0, help="share of the GPU a frame's persistent wave kernels launch (setting waveOccupancy)")
    ap.add_argument("--partition", default="replicas", choices=["replicas", "rows"],
                    help="under torchrun: replicas (every rank renders whole frames) or rows (every frame's rows split over the ranks)")
    ap.add_argument("--sort-connections", type=int, default=0, help="group connections by light before the any-hit queries")
    ap.add_argument("--sort-rays", type=int, default=0, help="group bounce waves' extension rays by direction octant")
    ap.add_argument("--no-raster", action="store_true", help="skip the SoftRasterizer leg")
    ap.add_argument("--wave-tail", type=int, default=WAVE_TAIL, help="first path length of the persistent tail kernel (0: off)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
