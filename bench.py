#!/usr/bin/env python3
"""Throughput of the GB300 path tracer on the medium-scene workload.

Workload (one step = one render launch): 256 spheres, 64 materials, 8 point
lights, 1920x1080, 8 bounces, 16 samples per pixel per launch = 33,177,600
paths (one path = one pixel-sample).  Synthetic seeded scene (scenes.config1);
the camera is set through the public API (atx_set_camera) as a caller would.

Metric: Mpaths/s, whole job (N replicas on N GPUs, one process per GPU,
`scaling: weak`).  The path state of a launch (four lanes of 8.3 Mi paths,
about 1 GB each) is larger than L2, so every step streams its working set
through HBM; no explicit flush.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the reference's per-pixel path restated on the CPU
(the oracle's literal-order build, OpenMP over all host cores) on a bounded
sample of the same workload: the reference's perPixel is device code only, so
it has no CPU path of its own; its own CUDA kernel, built from its sources, is
timed in the main line's ref_cuda_kernel.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

# Algorithmic HBM bytes of the wavefront path state (minimal records):
BYTES_PER_EXTENSION = 104   # ray record (origin, direction, throughput, seed: 44 B) written and read, hit record 2 x 8
BYTES_PER_SHADOW = 80       # shadow-ray record (origin, direction, contribution, path: 40 B) written and read
BYTES_PER_PIXEL = 52        # primary hit record written and read (2 x 8), accumulator read and written (2 x 16), RGBA8 (4)
CAMERA_BYTES = 148          # the camera a step sends (inverse projection and view, eye, viewport: kernel parameters)


def hbm_peak_gbs():
    """Measured copy bandwidth of the GB300s (MEASURED_PEAKS.json, driver-written), else the fallback."""
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0
METRIC = "Mpaths/s per GB300"
UNIT = "Mpaths/s"
WORKLOAD_MEDIUM = ("medium scene: 256 spheres, 64 materials, 8 lights, 1920x1080, 8 bounces, "
                   "16 spp per launch (one step = one launch)")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------- dist utils

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = False
        if self.world > 1:
            import torch.distributed as dist
            backend = os.environ.get("ATX_BENCH_BACKEND", "nccl")
            if backend == "nccl":
                import torch
                torch.cuda.set_device(self.local_rank)
            dist.init_process_group(backend=backend)
            self.pg = True

    def barrier(self):
        if self.pg:
            import torch.distributed as dist
            dist.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        import torch.distributed as dist
        dev = f"cuda:{self.local_rank}" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            import torch.distributed as dist
            dist.destroy_process_group()


# ------------------------------------------------------------------ clocks

class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        """Starts sampling every 100 ms; the caller keeps the GPU on the workload until the timed region."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        rows = [l.split(",") for l in out.strip().splitlines() if l.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "window": "untimed launches of the same workload for 0.4 s before and 0.25 s after the timed "
                          "region keep every sample under load"}


def soak(r, spp: int, seconds: float):
    """Untimed launches of the workload for about `seconds`, around the timed region while the clock
    sampler runs (the timed region itself is too short for more than a sample or two)."""
    t_end = time.perf_counter() + seconds
    while time.perf_counter() < t_end:
        for _ in range(32):
            r.render_frames(spp)
        r.synchronize()


# ------------------------------------------------------------ CPU baseline

def cpu_reference(sc, target_s: float, threads: int = 0):
    """Times the literal-order oracle (reference expressions, OpenMP) on the first rows of the image,
    all samples of one launch, sized to about target_s seconds.  Returns (Mpaths/s, sample text,
    threads, Mrays/s)."""
    import numpy as np

    from oracle import pyoracle as po

    po.build()
    view = po.view_for(sc)
    nthreads = threads or po.max_threads()

    def rows(nrows):
        ys = (np.arange(nrows, dtype=np.int64) * sc.height) // nrows       # evenly spaced rows
        return (ys[:, None] * sc.width + np.arange(sc.width)[None, :]).reshape(-1).astype(np.uint32)

    def run(nrows):
        px = rows(nrows)
        t0 = time.perf_counter()
        _, _, st = po.render(sc.spheres, sc.materials, sc.lights, view, max_bounces=sc.max_bounces, spp=sc.spp,
                             pixels=px, mode=po.LITERAL, threads=nthreads)
        return time.perf_counter() - t0, st, len(px)

    nrows = 4
    dt, _, _ = run(nrows)
    nrows = int(min(sc.height, max(2, nrows * target_s / max(dt, 1e-3))))
    dt, st, npx = run(nrows)
    paths = npx * sc.spp
    rays = st["ext_rays"] + st["shadow_rays"]
    sample = (f"{nrows} evenly spaced rows ({npx} pixels) x {sc.spp} spp of the {sc.width}x{sc.height} frame "
              f"= {paths} paths, {dt:.1f} s")
    return paths / dt / 1e6, sample, nthreads, rays / dt / 1e6


# -------------------------------------------------------------- our arm

def run_ours(args, dist: Dist):
    import ctypes as C

    import numpy as np
    import torch

    import ataraxia_gb300 as atx
    from ataraxia_gb300 import _native as N
    from ataraxia_gb300 import scenes

    dev = dist.local_rank
    torch.cuda.set_device(dev)
    sc = scenes.config1()
    cam = atx.Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction)
    settings = atx.Settings(accumulation=True, skyLight=False, maxBounces=sc.max_bounces)
    paths_step = sc.pixels * sc.spp

    def make(flags=0):
        r = atx.Renderer(device=dev, flags=flags)
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        r.set_camera(cam)
        r.set_settings(settings)
        return r

    # ---- device-timed throughput (inputs resident in HBM); consecutive renders overlap on the GPU
    # (ATX_FLAG_OVERLAP_RENDERS: the next launch's lanes start while the previous one's last bounces run)
    r = make(N.FLAG_OVERLAP_RENDERS)
    for _ in range(args.warmup):
        r.render_frames(sc.spp)
    r.synchronize()
    stream = torch.cuda.ExternalStream(r.stream, device=dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = Clocks(dev)
    clocks.start()
    soak(r, sc.spp, 0.4)
    s0 = r.stats()
    dist.barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        r.render_frames(sc.spp)
    r.join()                       # the stream after every lane of every launch
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    s1 = r.stats()
    soak(r, sc.spp, 0.25)
    clk = clocks.stop()
    dist.barrier()
    ms_local = ev0.elapsed_time(ev1)
    ms = dist.max(ms_local)
    launches = s1["kernel_launches"] - s0["kernel_launches"]
    rays = (s1["extension_rays"] - s0["extension_rays"]) + (s1["shadow_rays"] - s0["shadow_rays"])
    value = dist.world * args.steps * paths_step / (ms * 1e-3) / 1e6
    mrays = dist.world * rays / (ms_local * 1e-3) / 1e6
    r.close()

    # ---- end to end through the public API with host buffers (pinned)
    img_bytes = sc.pixels * 4
    hbuf = C.c_void_p()
    N.check(N.lib().atx_host_alloc(img_bytes, C.byref(hbuf)))
    host_img = np.ctypeslib.as_array((C.c_uint32 * sc.pixels).from_address(hbuf.value))
    sph = np.ascontiguousarray(sc.spheres)
    mats = np.ascontiguousarray(sc.materials)
    lts = np.ascontiguousarray(sc.lights)
    r = atx.Renderer(device=dev, flags=N.FLAG_OVERLAP_RENDERS)
    r.on_resize(sc.width, sc.height)
    r.set_settings(settings)

    # progressive rendering, as the reference's Render loop: the scene stays resident (it is uploaded
    # again only for a new scene or at frame 1, Renderer.cu:175-182); each step sends the camera
    # (kernel parameters), renders and reads the RGBA8 image back into pinned host memory
    r.set_scene(sph, mats, lts)

    # each step's image goes to one of two pinned host buffers by an asynchronous read that is waited for
    # one step later, while the next launch runs (renders alternate between two device images)
    hbufs = [hbuf, C.c_void_p()]
    N.check(N.lib().atx_host_alloc(img_bytes, C.byref(hbufs[1])))
    pending = []

    def frame_step():
        r.set_camera(cam)
        r.render_frames(sc.spp)
        t = C.c_uint64()
        N.check(N.lib().atx_read_image_async(r._h, hbufs[len(pending) % 2], sc.pixels, C.byref(t)))  # D2H
        pending.append(t.value)
        if len(pending) >= 2:
            N.check(N.lib().atx_wait_read(r._h, pending[-2]))

    def drain():
        if pending:
            N.check(N.lib().atx_wait_read(r._h, pending[-1]))

    def e2e_run(step):
        for _ in range(args.warmup):
            step()
        drain()
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        drain()                    # the last step's image has landed
        return dist.max(time.perf_counter() - t0)

    e2e_s = e2e_run(frame_step)

    # the same with the scene uploaded every step (tables, light and direction buffers rebuilt, at the
    # cheaper 16 cells along a face's edge that suit one render per scene)
    r.set_tuning(cell_res=16)

    def scene_step():
        r.set_scene(sph, mats, lts)
        frame_step()
    e2e_scene_s = e2e_run(scene_step)
    r.close()
    N.check(N.lib().atx_host_free(hbufs[0]))
    N.check(N.lib().atx_host_free(hbufs[1]))
    h2d_scene = len(sph) * 24 + len(mats) * 48 + len(lts) * 32      # device layout copied by atx_set_scene
    e2e = {"value": round(dist.world * args.steps * paths_step / e2e_s / 1e6, 2), "unit": UNIT,
           "h2d_bytes_per_step": CAMERA_BYTES, "d2h_bytes_per_step": img_bytes,
           "ms_per_step": round(e2e_s * 1e3 / args.steps, 3),
           "what": "atx_set_camera + atx_render (16 frames) + atx_read_image_async of the RGBA8 image into one of "
                   "two pinned host buffers per step, each read waited for one step later and the last before the "
                   "clock stops; scene resident (uploaded once, as the reference's Render loop re-uploads it only "
                   "for a new scene or frame 1)",
           "with_scene_upload": {"value": round(dist.world * args.steps * paths_step / e2e_scene_s / 1e6, 2),
                                 "what": "atx_set_scene every step as well (light and direction buffers rebuilt, "
                                         "16 cells along a face's edge)",
                                 "h2d_bytes_per_step": CAMERA_BYTES + h2d_scene,
                                 "ms_per_step": round(e2e_scene_s * 1e3 / args.steps, 3)}}
    _ = host_img

    # ---- roofline: one render launch against HBM, from per-kernel events (one lane, kernels serialised)
    rp = make(N.FLAG_PROFILE_KERNELS)
    for _ in range(max(1, args.warmup)):
        rp.render_frames(sc.spp)
    rp.synchronize()
    rp.reset_kernel_times()
    p0 = rp.stats()
    prof_steps = max(2, min(args.steps, 8))
    for _ in range(prof_steps):
        rp.render_frames(sc.spp)
    kt = rp.kernel_times()
    p1 = rp.stats()
    rp.close()
    # the primary ray of a pixel is traced once per launch (its samples share it)
    ext_after0 = (p1["extension_rays"] - p0["extension_rays"]) - sc.pixels * prof_steps
    sh_rays = p1["shadow_rays"] - p0["shadow_rays"]
    shaded0 = p1["shaded_first"] - p0["shaded_first"]
    alg_bytes = (BYTES_PER_EXTENSION * ext_after0 + BYTES_PER_SHADOW * sh_rays
                 + BYTES_PER_PIXEL * sc.pixels * prof_steps) / prof_steps
    total_kernel_ms = kt["extend_ms"] + kt["shadow_ms"] + kt["accumulate_ms"] + kt["other_ms"]
    launch_ms = total_kernel_ms / prof_steps
    peak = hbm_peak_gbs()
    # the launch's device time as the bench runs it (overlapped lanes); the serialised per-kernel
    # profile beside it
    step_ms = ms_local / args.steps
    achieved = alg_bytes / (step_ms * 1e-3) / 1e9
    achieved_serial = alg_bytes / (launch_ms * 1e-3) / 1e9
    roofline = {
        "kernel": "one atx_render of the workload: k_primary, k_shadow (first-bounce pixel-light rays), "
                  "k_first, k_shade (bounce 1), k_paths (bounces 2-7), k_accumulate per lane",
        "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
        "frac": round(achieved / peak, 4) if peak else None,
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth, burst)",
        "traffic": None,
        "algorithmic_bytes_per_launch": round(alg_bytes),
        "algorithmic_bytes": f"{BYTES_PER_EXTENSION} B per extension ray after the first bounce (ray record "
                             f"2x44, hit record 2x8), {BYTES_PER_SHADOW} B per shadow ray (record 2x40), "
                             f"{BYTES_PER_PIXEL} B per pixel (primary hit 2x8, accumulator 2x16, RGBA8 4)",
        "units_per_launch": {"extension_rays_after_first_bounce": round(ext_after0 / prof_steps),
                             "shadow_rays": round(sh_rays / prof_steps),
                             "first_bounce_shaded_paths": round(shaded0 / prof_steps),
                             "pixels": sc.pixels},
        "avg_launch_ms": round(step_ms, 4),
        "launch_ms_source": "CUDA events on the renderer's stream over the timed launches (value's own clock)",
        "serialised_profile": {"launch_ms": round(launch_ms, 4), "achieved": round(achieved_serial, 1),
                               "frac": round(achieved_serial / peak, 4) if peak else None,
                               "what": "per-kernel CUDA events of one lane, kernels one after another"},
        "kernel_launches_per_launch": round((kt["extend_launches"] + kt["shadow_launches"] +
                                             kt["accumulate_launches"] + kt["other_launches"]) / prof_steps, 1),
        "kernel_ms_per_step": {k: round(kt[k] / prof_steps, 3) for k in
                               ("extend_ms", "shadow_ms", "accumulate_ms", "other_ms")},
    }
    # DRAM bytes of the same launch's kernels, from an ncu capture summarised in profiles/
    traffic_file = ROOT / "profiles" / "render_traffic_medium_scene.txt"
    if traffic_file.exists():
        for line in traffic_file.read_text().splitlines():
            if line.startswith("dram_bytes_per_launch:"):
                roofline["traffic"] = int(line.split(":", 1)[1])
                roofline["traffic_source"] = "profiles/render_traffic_medium_scene.txt (ncu)"

    # FP32 roofline: FP32 work executed by the same launch's kernels (ncu instruction counts, summarised in
    # profiles/) over the launch's device time, against the FP32 pipe peak measured on this GPU
    fp32_file = ROOT / "profiles" / "fp32_ops_medium_scene.md"
    flops = None
    if fp32_file.exists():
        for line in fp32_file.read_text().splitlines():
            if line.startswith("fp32_flops_per_launch:"):
                flops = int(line.split(":", 1)[1])
    if flops:
        from baseline import fp32

        fpeak = fp32.peak_tflops(dev)
        f_ach = flops / (step_ms * 1e-3) / 1e12
        f_ser = flops / (launch_ms * 1e-3) / 1e12
        out_fp32 = {"bound": "fp32", "achieved": round(f_ach, 2), "peak": round(fpeak, 1), "unit": "TFLOP/s",
                    "frac": round(f_ach / fpeak, 4) if fpeak else None,
                    "achieved_serialised_profile": round(f_ser, 2),
                    "frac_serialised_profile": round(f_ser / fpeak, 4) if fpeak else None,
                    "flops_per_launch": flops,
                    "flops_source": "profiles/fp32_ops_medium_scene.md (ncu: FADD + FMUL + 2 FFMA + 2 FADD2 + "
                                    "2 FMUL2 + 4 FFMA2 thread instructions of one launch's kernels)",
                    "peak_source": "baseline/fp32_peak.cu: register-resident FFMA chains on every SM of this GPU, "
                                   "best of five launches"}
        # the algorithmic work of brute-force scenes: every ray tests every sphere (20 FLOP per test, FMA
        # as 2) plus 120 per shaded hit; the tile masks, light and direction buffers skip most of those
        # tests, so this rate can exceed the pipe's peak
        rays_launch = (ext_after0 + sc.pixels * prof_steps + sh_rays) / prof_steps
        shaded_launch = (shaded0 + ext_after0) / prof_steps
        bf = rays_launch * len(sc.spheres) * 20 + shaded_launch * 120
        out_fp32["brute_force_equivalent"] = {
            "flops_per_launch": round(bf), "achieved": round(bf / (step_ms * 1e-3) / 1e12, 2),
            "frac": round(bf / (step_ms * 1e-3) / 1e12 / fpeak, 4) if fpeak else None,
            "what": "the traced rays (primary per pixel, extension, shadow) at 20 FLOP per ray-sphere test "
                    f"against all {len(sc.spheres)} spheres, plus 120 per shaded first-bounce path and per extension ray "
                    "after it (an upper bound on the shaded hits), over the same launch time"}
    else:
        out_fp32 = None

    ref_kernel = None
    if dist.world == 1 and not args.no_ref_kernel:
        ref_kernel = time_reference_kernel(sc, cam, dev, args)

    out = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes.config1)",
        "config": {"workload": WORKLOAD_MEDIUM,
                   "paths_per_step": paths_step, "parallelism": f"replicas x{dist.world}",
                   "l2": "working set > L2: four lanes of 8.3 Mi-path wave state (about 1 GB each) per launch"},
        "mrays_per_s": round(mrays, 1),
        "rays_per_path": round(rays / (args.steps * paths_step), 4),
        "primary_hit_frac": round(shaded0 / (prof_steps * paths_step), 4),
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": roofline,
        "fp32_roofline": out_fp32,
        "e2e": e2e,
    }
    if ref_kernel:
        out["ref_cuda_kernel"] = ref_kernel
        if "kernel_mpaths_s" in ref_kernel:
            out["vs_ref_cuda_kernel"] = round(value / ref_kernel["kernel_mpaths_s"], 2)
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        v, sample, cores, mr = cpu_reference(sc, args.cpu_seconds)
        out["cpu_baseline"] = {"value": round(v, 4), "unit": UNIT, "cores": cores, "kind": "port",
                               "cpu": cpu_model(), "sample": sample, "mrays_per_s": round(mr, 3),
                               "what": "reference per-pixel path restated in C (literal expression order, "
                                       "within 1e-3 of the reference's own kernel built with IEEE arithmetic "
                                       "on >= 99.99% of pixels), OpenMP over rows"}
        out["cpu_baseline_small_scene"] = cpu_small_scene()
    if dist.world == 1 and not args.no_extra:
        out["small_scene"] = small_scene_leg(args, dev)
        out["large_scene"] = large_scene_leg(args, dev)
        out["batch"] = batch_compare(args, dev, max(3, min(args.steps, 8)))
        out["serve"] = serve_leg(args)
    return out


def time_reference_kernel(sc, cam, dev, args) -> dict:
    """The reference's own kernelRender, compiled from its unmodified Renderer.cu and BRDF.cu with its own
    flags (baseline/refbuild, -use_fast_math), launched as Renderer::Render launches it: one sample per
    pixel per launch, (opt/32 x opt/32) blocks, the default stream.  Kernel-only device time (CUDA events)
    over the same samples per pixel as a few of our steps, and the reference's whole per-frame Render()
    sequence (scene upload at frame 1, ray-direction upload, syncs, image copy) by wall clock."""
    import ataraxia_gb300 as atx
    from baseline import refbuild

    if not refbuild.available("fast"):
        return {"unavailable": "the reference's device image was not built (needs the reference tree)"}
    _, iv, _, ip = atx.camera_matrices(cam, sc.width, sc.height)
    dirs = refbuild.ray_dirs(iv, ip, sc.width, sc.height)
    name, block = refbuild.kernel_info("fast")
    with refbuild.RefRenderer(sc.spheres, sc.materials, sc.lights, sc.width, sc.height, dirs, sc.camera_position,
                              sc.camera_direction, sc.max_bounces) as ref:
        ref.frames(3)
        frames = sc.spp * max(1, min(args.steps, 4))
        k_ms = ref.time_frames(frames)
        ref.set_frame(1)
        ref.frame(full=True)                       # frame 1: scene upload, accumulator cleared
        t0 = time.perf_counter()
        for _ in range(sc.spp):
            ref.frame(full=True)
        r_s = time.perf_counter() - t0
    return {"kernel_mpaths_s": round(frames * sc.pixels / (k_ms * 1e-3) / 1e6, 2),
            "render_mpaths_s": round(sc.spp * sc.pixels / r_s / 1e6, 2),
            "kernel_ms_per_frame": round(k_ms / frames, 3), "render_ms_per_frame": round(r_s * 1e3 / sc.spp, 3),
            "block": [block, block], "kernel": name,
            "what": "the reference's kernelRender compiled from its unmodified Renderer.cu + BRDF.cu "
                    "(baseline/refbuild: own minimal glm, headless Image/Input stubs; -use_fast_math "
                    "--expt-relaxed-constexpr -rdc=true for sm_103a), 1 spp per launch; render_* is the "
                    "reference's per-frame Render() sequence: ray-direction cudaMalloc + upload + syncs, "
                    "launch, image copy"}


def batch_compare(args, dev: int, steps: int) -> dict:
    """The batched mix (64 scenes, seed 3): the plain wavefront renderer launched once per scene against
    one batched pass (all scenes, one CUDA graph) per step.  The plain arm is timed two ways: the device
    time of its render calls alone (CUDA events around each launch, the scene already set), and as a
    caller sees it (wall clock over the whole loop: per scene resize, scene upload with its acceleration
    structures, camera, settings, the launch and the RGBA8 read-back; built with the cheaper 16 cells
    along a face's edge, which suit one render per scene).  gpu_idle_frac = the share of the
    caller's loop in which no render kernel of the plain arm runs.  saturated_ceiling = the mix's paths
    over the device time they take when every scene is rendered alone in launches of at least 64 Mi
    paths: what a launch structure that keeps each path's work can approach."""
    import numpy as np
    import torch

    import ataraxia_gb300 as atx
    from ataraxia_gb300 import scenes

    torch.cuda.set_device(dev)
    mix = scenes.config3(count=args.mix_scenes)
    if args.max_pass_spp:   # slices of at most this many frames per scene and pass, as a server makes
        mix = [scenes.SyntheticScene(**{**sc.__dict__, "spp": min(sc.spp, args.max_pass_spp)}) for sc in mix]
    paths = sum(s.width * s.height * s.spp for s in mix)

    # plain: one renderer, one launch per scene
    r = atx.Renderer(device=dev, bvh_threshold=args.bvh_threshold, bvh_leaf_size=args.bvh_leaf)
    stream = torch.cuda.ExternalStream(r.stream, device=dev)
    img = {sc.width * sc.height: np.empty(sc.width * sc.height, np.uint32) for sc in mix}
    plain_ms = 0.0
    caller_s = 0.0
    for rep in range(3):                       # rep 0 warms up (allocations, BVH builds)
        if rep == 2:
            # a caller that renders each scene once does best with the cheaper light and direction buffers
            # (16 cells along a face's edge, the server's choice for its jobs)
            r.set_tuning(cell_res=16)
        t0 = time.perf_counter()
        for sc in mix:
            r.on_resize(sc.width, sc.height)
            r.set_scene(sc.spheres, sc.materials, sc.lights)
            r.set_camera(atx.Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction))
            r.set_settings(atx.Settings(True, sc.sky_light, sc.max_bounces))
            if rep == 1:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                r.render_frames(sc.spp)
                e1.record(stream)
                e1.synchronize()
                plain_ms += e0.elapsed_time(e1)
            else:
                r.render_frames(sc.spp)
                r.get_image(out=img[sc.width * sc.height])
        r.synchronize()
        if rep == 2:
            caller_s = time.perf_counter() - t0
    r.close()

    # ceiling for any launch structure that keeps each path's work: every scene rendered alone in launches
    # of >= 64 Mi paths (its tail amortised), device time per path summed over the mix's paths
    r = atx.Renderer(device=dev, bvh_threshold=args.bvh_threshold, bvh_leaf_size=args.bvh_leaf)
    stream = torch.cuda.ExternalStream(r.stream, device=dev)
    ideal_ms = 0.0
    for sc in mix:
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        r.set_camera(atx.Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction))
        r.set_settings(atx.Settings(True, sc.sky_light, sc.max_bounces))
        big = max(sc.spp, -(-(64 << 20) // (sc.width * sc.height)))
        r.render_frames(sc.spp)                # warm: per-camera tables built
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r.render_frames(big)
        e1.record(stream)
        e1.synchronize()
        ideal_ms += e0.elapsed_time(e1) * sc.spp / big
    r.close()

    b = atx.Batch(device=dev, bvh_threshold=args.bvh_threshold, bvh_leaf_size=args.bvh_leaf)
    if args.lanes or args.lane_wave:
        b.set_tuning(lanes=args.lanes, lane_wave_paths=args.lane_wave << 20)
    ids = [b.add_synthetic(sc) for sc in mix]
    for i, sc in zip(ids, mix):
        b.set_spp(i, sc.spp)
    if args.autotune:
        b.autotune()
    for _ in range(args.warmup):
        b.run()
    b.synchronize()
    s0 = b.stats()
    t0 = time.perf_counter()
    pass_ms = []
    for _ in range(steps):
        b.run()
        b.synchronize()
        pass_ms.append(b.stats()["last_pass_ms"])
    wall = time.perf_counter() - t0
    s1 = b.stats()
    tun = b.tuning()
    b.close()
    batched_ms = statistics.mean(pass_ms)
    return {"scenes": len(mix), "paths_per_pass": paths,
            "plain_device_ms": round(plain_ms, 3), "plain_mpaths_s": round(paths / (plain_ms * 1e-3) / 1e6, 1),
            "plain_caller_ms": round(caller_s * 1e3, 3),
            "plain_caller_mpaths_s": round(paths / caller_s / 1e6, 1),
            "plain_gpu_idle_frac": round(max(0.0, 1.0 - plain_ms / (caller_s * 1e3)), 3),
            "batched_ms_per_pass": round(batched_ms, 3),
            "batched_mpaths_s": round(paths / (batched_ms * 1e-3) / 1e6, 1),
            "batched_wall_mpaths_s": round(steps * paths / wall / 1e6, 1),
            "saturated_ceiling_mpaths_s": round(paths / (ideal_ms * 1e-3) / 1e6, 1),
            "batched_frac_of_ceiling": round(ideal_ms / batched_ms, 3),
            "speedup_vs_plain_device": round(plain_ms / batched_ms, 3),
            "speedup_vs_plain_caller": round(caller_s * 1e3 / (wall * 1e3 / steps), 3),
            "graph_launches": s1["graph_launches"] - s0["graph_launches"],
            "rays_per_path": round(((s1["extension_rays"] - s0["extension_rays"]) +
                                    (s1["shadow_rays"] - s0["shadow_rays"])) / (steps * paths), 3),
            "tuning": tun}


def run_batch_compare(args, dist: Dist):
    return {"mode": "batch", **batch_compare(args, dist.local_rank, args.steps)}


def large_scene_leg(args, dev: int) -> dict:
    """The large scene (seed 2): 65,536 clustered spheres through the LBVH, 3840x2160, 8 bounces, 4 spp
    per launch; device time over launches with the scene resident."""
    import torch

    import ataraxia_gb300 as atx
    from ataraxia_gb300 import scenes

    from ataraxia_gb300 import _native as N

    sc = scenes.config2()
    r = atx.Renderer(device=dev, bvh_leaf_size=args.bvh_leaf, flags=N.FLAG_OVERLAP_RENDERS)
    r.on_resize(sc.width, sc.height)
    r.set_scene(sc.spheres, sc.materials, sc.lights)
    r.set_camera(atx.Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction))
    r.set_settings(atx.Settings(accumulation=True, skyLight=False, maxBounces=sc.max_bounces))
    t0 = time.perf_counter()
    tuned = r.autotune(sc.spp, passes=3, use_cache=False) if not args.bvh_leaf else r.tuning()
    tune_s = time.perf_counter() - t0
    for _ in range(3):
        r.render_frames(sc.spp)
    r.synchronize()
    stream = torch.cuda.ExternalStream(r.stream, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0 = r.stats()
    steps = max(3, min(args.steps, 10))
    e0.record(stream)
    for _ in range(steps):
        r.render_frames(sc.spp)
    r.join()
    e1.record(stream)
    e1.synchronize()
    s1 = r.stats()
    r.close()
    ms = e0.elapsed_time(e1)
    rays = (s1["extension_rays"] - s0["extension_rays"]) + (s1["shadow_rays"] - s0["shadow_rays"])
    return {"workload": "large scene: 65,536 spheres in 32 clusters, 256 materials, 16 lights, 3840x2160, "
                        "8 bounces, 4 spp per launch (LBVH)",
            "mpaths_s": round(steps * sc.pixels * sc.spp / (ms * 1e-3) / 1e6, 1),
            "mrays_s": round(rays / (ms * 1e-3) / 1e6, 1), "ms_per_launch": round(ms / steps, 3),
            "launches": steps, "bvh_in_use": int(s1["bvh_in_use"]),
            "tuning": {k: tuned[k] for k in ("bvh_leaf_size", "lanes", "wave_paths", "threads", "wave_spp",
                                              "path_kernel")},
            "tuning_source": "atx_autotune on this scene, camera and GPU" if not args.bvh_leaf else "--bvh-leaf",
            "autotune_s": round(tune_s, 2)}


def small_scene_leg(args, dev: int) -> dict:
    """The small scene (seed 0) as its workload states it: 1280x720, 5 bounces, 64 accumulated frames.
    Ours renders the 64 frames in one launch and, as the reference's interactive loop does, one frame per
    call (overlapped renders); the reference's own kernelRender renders them one frame per launch
    (kernel-only device time, and with its per-frame Render() sequence)."""
    import torch

    import ataraxia_gb300 as atx
    from ataraxia_gb300 import _native as N
    from ataraxia_gb300 import scenes
    from baseline import refbuild

    sc = scenes.config0()
    frames = sc.frames
    cam = atx.Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction)
    out = {"workload": "small scene: 8 spheres + ground, 8 materials, 1 light, 1280x720, 5 bounces, 64 frames"}
    r = atx.Renderer(device=dev, flags=N.FLAG_OVERLAP_RENDERS)
    r.on_resize(sc.width, sc.height)
    r.set_scene(sc.spheres, sc.materials, sc.lights)
    r.set_camera(cam)
    r.set_settings(atx.Settings(accumulation=True, skyLight=False, maxBounces=sc.max_bounces))
    stream = torch.cuda.ExternalStream(r.stream, device=dev)
    for label, per_call in (("one_launch", frames), ("frame_per_call", 1)):
        for _ in range(3):
            r.reset_frame_index()
            for _ in range(frames // per_call):
                r.render_frames(per_call)
        r.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r.reset_frame_index()
        e0.record(stream)
        for _ in range(frames // per_call):
            r.render_frames(per_call)
        r.join()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[f"ours_{label}_mpaths_s"] = round(sc.pixels * frames / (ms * 1e-3) / 1e6, 1)
        out[f"ours_{label}_ms"] = round(ms, 3)
    r.close()
    if refbuild.available("fast"):
        _, iv, _, ip = atx.camera_matrices(cam, sc.width, sc.height)
        dirs = refbuild.ray_dirs(iv, ip, sc.width, sc.height)
        with refbuild.RefRenderer(sc.spheres, sc.materials, sc.lights, sc.width, sc.height, dirs,
                                  sc.camera_position, sc.camera_direction, sc.max_bounces) as ref:
            ref.frames(3)
            ref.set_frame(1)
            k_ms = ref.time_frames(frames)
            ref.set_frame(1)
            t0 = time.perf_counter()
            ref.frames(frames, full=True)
            r_s = time.perf_counter() - t0
        out["ref_kernel_mpaths_s"] = round(sc.pixels * frames / (k_ms * 1e-3) / 1e6, 1)
        out["ref_render_mpaths_s"] = round(sc.pixels * frames / r_s / 1e6, 1)
        out["vs_ref_kernel_one_launch"] = round(out["ours_one_launch_mpaths_s"] / out["ref_kernel_mpaths_s"], 2)
        out["vs_ref_render_frame_per_call"] = round(out["ours_frame_per_call_mpaths_s"] /
                                                     out["ref_render_mpaths_s"], 2)
    return out


def serve_leg(args) -> dict:
    """A short serving run (seed 4) at one arrival rate: the continuous-batching server (arrival order)
    against FIFO one-launch-per-job, p50/p99 time to target spp."""
    from ataraxia_gb300 import scenes

    pool = scenes.scene_pool(4, args.pool)
    jobs = scenes.config4(seed=4, rate=args.line_serve_rate, duration_s=args.line_serve_seconds, pool=pool)
    return {"rate_jobs_s": args.line_serve_rate, "seconds": args.line_serve_seconds,
            "hbm_budget_gb": args.hbm_budget_gb, "target_spp": [16, 64, 256, 1024],
            "batched": serve_batched(jobs, args.line_serve_seconds, args, "arrival"),
            "batched_smallest_first": serve_batched(jobs, args.line_serve_seconds, args, "smallest"),
            "fifo": serve_fifo(jobs, args.line_serve_seconds, args.max_pending)}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo), with the machine architecture."""
    import platform

    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return f"{platform.machine()} {line.split(':', 1)[1].strip()}"
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu part")):
                return f"{platform.machine()} {line.split(':', 1)[1].strip()}"
    except OSError:
        pass
    return platform.machine()


def cpu_small_scene(threads: int = 0) -> dict:
    """The small scene (seed 0) in full on the host cores: 1280x720, 5 bounces, 64 frames, the
    reference's per-pixel path restated in C (literal expression order), OpenMP over pixels."""
    from ataraxia_gb300 import scenes
    from oracle import pyoracle as po

    po.build()
    sc = scenes.config0()
    view = po.view_for(sc)
    nthreads = threads or po.max_threads()
    t0 = time.perf_counter()
    _, _, st = po.render(sc.spheres, sc.materials, sc.lights, view, max_bounces=sc.max_bounces, spp=64,
                         mode=po.LITERAL, threads=nthreads)
    dt = time.perf_counter() - t0
    paths = sc.pixels * 64
    return {"value": round(paths / dt / 1e6, 3), "unit": UNIT, "cores": nthreads, "kind": "port",
            "cpu": cpu_model(), "seconds": round(dt, 2),
            "mrays_per_s": round((st["ext_rays"] + st["shadow_rays"]) / dt / 1e6, 3),
            "sample": "small scene in full: 9 spheres, 1280x720, 5 bounces, 64 frames = 58,982,400 paths"}


def _pct(v, q):
    import numpy as np

    return round(float(np.percentile(np.asarray(v), q)), 4) if v else None


def serve_batched(jobs, duration, args, policy="arrival"):
    """Poisson arrivals into the continuous-batching server for `duration` seconds.  A driver thread
    submits each job at its arrival time (BUSY = rejected once max_pending jobs wait); the main thread
    collects finished jobs and releases them.  Latency = done time - intended arrival time."""
    import threading

    import ataraxia_gb300 as atx

    s = atx.Server(hbm_budget_bytes=int(args.hbm_budget_gb * 1e9), max_active_jobs=args.max_active,
                   pass_spp=args.pass_spp, max_pending=args.max_pending, max_pass_paths=args.max_pass_paths,
                   host_executor=getattr(args, "host_executor", False), policy=policy)
    lock = threading.Lock()
    outstanding = {}   # job id -> (intended arrival on the server clock, paths)
    rejected = [0]
    t0 = s.now()
    wall0 = time.perf_counter()

    def driver():
        for j in jobs:
            if j.arrival_s >= duration:
                break
            delay = j.arrival_s - (time.perf_counter() - wall0)
            if delay > 0:
                time.sleep(delay)
            try:
                jid = s.submit(j.scene, j.target_spp)
            except atx.AtxError:
                rejected[0] += 1
                continue
            with lock:
                outstanding[jid] = (t0 + j.arrival_s, j.scene.width * j.scene.height * j.target_spp)

    th = threading.Thread(target=driver)
    th.start()
    lat, done_paths, submitted = [], 0, 0
    end = t0 + duration
    while True:
        now = s.now()
        with lock:
            ids = list(outstanding.items())
        for jid, (arr, paths) in ids:
            info = s.poll(jid)
            if info["state"] == "done" and info["done_s"] <= end:
                lat.append(info["done_s"] - arr)
                done_paths += paths
                s.release(jid)
                with lock:
                    del outstanding[jid]
        if now >= end:
            break
        time.sleep(0.02)
    th.join()
    st = s.stats()
    with lock:
        incomplete = len(outstanding)
    for jid in list(outstanding):
        s.cancel(jid)
    s.close()
    span = duration
    return {"submitted": int(st["submitted"]), "rejected": rejected[0], "completed": len(lat),
            "incomplete": incomplete, "jobs_per_s": round(len(lat) / span, 2),
            "mpaths_s": round(st["paths"] / span / 1e6, 1), "completed_mpaths_s": round(done_paths / span / 1e6, 1),
            "p50_s": _pct(lat, 50), "p99_s": _pct(lat, 99), "passes": int(st["passes"]),
            "busy_frac": round(st["busy_s"] / span, 3)}


def serve_fifo(jobs, duration, max_pending):
    """One launch per job in arrival order on the plain renderer, image read back after each; jobs
    arriving while max_pending jobs wait are rejected, as the server's queue bound does.  Light and
    direction buffers at 16 cells along a face's edge, the server's setting for jobs rendered once."""
    from collections import deque

    import ataraxia_gb300 as atx

    r = atx.Renderer()
    r.set_tuning(cell_res=16)
    wall0 = time.perf_counter()
    lat, paths, rejected = [], 0, 0
    queue, nxt = deque(), 0

    def arrivals(upto):
        nonlocal nxt, rejected
        while nxt < len(jobs) and jobs[nxt].arrival_s <= min(upto, duration):
            if len(queue) >= max_pending:
                rejected += 1
            else:
                queue.append(jobs[nxt])
            nxt += 1

    while True:
        now = time.perf_counter() - wall0
        if now >= duration:
            break
        arrivals(now)
        if not queue:
            if nxt >= len(jobs) or jobs[nxt].arrival_s >= duration:
                break
            time.sleep(max(0.0, jobs[nxt].arrival_s - now))
            continue
        j = queue.popleft()
        sc = j.scene
        r.on_resize(sc.width, sc.height)
        r.set_scene(sc.spheres, sc.materials, sc.lights)
        r.set_camera(atx.Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction))
        r.set_settings(atx.Settings(accumulation=False, skyLight=sc.sky_light, maxBounces=sc.max_bounces))
        r.render_frames(j.target_spp)
        r.get_image()
        t = time.perf_counter() - wall0
        if t > duration:
            queue.appendleft(j)
            break
        lat.append(t - j.arrival_s)
        paths += sc.width * sc.height * j.target_spp
    arrivals(duration)
    r.close()
    return {"rejected": rejected, "completed": len(lat), "incomplete": len(queue),
            "jobs_per_s": round(len(lat) / duration, 2), "mpaths_s": round(paths / duration / 1e6, 1),
            "p50_s": _pct(lat, 50), "p99_s": _pct(lat, 99)}


def run_serve(args, dist: Dist):
    """Serving workload (seed 4): Poisson arrivals at each rate for --serve-seconds; continuous batching
    with an HBM budget against FIFO one-launch-per-job."""
    from ataraxia_gb300 import scenes

    pool = scenes.scene_pool(4, args.pool)
    out = {"mode": "serve", "seconds": args.serve_seconds, "hbm_budget_gb": args.hbm_budget_gb,
           "pool_scenes": len(pool), "rates": {}}
    for rate in [float(x) for x in args.rates.split(",")]:
        jobs = scenes.config4(seed=4, rate=rate, duration_s=args.serve_seconds, pool=pool)
        res = {}
        for pol in ("arrival", "smallest") if args.policy == "both" else (args.policy,):
            res["batched_" + pol] = serve_batched(jobs, args.serve_seconds, args, pol)
        if not args.no_fifo:
            res["fifo"] = serve_fifo(jobs, args.serve_seconds, args.max_pending)
        out["rates"][str(rate)] = res
        log(json.dumps({str(rate): res}))
    return out


def run_render_only(args, dist: Dist):
    """Warm-up and timed launches of the workload, nothing else (profiler captures)."""
    import ataraxia_gb300 as atx
    from ataraxia_gb300 import scenes

    sc = {"medium": scenes.config1, "large": scenes.config2, "small": scenes.config0}[args.workload]()
    if args.width and args.height:
        sc = sc.with_resolution(args.width, args.height)
    from ataraxia_gb300 import _native as N

    # the bench's own renderer: overlapped renders (4 lanes)
    r = atx.Renderer(device=dist.local_rank, bvh_threshold=args.bvh_threshold, bvh_leaf_size=args.bvh_leaf,
                     wave_paths=args.wave_paths, flags=N.FLAG_OVERLAP_RENDERS)
    r.on_resize(sc.width, sc.height)
    r.set_scene(sc.spheres, sc.materials, sc.lights)
    r.set_camera(atx.Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction))
    r.set_settings(atx.Settings(accumulation=True, skyLight=False, maxBounces=sc.max_bounces))
    for _ in range(args.warmup):
        r.render_frames(sc.spp)
    r.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r.render_frames(sc.spp)
    r.synchronize()
    dt = time.perf_counter() - t0
    st = r.stats()
    r.close()
    return {"mode": "render", "workload": args.workload, "bvh": st["bvh_in_use"], "bvh_leaf": args.bvh_leaf,
            "wave_paths": args.wave_paths, "width": sc.width, "height": sc.height, "steps": args.steps,
            "wall_ms_per_step": round(dt * 1e3 / args.steps, 3),
            "Mpaths_per_s_wall": round(args.steps * sc.pixels * sc.spp / dt / 1e6, 1),
            "kernel_launches": st["kernel_launches"]}


# -------------------------------------------------------- reference arm

def run_reference(args, dist: Dist):
    from ataraxia_gb300 import scenes

    sc = scenes.config1()
    vals = []
    sample = ""
    cores = 0
    mrays = []
    for i in range(args.warmup + args.steps):
        v, sample, cores, mr = cpu_reference(sc, args.ref_step_seconds)
        if i >= args.warmup:
            vals.append(v)
            mrays.append(mr)
    value = statistics.mean(vals)
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes.config1)",
        "config": {"workload": WORKLOAD_MEDIUM, "parallelism": "host cores (OpenMP)"},
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample + " per step"},
        "mrays_per_s": round(statistics.mean(mrays), 3),
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's perPixel is device code only, with no host path of its own; this arm runs it "
                "restated in C (the oracle's literal mode, within 1e-3 of the reference's kernel built with IEEE "
                "arithmetic on >= 99.99% of pixels) on the host cores; the reference's own CUDA kernel, compiled "
                "from its sources, is timed in the main line's ref_cuda_kernel",
    }


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ref-kernel", action="store_true", help="skip timing the reference's own CUDA kernel")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the large-scene, batched-mix and serving legs of the default line")
    ap.add_argument("--line-serve-rate", type=float, default=200.0, help="serving leg of the default line: jobs/s")
    ap.add_argument("--line-serve-seconds", type=float, default=10.0, help="serving leg of the default line: seconds")
    ap.add_argument("--ref-step-seconds", type=float, default=3.0)
    ap.add_argument("--mode", choices=["full", "render", "batch", "serve"], default="full",
                    help="render: only warm-up + timed launches of the workload (for profiler captures); "
                         "batch: the 64-scene mix, plain renderer per scene vs one batched pass")
    ap.add_argument("--mix-scenes", type=int, default=64, help="batch mode: scenes in the mix")
    ap.add_argument("--rates", default="50,200,800", help="serve mode: arrival rates (jobs/s)")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="serve mode: run length per rate")
    ap.add_argument("--hbm-budget-gb", type=float, default=120.0, help="serve mode: admission budget")
    ap.add_argument("--max-active", type=int, default=0, help="serve mode: jobs rendered together (0 = library default)")
    ap.add_argument("--pass-spp", type=int, default=0, help="serve mode: frames per job per pass (0 = library default)")
    ap.add_argument("--max-pending", type=int, default=4096, help="serve mode: queue bound (then BUSY)")
    ap.add_argument("--pool", type=int, default=512, help="serve mode: scenes in the job pool")
    ap.add_argument("--no-fifo", action="store_true", help="serve mode: skip the FIFO baseline")
    ap.add_argument("--policy", default="both", choices=["arrival", "smallest", "both"],
                    help="serve mode: admission order of the batching server")
    ap.add_argument("--max-pass-paths", type=int, default=0, help="serve mode: bound on paths per pass (0 = default)")
    ap.add_argument("--lanes", type=int, default=0, help="batch mode: concurrent lanes (0 = library default)")
    ap.add_argument("--max-pass-spp", type=int, default=0, help="batch mode: cap each scene's frames per pass")
    ap.add_argument("--autotune", action="store_true", help="batch mode: pick lanes / path state by timing first")
    ap.add_argument("--lane-wave", type=int, default=0, help="batch mode: path state per lane, Mi paths")
    ap.add_argument("--width", type=int, default=0, help="render mode: override the viewport width")
    ap.add_argument("--height", type=int, default=0, help="render mode: override the viewport height")
    ap.add_argument("--workload", choices=["medium", "large", "small"], default="medium",
                    help="render mode: scene (small = 8+1 spheres 720p, medium = 256 spheres 1080p, "
                         "large = 65,536 clustered spheres 4K)")
    ap.add_argument("--bvh-threshold", type=int, default=0, help="render mode: LBVH from this sphere count (0 = default)")
    ap.add_argument("--bvh-leaf", type=int, default=0, help="render mode: LBVH leaf size (0 = default)")
    ap.add_argument("--wave-paths", type=int, default=0, help="render mode: paths per wave (0 = default)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        log("warmup raised to 3 (minimum)")
        args.warmup = 3

    dist = Dist()
    try:
        if args.mode == "render":
            out = run_render_only(args, dist)
        elif args.mode == "batch":
            out = run_batch_compare(args, dist)
        elif args.mode == "serve":
            out = run_serve(args, dist)
        elif args.impl == "reference":
            if dist.rank != 0:
                return 0
            out = run_reference(args, dist)
        else:
            out = run_ours(args, dist)
        if dist.rank == 0:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
