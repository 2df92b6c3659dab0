"""Benchmark: Mrays/s of one rendered frame of the 1M-triangle spectral icosphere field on one GB300.

Workload (one "step" = one frame): 800 icospheres x 1,280 triangles (1,024,000 triangles, seeded), 1920 x 1080,
16 samples per pixel, path depth 12 (Russian roulette from depth 4), hero-wavelength spectral transport with 4
wavelengths over 360-830 nm through a device-generated rgb2spec table (res 64), 1024 x 512 FP32 sky map with a
5e3-radiance 0.5-degree sun, environment importance sampling with MIS, PCG32 seed 1. Synthetic, seeded data.

value : rays (primary + extension + shadow, counted on the device) / device time of the frame, rendered by the
        wavefront integrator (one CUDA-graph launch per frame), scene resident in HBM, L2 flushed (256 MiB write)
        before every timed frame.
e2e   : the same rays through the C ABI with host buffers: SceneData in from pinned host memory, the accumulation
        image (RGBA32F) read back to pinned host memory every frame, timed on the host clock.
roofline : the closest-hit traversal kernel (kWfIntersect) of one profiling frame of the same workload (stage-by-stage
        launches with device timers and fetch-byte counting): node (80 B) + triangle (48 B) bytes it fetches / its
        device time, against the measured HBM copy bandwidth.
megakernel : the same frame by the one-thread-per-pixel megakernel (vkrt's raygen structure), for comparison.
adjoint : the path-replay adjoint of the inverse-rendering Cornell box (128 x 128, 16 spp, depth 6, five 64 x 64
        albedo + roughness textures): device time of the adjoint call / device time of the forward frame.
batch : 64 uneven icosphere fields (10k-500k triangles, 256^2-1024^2, 8 spp, depth 10, RGB) in one autotuned graph
        launch vs 64 sequential megakernel (and wavefront) frames.
convergence : time to relMSE <= 1e-3 against a 2048-spp reference, plain wavefront vs radiance-cache frames.
--impl reference : the CPU restatement of vkrt's integrator (the oracle, a port: vkrt's own renderer needs Vulkan
        and is unavailable here) on all host cores, on a bounded block of rows of the same frame per step.
"""
from __future__ import annotations

import argparse
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

METRIC = "Mrays/s"
WORKLOAD = "icosphere-field-1M-tris 1920x1080 16spp depth12 hero-spectral env-IS"


def _config(width, height, spp, depth, tris, extra=None):
    c = {"workload": WORKLOAD, "triangles": tris, "width": width, "height": height, "spp": spp, "max_depth": depth,
         "render_mode": "spectral-hero-4", "rng": "pcg32 seed 1", "environment": "1024x512 fp32 sky + sun, IS+MIS",
         "l2": "flushed before every timed frame (256 MiB write)"}
    if extra:
        c.update(extra)
    return c


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def _traffic_per_launch():
    """DRAM bytes per kWfIntersect launch of the headline frame from the committed ncu capture, when one exists."""
    p = ROOT / "profiles" / "kWfIntersect_dram_icosphere1M_1920x1080x16spp.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get("dram_bytes_per_launch")
        except Exception:
            return None
    return None


def build_scene(spp=16, depth=12, width=1920, height=1080, n_spheres=800):
    from vkrt_gb300 import scenes
    return scenes.icosphere_field(n_spheres=n_spheres, width=width, height=height, spp=spp, max_depth=depth, seed=1,
                                  spectral=True)


def _rays(st):
    return st["primaryRays"] + st["extensionRays"] + st["shadowRays"]


def _device_frames(ctx, sd, stream, flush, frame, n, torch):
    """n frames, each after an L2 flush, timed with CUDA events on the context stream; returns (ms list, rays,
    kernel launches)."""
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
    rays = launches = 0
    for k in range(n):
        sd["frameNumber"] = frame[0]
        frame[0] += 1
        with torch.cuda.stream(stream):
            flush.zero_()
            events[k][0].record(stream)
            ctx.render_frame(sd)
            events[k][1].record(stream)
        ctx.sync()
        st = ctx.stats()
        rays += _rays(st)
        launches += st["kernelLaunches"]
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in events], rays, launches


def adjoint_ratio(local: int) -> dict:
    """Device time of the path-replay adjoint over the forward frame on the inverse-rendering Cornell box."""
    import torch
    from vkrt_gb300 import RenderContext, abi, scenes
    s = scenes.inverse_rendering_cornell(128, 128, 16, 6, target=False)
    t = scenes.inverse_rendering_cornell(128, 128, 16, 6, target=True)
    ctx = RenderContext(device=local, rng_mode=abi.RNG_PCG32, integrator=abi.INTEGRATOR_WAVEFRONT)
    ctx.upload_scene(t)
    ctx.render_frame(t.scene_data)
    target = ctx.read_accumulation()[..., :3].copy()
    ctx.upload_scene(s)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))

    def timed(fn, reps=20):
        ts = []
        for _ in range(reps + 3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts[3:]))

    def forward():
        ctx.reset_accumulation()
        ctx.render_frame(s.scene_data)
    fwd = timed(forward)
    forward()
    img = ctx.read_accumulation()
    d = np.zeros_like(img)
    d[..., :3] = 2.0 * (img[..., :3] - target) / target.size
    dev = torch.from_numpy(d).to(f"cuda:{local}")
    torch.cuda.synchronize()
    adj = timed(lambda: ctx.render_adjoint_device(s.scene_data, dev.data_ptr()))
    ctx.close()
    return {"workload": "inverse-rendering cornell 128x128 16spp depth6, 5 walls x (64x64 albedo + roughness)",
            "forward_ms": round(fwd, 3), "adjoint_ms": round(adj, 3), "ratio": round(adj / fwd, 2),
            "integrator": "wavefront (primal + adjoint passes)",
            "gradients": "albedo texels, roughness texels, emission radiance; FP64 central-difference tests"}


def convergence_measure(local: int, scene, mega_ms: float, max_frames: int = 96, ref_frames: int = 128) -> dict:
    """Time to relMSE <= 1e-3 on the benchmark frame (16 spp per frame) for the plain wavefront tracer and for the
    radiance-cache tracer, against a 2048-spp reference of the same scene rendered by the GPU tracer (which matches
    the FP64 oracle per sample in the tests). relMSE = mean over pixels and channels of (x - ref)^2 / (ref^2 + 1e-2)."""
    import torch
    from vkrt_gb300 import RenderContext, abi

    ctx = RenderContext(device=local, rng_mode=abi.RNG_PCG32, rng_seed=1, environment_sampling=abi.ENV_IMPORTANCE,
                        integrator=abi.INTEGRATOR_WAVEFRONT)
    ctx.upload_scene(scene)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    sd = scene.scene_data.copy()
    ctx.reset_accumulation()
    for f in range(ref_frames):
        sd["frameNumber"] = 1_000_000 + f
        ctx.render_frame(sd)
    ref = ctx.read_accumulation()[..., :3].astype(np.float64)
    den = ref ** 2 + 1e-2

    def curve(**cache):
        ctx.nrc_configure(**cache)
        ctx.reset_accumulation()
        total, pts, reached = 0.0, [], None
        for f in range(max_frames):
            sd["frameNumber"] = f
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.render_frame(sd)
            b.record(stream)
            b.synchronize()
            total += a.elapsed_time(b)
            err = float(np.mean((ctx.read_accumulation()[..., :3] - ref) ** 2 / den))
            pts.append([f + 1, round(total, 1), round(err, 6)])
            if err <= 1e-3:
                reached = {"frames": f + 1, "spp": 16 * (f + 1), "ms": round(total, 1)}
                break
        return {"reached": reached, "curve": pts[:: max(1, len(pts) // 12)] + ([pts[-1]] if pts else [])}

    plain = curve(enabled=0)
    cached = curve(enabled=1, terminationDepth=2, trainingPaths=65536, trainingSteps=4, learningRate=1e-2, seed=3)
    ctx.close()
    out = {"threshold": 1e-3, "reference": f"{16 * ref_frames} spp, GPU wavefront tracer, independent seeds",
           "plain_wavefront": plain, "radiance_cache": cached}
    if plain["reached"]:
        # the megakernel renders the same samples (tests: identical images), so it needs the same frames
        out["megakernel_ms"] = round(plain["reached"]["frames"] * mega_ms, 1)
        out["wavefront_over_megakernel"] = round(plain["reached"]["ms"] / out["megakernel_ms"], 4)
    return out


def batch_measure(local: int) -> dict:
    """Uneven batch: 64 seeded icosphere fields (10k-500k triangles, 256^2-1024^2, 8 spp, depth 10, RGB) rendered
    as one autotuned graph launch, against 64 sequential megakernel frames and 64 sequential wavefront frames."""
    import torch
    from vkrt_gb300 import RenderContext, abi, scenes
    from vkrt_gb300.context import autotune_batch, render_batch

    ss = scenes.batch_workload(64, seed=2)
    ctxs = []
    for sc in ss:
        c = RenderContext(device=local, rng_mode=abi.RNG_PCG32, environment_sampling=abi.ENV_IMPORTANCE,
                          integrator=abi.INTEGRATOR_WAVEFRONT)
        c.upload_scene(sc)
        ctxs.append(c)
    sds = np.concatenate([sc.scene_data for sc in ss])
    torch.cuda.synchronize()

    def sequential(integrator):
        ms = rays = 0.0
        for c, sc in zip(ctxs, ss):
            c.set_integrator(integrator)
            st = torch.cuda.ExternalStream(c.stream, device=torch.device("cuda", local))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            c.render_frame(sc.scene_data)
            b.record(st)
            b.synchronize()
            ms += a.elapsed_time(b)
            rays += _rays(c.stats())
        for c in ctxs:
            c.set_integrator(abi.INTEGRATOR_WAVEFRONT)
        return ms, rays

    sequential(abi.INTEGRATOR_WAVEFRONT)  # warm-up: graphs, buffers
    t0 = time.perf_counter()
    best, tuned_ms = autotune_batch(ctxs, sds, frames_per_trial=1)
    tune_s = time.perf_counter() - t0
    stream0 = torch.cuda.ExternalStream(ctxs[0].stream, device=torch.device("cuda", local))
    render_batch(ctxs, sds)  # warm-up of the tuned shape
    torch.cuda.synchronize()
    bms = []
    for _ in range(2):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream0)
        render_batch(ctxs, sds)
        b.record(stream0)
        b.synchronize()
        bms.append(a.elapsed_time(b))
    brays = _rays(ctxs[0].stats())
    mega_ms, mega_rays = sequential(abi.INTEGRATOR_MEGAKERNEL)
    wave_ms, wave_rays = sequential(abi.INTEGRATOR_WAVEFRONT)
    for c in ctxs:
        c.close()
    batched = float(min(bms))
    return {"workload": "64 icosphere fields, 10k-500k triangles (log-uniform), 256^2-1024^2, 8 spp, depth 10, RGB",
            "triangles": int(sum(sc.triangle_count for sc in ss)), "pixels": int(sum(sc.width * sc.height for sc in ss)),
            "batched_ms": round(batched, 2), "batched_Mrays_s": round(brays / (batched * 1e-3) / 1e6, 1),
            "sequential_megakernel_ms": round(mega_ms, 2),
            "sequential_megakernel_Mrays_s": round(mega_rays / (mega_ms * 1e-3) / 1e6, 1),
            "sequential_wavefront_ms": round(wave_ms, 2),
            "speedup_vs_sequential_megakernel": round(mega_ms / batched, 2),
            "speedup_vs_sequential_wavefront": round(wave_ms / batched, 2),
            "autotune_s": round(tune_s, 1),
            "autotuned": {k: int(best[k][0]) for k in ("queueCapacity", "tileWidth", "tileHeight", "sortByMaterial",
                                                       "intersectBlocksPerSM", "shadeBlocksPerSM")}}


def selection_overlay_measure(ctx, sd, stream, torch) -> dict:
    """Selection mask (a pixel-centre ray per pixel against the picked mesh) plus outline on the benchmark frame:
    the mesh under the film centre is selected; device ms per overlay call (CUDA events, mean of 5 after 1)."""
    from vkrt_gb300 import abi
    mesh = ctx.pick_mesh(sd, ctx.width // 2, ctx.height // 2)
    osd = sd.copy()
    osd["selectionEnabled"] = 1 if mesh != abi.INVALID_INDEX else 0
    osd["selectedMeshIndex"] = mesh
    ctx.render_selection_overlay(osd)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(5):
        ctx.render_selection_overlay(osd)
    b.record(stream)
    b.synchronize()
    return {"workload": f"{ctx.width}x{ctx.height}, mesh {mesh} (under the film centre) selected",
            "ms": round(a.elapsed_time(b) / 5, 3), "mask_pixels": int(ctx.read_selection_mask().sum())}


def features_and_materials_measure(ctx, scene, sd, stream, flush, frame, torch, local) -> dict:
    """Two costs beyond the headline frame, each the mean of 2 timed frames after 1 (CUDA events, L2 flushed):
    the frame with denoiser feature films (albedo and normal), and the frame with vkrt's full material stack: every
    third sphere glass (IOR 1.5, Abbe number 40, absorption 0.5 with tint (0.8, 0.9, 1)), every third clear-coated
    with an Oren-Nayar base, every third subsurface, which runs the full-stack kernels (transmissive interface,
    media, per-lane hero pdfs, transmission-aware shadow rays)."""
    import copy
    from vkrt_gb300 import RenderContext, abi
    out = {}
    ctx.set_denoiser_features(True)
    _device_frames(ctx, sd, stream, flush, frame, 1, torch)
    fms, frays, _ = _device_frames(ctx, sd, stream, flush, frame, 2, torch)
    ctx.set_denoiser_features(False)
    out["features"] = {"ms_per_frame": round(float(np.mean(fms)), 3),
                       "value": round(frays / (sum(fms) * 1e-3) / 1e6, 2), "unit": "Mrays/s"}
    s = copy.copy(scene)
    m = scene.materials.copy()
    n = len(m)
    glass, coat, sss = np.arange(0, n, 3), np.arange(1, n, 3), np.arange(2, n, 3)
    m["transmission"][glass] = 1.0
    m["metallic"][glass] = 0.0
    m["roughness"][glass] = 0.05
    m["baseColor"][glass] = 1.0
    m["abbeNumber"][glass] = 40.0
    m["absorptionCoefficient"][glass] = 0.5
    m["attenuationColor"][glass] = (0.8, 0.9, 1.0)
    m["clearcoat"][coat] = 1.0
    m["clearcoatGloss"][coat] = 0.8
    m["diffuseRoughness"][coat] = 0.6
    m["subsurface"][sss] = 0.7
    s.materials = m
    mctx = RenderContext(device=local, rng_mode=abi.RNG_PCG32, rng_seed=1, environment_sampling=abi.ENV_IMPORTANCE,
                         integrator=abi.INTEGRATOR_WAVEFRONT)
    mctx.upload_scene(s)
    mstream = torch.cuda.ExternalStream(mctx.stream, device=torch.device("cuda", local))
    msd = s.scene_data.copy()
    _device_frames(mctx, msd, mstream, flush, frame, 1, torch)
    mms, mrays, _ = _device_frames(mctx, msd, mstream, flush, frame, 2, torch)
    mctx.close()
    out["materials_full"] = {"workload": "the headline frame with 1/3 glass (dispersive, absorbing), 1/3 clear coat "
                                         "over Oren-Nayar, 1/3 subsurface spheres", "ms_per_frame":
                             round(float(np.mean(mms)), 3), "value": round(mrays / (sum(mms) * 1e-3) / 1e6, 2),
                             "unit": "Mrays/s"}
    return out


def run_ours(args) -> dict | None:
    import torch
    from vkrt_gb300 import RenderContext, abi

    rank, world, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    scene = build_scene()
    ctx = RenderContext(device=local, rng_mode=abi.RNG_PCG32, rng_seed=1, environment_sampling=abi.ENV_IMPORTANCE,
                        integrator=abi.INTEGRATOR_WAVEFRONT)
    table, info = ctx.generate_rgb2spec(64)  # device rgb2spec fit (setup, not timed)
    scene.rgb2spec = table
    scene.scene_data["rgb2specSRGB"] = info
    ctx.upload_scene(scene)
    if args.stage_launches:  # stage kernels launched one by one instead of one conditional graph (for ncu)
        ctx.set_wavefront_config(useGraph=0)
    sd = scene.scene_data.copy()
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    frame = [rank * 100000]

    _device_frames(ctx, sd, stream, flush, frame, args.warmup, torch)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.nvtx.range_push("timed")
    ms, rays, launches = _device_frames(ctx, sd, stream, flush, frame, args.steps, torch)
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    total_ms = float(sum(ms))
    if world > 1:
        t = torch.tensor([total_ms], device=f"cuda:{local}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
        rt = torch.tensor([float(rays)], device=f"cuda:{local}")
        torch.distributed.all_reduce(rt)
        rays_all = int(rt.item())
    else:
        rays_all = rays
    value = rays_all / (total_ms * 1e-3) / 1e6
    mean_ms = total_ms / args.steps

    # profiling frame: stage-by-stage launches, device timers and fetch-byte counting (not part of the value)
    ctx.set_wavefront_config(profileStages=1)
    sd["frameNumber"] = frame[0]
    frame[0] += 1
    with torch.cuda.stream(stream):
        flush.zero_()
    ctx.render_frame(sd)
    ctx.sync()
    pst = ctx.stats()
    ctx.set_wavefront_config(profileStages=0)
    stage_ms = {n: round(float(v), 3) for n, v in zip(abi.WAVEFRONT_STAGES, pst["stageMs"])}
    peak, peak_kind = _peaks()
    closest_bytes = pst["nodeFetchBytes"] + pst["triFetchBytes"]
    shadow_bytes = pst["shadowNodeFetchBytes"] + pst["shadowTriFetchBytes"]
    isect_ms = max(stage_ms["intersect"], 1e-6)
    shadow_ms = max(stage_ms["shadow"], 1e-6)
    achieved = closest_bytes / (isect_ms * 1e-3) / 1e9
    isect_launches = 2 * pst["wavefrontBodies"]
    traffic = _traffic_per_launch()  # the committed capture is of this frame (build_scene's defaults)

    # the same frame by the megakernel
    mctx = RenderContext(device=local, rng_mode=abi.RNG_PCG32, rng_seed=1, environment_sampling=abi.ENV_IMPORTANCE,
                         integrator=abi.INTEGRATOR_MEGAKERNEL)
    mctx.upload_scene(scene)
    mstream = torch.cuda.ExternalStream(mctx.stream, device=torch.device("cuda", local))
    msd = scene.scene_data.copy()
    _device_frames(mctx, msd, mstream, flush, frame, 1, torch)
    mms, mrays, _ = _device_frames(mctx, msd, mstream, flush, frame, 2, torch)
    mctx.close()
    mega_ms = float(np.mean(mms))

    # end to end through the C ABI: SceneData from pinned host memory in, accumulation to pinned host memory out
    host_sd = torch.empty(abi.SCENE_DATA.itemsize, dtype=torch.uint8, pin_memory=True)
    sd_view = np.frombuffer(host_sd.numpy(), dtype=abi.SCENE_DATA)
    sd_view[:] = sd
    out = torch.empty((ctx.height, ctx.width, 4), dtype=torch.float32, pin_memory=True)
    out_np = out.numpy()
    e2e_steps = max(1, min(args.steps, 5))
    ctx.sync()
    t0 = time.perf_counter()
    e2e_rays = 0
    for k in range(e2e_steps):
        sd_view["frameNumber"] = frame[0]
        frame[0] += 1
        ctx.render_frame(sd_view)
        ctx.read_accumulation(out_np)
        e2e_rays += _rays(ctx.stats())
    e2e_s = time.perf_counter() - t0
    e2e_value = e2e_rays / e2e_s / 1e6

    overlay = selection_overlay_measure(ctx, sd, stream, torch)
    extra = features_and_materials_measure(ctx, scene, sd, stream, flush, frame, torch, local) if world == 1 else {}

    result = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(mean_ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded icosphere field, procedural sky)",
        "config": _config(1920, 1080, 16, 12, scene.triangle_count,
                          {"integrator": "wavefront (one CUDA-graph launch per frame)",
                           "parallelism": f"replicas x{world} (independent sample sets)",
                           "rays_per_frame": int(rays / args.steps), "bvh_nodes": pst["bvhNodeCount"],
                           "bvh_mbytes": round(pst["bvhBytes"] / 2 ** 20, 1)}),
        "e2e": {"value": round(e2e_value, 2), "unit": "Mrays/s", "h2d_bytes_per_step": abi.SCENE_DATA.itemsize,
                "d2h_bytes_per_step": int(out.numel() * 4), "steps": e2e_steps},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": "kWfIntersect",
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst copy)",
                     "algorithmic_bytes_per_launch": int(closest_bytes / max(isect_launches, 1)),
                     "launches": isect_launches,
                     "note": "80 B per node visit + 48 B per triangle test of closest-hit rays / kernel time, "
                             "profiling frame; the 65 MB BVH is L2-resident, so frac > 1 is possible",
                     "shadow_kernel": {"kernel": "kWfShadow",
                                       "achieved": round(shadow_bytes / (shadow_ms * 1e-3) / 1e9, 1),
                                       "frac": round(shadow_bytes / (shadow_ms * 1e-3) / 1e9 / peak, 4)},
                     "stage_ms": stage_ms},
        "megakernel": {"ms_per_step": round(mega_ms, 2), "value": round(mrays / (sum(mms) * 1e-3) / 1e6, 2),
                       "unit": "Mrays/s", "speedup_of_wavefront": round(mega_ms / mean_ms, 2)},
        "clocks": clk,
        "gpu_launches": int(launches),
        "selection_overlay": overlay,
        **extra,
    }
    if rank == 0 and world == 1 and not args.no_adjoint:
        result["adjoint"] = adjoint_ratio(local)
    if rank == 0 and world == 1 and not args.no_batch:
        result["batch"] = batch_measure(local)
    if rank == 0 and world == 1 and not args.no_convergence:
        result["convergence"] = convergence_measure(local, scene, mega_ms)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(scene, budget_s=args.cpu_seconds)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return result if rank == 0 else None


def cpu_baseline(scene, budget_s: float = 12.0, threads: int = 0) -> dict:
    """The oracle (CPU restatement of vkrt's integrator, FP32) on all host cores, rows of the same frame."""
    from oracle import cpu
    from vkrt_gb300 import abi

    import copy
    sd = scene.scene_data.copy()
    if scene.rgb2spec is None:
        # no device table on this path: the oracle's own fit (the per-lookup cost does not depend on res), on a copy
        # of the scene so that repeated calls see the scene as given
        scene = copy.copy(scene)
        scene.rgb2spec = cpu.rgb2spec_generate(16, threads)
        sd["rgb2specSRGB"] = (16, 0, 16)
    orc = cpu.OracleScene(scene, environment_sampling=abi.ENV_IMPORTANCE)
    ncores = threads or os.cpu_count() or 1
    height = int(sd["viewportRect"][0][1] + sd["viewportRect"][0][3])
    mid = height // 2
    # calibration on a block of rows at the frame's centre, then a block sized to the budget (centred, clamped)
    rows = max(1, min(height, 8))
    t0 = time.perf_counter()
    acc, st = orc.render(sd, rng_mode=abi.RNG_PCG32, rows=(mid - rows // 2, mid - rows // 2 + rows), threads=threads)
    dt = time.perf_counter() - t0
    rows = int(max(1, min(height, rows * budget_s / max(dt, 1e-3))))
    lo = max(0, min(height - rows, mid - rows // 2))
    t0 = time.perf_counter()
    acc, st = orc.render(sd, rng_mode=abi.RNG_PCG32, rows=(lo, lo + rows), threads=threads)
    dt = time.perf_counter() - t0
    rays = st["primaryRays"] + st["extensionRays"] + st["shadowRays"]
    orc.close()
    return {"value": round(rays / dt / 1e6, 3), "unit": "Mrays/s", "cores": ncores, "kind": "port",
            "sample": f"{rows} rows x {int(sd['viewportRect'][0][2])} px x {int(sd['samplesPerPixel'][0])} spp of the same "
                      f"frame ({rays} rays, {dt:.1f} s)"}


def run_reference(args) -> dict | None:
    rank, world, _ = _dist()
    if rank != 0:
        return None
    scene = build_scene()
    steps = []
    res = None
    for k in range(args.warmup + args.steps):
        r = cpu_baseline(scene, budget_s=args.cpu_seconds)
        if k >= args.warmup:
            steps.append(r)
        res = r
    value = float(np.mean([s["value"] for s in steps]))
    return {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded icosphere field, procedural sky)",
            "config": _config(1920, 1080, 16, 12, scene.triangle_count),
            "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": res["cores"], "kind": "port",
                             "sample": res["sample"]},
            "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "vkrt's own renderer needs Vulkan ray tracing (no graphics stack on this box): the CPU "
                    "restatement of its integrator stands in"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-convergence", action="store_true")
    ap.add_argument("--stage-launches", action="store_true",
                    help="launch the wavefront stages one by one instead of as one CUDA graph (ncu cannot profile "
                         "kernel nodes of graphs with conditional nodes)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    res = run_reference(args) if args.impl == "reference" else run_ours(args)
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
