"""Renders frames of the seeded spectral icosphere field and prints their counters, for profiling runs.

    python -m vkrt_gb300.profile --width 640 --height 360 --spp 4 --frames 1 --warmup 0 --stage-launches

prints one JSON line: rays by kind, node/triangle fetch bytes (with --stage-launches, which launches the wavefront
stages one by one and times them), per-stage device milliseconds and the frame's device time. Under ncu, the kernels of
every rendered frame (warm-up included) are captured; --warmup 0 --frames 1 keeps the capture to one frame.
--cache renders with the radiance cache (default settings: 2^16 training paths and 4 training steps per frame, render
paths ending at bounce 2), so its training and inference kernels run in every frame.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import RenderContext, abi, scenes


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser()
    ap.add_argument("--width", type=int, default=640)
    ap.add_argument("--height", type=int, default=360)
    ap.add_argument("--spp", type=int, default=4)
    ap.add_argument("--depth", type=int, default=12)
    ap.add_argument("--spheres", type=int, default=800)
    ap.add_argument("--frames", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=0)
    ap.add_argument("--integrator", choices=["wavefront", "megakernel"], default="wavefront")
    ap.add_argument("--stage-launches", action="store_true")
    ap.add_argument("--rgb", action="store_true", help="RGB transport instead of hero spectral")
    ap.add_argument("--cache", action="store_true", help="render with the radiance cache (wavefront only)")
    ap.add_argument("--shade-blocks", type=int, default=0, help="shade kernel residency (blocks per SM; 0 = default)")
    a = ap.parse_args(argv)
    import torch

    scene = scenes.icosphere_field(n_spheres=a.spheres, width=a.width, height=a.height, spp=a.spp, max_depth=a.depth,
                                   seed=1, spectral=not a.rgb)
    integ = abi.INTEGRATOR_WAVEFRONT if a.integrator == "wavefront" else abi.INTEGRATOR_MEGAKERNEL
    ctx = RenderContext(rng_mode=abi.RNG_PCG32, environment_sampling=abi.ENV_IMPORTANCE, integrator=integ)
    if not a.rgb:
        scene.rgb2spec, info = ctx.generate_rgb2spec(64)
        scene.scene_data["rgb2specSRGB"] = info
    ctx.upload_scene(scene)
    if a.stage_launches:
        ctx.set_wavefront_config(profileStages=1)
    if a.shade_blocks:
        ctx.set_wavefront_config(shadeBlocksPerSM=a.shade_blocks)
    if a.cache:
        ctx.nrc_configure(enabled=1)
    stream = torch.cuda.ExternalStream(ctx.stream)
    sd = scene.scene_data.copy()
    out = {}
    for f in range(a.warmup + a.frames):
        sd["frameNumber"] = f
        ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev[0].record(stream)
        ctx.render_frame(sd)
        ev[1].record(stream)
        ctx.sync()
        st = ctx.stats()
        if f >= a.warmup:
            for k in ("primaryRays", "extensionRays", "shadowRays", "nodeFetchBytes", "triFetchBytes",
                      "shadowNodeFetchBytes", "shadowTriFetchBytes", "kernelLaunches", "wavefrontBodies",
                      "cacheTrainingRecords"):
                out[k] = out.get(k, 0) + int(st[k])
            ms = dict(zip(abi.WAVEFRONT_STAGES, st["stageMs"]))
            for k, v in ms.items():
                out.setdefault("stage_ms", {})[k] = round(out.get("stage_ms", {}).get(k, 0.0) + float(v), 3)
            out["frame_ms"] = round(out.get("frame_ms", 0.0) + ev[0].elapsed_time(ev[1]), 3)
    out["workload"] = {"width": a.width, "height": a.height, "spp": a.spp, "depth": a.depth, "spheres": a.spheres,
                       "triangles": scene.triangle_count, "frames": a.frames, "integrator": a.integrator,
                       "mode": "rgb" if a.rgb else "hero-spectral", "cache": a.cache,
                       "shade_blocks": a.shade_blocks}
    ctx.close()
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main()
