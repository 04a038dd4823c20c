"""Time-to-error measurements of the path-tracer pass.

relMSE(I, R) = mean over pixels and RGB of (I - R)^2 / (R^2 + 1e-2), reduced
in FP64. The reference R is a high-spp render of the plain tracer on the
same GPU (its own relMSE against the limit is reported beside it).

time_to_relmse runs frames until the accumulated image reaches the target:
 * plain: `spp_per_frame` samples per frame, accumulated from frame 0;
 * cache: 1 sample per frame with the radiance cache (each frame also runs
   the cache's training paths and optimiser steps); the first `warmup`
   frames only train the cache (training paths and optimiser steps, no
   image), and their time counts.
Render time is measured with CUDA events on the pass's stream; the relMSE
checks between frames are outside the timed region.
"""
from __future__ import annotations

import math


def relmse(img, ref, eps: float = 1e-2) -> float:
    a = img.double()
    r = ref.double()
    return float(((a - r) ** 2 / (r * r + eps)).mean().item())


def relmse_rgb(img, ref, eps: float = 1e-2) -> list:
    """relMSE of each channel (images of interleaved RGB floats)."""
    a = img.double().reshape(-1, 3)
    r = ref.double().reshape(-1, 3)
    return [float(x) for x in ((a - r) ** 2 / (r * r + eps)).mean(0).tolist()]


def render_reference(ctx, scene, width, height, camera, spp_total: int, chunk: int = 256, seed: int = 9001, **kw):
    import torch
    out = torch.empty(width * height * 3, dtype=torch.float32, device="cuda")
    done = 0
    while done < spp_total:
        s = min(chunk, spp_total - done)
        ctx.render(scene, width, height, s, camera, seed=seed, accumulate=done > 0, out=out, **kw)
        done += s
    ctx.sync()
    return out.clone()


def time_to_relmse(ctx, scene, ref, width, height, camera, *, mode: str = "plain", target: float = 1e-3,
                   spp_per_frame: int = 1, max_frames: int = 4096, warmup: int = 0, seed: int = 7,
                   stream=None, **kw) -> dict:
    import torch
    out = torch.empty(width * height * 3, dtype=torch.float32, device="cuda")
    cache = mode == "cache"
    t_ms = 0.0
    curve = []
    spp = 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    st = stream if stream is not None else torch.cuda.current_stream()
    for f in range(max_frames):
        accumulate = f > warmup if cache else f > 0
        e0.record(st)
        ctx.render(scene, width, height, spp_per_frame, camera, seed=seed + f, accumulate=accumulate, cache=cache,
                   out=out, train_only=cache and f < warmup, **kw)
        e1.record(st)
        ctx.sync()
        t_ms += e0.elapsed_time(e1)
        if cache and f < warmup:
            continue
        spp += spp_per_frame
        r = relmse(out, ref)
        curve.append((round(t_ms, 3), spp, r))
        if r <= target:
            return {"reached": True, "time_ms": t_ms, "frames": f + 1, "spp": spp, "relmse": r,
                    "relmse_rgb": relmse_rgb(out, ref), "curve": curve[-8:]}
    return {"reached": False, "time_ms": t_ms, "frames": max_frames, "spp": spp,
            "relmse": curve[-1][2] if curve else math.nan, "relmse_rgb": relmse_rgb(out, ref), "curve": curve[-8:]}
