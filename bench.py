"""Benchmark of the path-tracer pass on GB300.

Headline workload (one "step"): closest-hit traversal of 8,388,608 incoherent
rays (origins uniform in the Cornell box, directions uniform on the sphere)
through the 256,012-triangle Cornell-box scene with 200 level-3 icospheres —
the incoherent test of the 1920x1080 path-tracing configuration. Metric:
Mrays/s closest hit.

  value  rays / device time, rays and hits resident in HBM
  e2e    the same through the C ABI with pinned HOST buffers: every step
         copies the rays in and the hits out inside the timed region
  roofline  the traversal kernel against the bound it hits: instruction
         issue (warp instructions per ray from the committed ncu summary of
         the workload x rays / kernel time, against 4 warp instructions per
         cycle per SM at the SM clock sampled during the timed steps). Beside
         it: its L2 bytes per ray against an L2 read bandwidth measured here
         by a hand-written kernel (probe/l2_read.cu), its DRAM bytes against
         the measured HBM copy peak, and the accounting figure: algorithmic
         bytes per ray counted by the CPU oracle on the binary binned-SAH BVH
         (32 B ray + 8 B hit + 32 B per node box fetched + 36 B per triangle
         tested) x rays / kernel time, against the HBM peak
  cpu_baseline  the CPU oracle (scalar C++, all host threads) on the same
         workload, timed on this host

Output: the measured blocks beyond the headline (path tracer, 1M-triangle
soup, time to relMSE, batched and large scenes) go on one JSON line of their
own, {"bench_blocks": ...}, printed first; the contract line comes last and
carries their headline figures as scalar `target_*` keys.

Multi-GPU: the pass does not exchange data between GPUs; N ranks trace N
independent ray batches of the same size (replicas, weak scaling).

--impl reference: the reference renderer has no ray tracer; its arm times
the CPU restatement of the path (the oracle) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_RAYS = 8_388_608
METRIC = "Mrays/s closest-hit"
UNIT = "Mrays/s"
PROFILES = os.path.join(ROOT, "profiles")
# Tree of the Cornell blocks (path tracer, cache frames, time to relMSE):
# binned SAH with spatial splits, split budget 8 (the SAH stops splitting
# before the budget), collapsed to 8-wide nodes by the SAH-optimal rule; hits
# are those of any other tree.
CORNELL_BVH = dict(spatial_splits=True, split_budget=8.0, sah_collapse=True)
# Radiance cache of the cache blocks: 65,536 training paths per frame (the
# workload's figure), 6 Adam steps of 16,384 samples at lr 1e-2, queries on
# the exponential moving average (0.98) of the iterates, GGX alpha below 0.05
# counted as specular. Chosen on the Cornell time-to-relMSE workload, training
# seeds 1, 3, 5 per setting (speed-up over the plain tracer in waves of 2^25
# paths): 6 steps 3.18-3.32x over two runs; 4 / 5 / 7 / 8 / 12 steps 3.00 /
# 3.00 / 3.14 / 3.07 / 2.82x (medians); around 6 steps, averages 0.95 / 0.97
# / 0.99, batches of 12,288 / 20,480 and 12 / 24 warm-up frames were slower.
CACHE_SETTINGS = dict(train_paths=65536, train_steps=6, batch=16384, learning_rate=1e-2, weight_average=0.98,
                      specular_alpha=0.05)
# training-only frames before the first cache frame of the time-to-relMSE
# block (8 / 16 / 24 / 32 measured over 3 seeds: 16 is the fastest)
CACHE_WARMUP = 16


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--rays", type=int, default=N_RAYS)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extra", action="store_true", help="skip the path-tracer and 1M-triangle blocks")
    p.add_argument("--workload", default="cornell", choices=["cornell", "soup1m"],
                   help="traversal workload of the timed steps (cornell: the headline)")
    p.add_argument("--bvh", default="spatial", choices=["spatial", "binned"],
                   help="tree of the timed scene: binned SAH with spatial splits (default) or binned SAH alone")
    p.add_argument("--split-budget", type=float, default=8.0,
                   help="with --bvh spatial: extra references per triangle the splits may add")
    p.add_argument("--collapse", default="sah", choices=["sah", "greedy"],
                   help="binary tree -> 8-wide nodes: SAH-optimal (default) or greedy")
    p.add_argument("--extra", default="path_tracer,incoherent_1m_tris,time_to_relmse_1080p,batched_256_scenes,"
                                      "large_scene_4k",
                   help="comma-separated extra blocks to run (also: cache_frames)")
    return p.parse_args()


def workload(rank: int, n_rays: int, kind: str = "cornell"):
    from foundation_gb300 import replicas
    return replicas.shard_workload(kind, rank, n_rays)


L2_BYTES = 129 * 10**6  # GB300 L2


def l2_note(n_rays: int) -> str:
    """How the timed steps relate to L2: the default 8,388,608 rays (268 MB)
    stream past it every step; a smaller --rays keeps them in it."""
    mb = 32 * n_rays / 1e6
    if 32 * n_rays > L2_BYTES:
        return f"inputs larger than L2: {mb:.0f} MB of rays streamed per step per GPU"
    return f"inputs within L2: {mb:.1f} MB of rays per step per GPU, no flush between steps"


def config_block(sc, n_rays, world, kind: str = "cornell"):
    if kind == "soup1m":
        return {
            "workload": "soup1m incoherent closest-hit",
            "scene": "1,048,576-triangle soup in the unit cube (seed 2)",
            "scene_tris": sc.num_tris,
            "rays_per_step_per_gpu": n_rays,
            "rays": "origins uniform in the cube, directions uniform on S^2",
            "l2": l2_note(n_rays),
            "parallelism": f"replicas x{world}",
        }
    return {
        "workload": "cornell200 incoherent closest-hit",
        "scene": "Cornell box + 200 level-3 icospheres (seed 1)",
        "scene_tris": sc.num_tris,
        "rays_per_step_per_gpu": n_rays,
        "rays": "origins uniform in the box, directions uniform on S^2",
        "l2": l2_note(n_rays),
        "parallelism": f"replicas x{world}",
    }


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms."""

    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid: str | None):
        self.uuid = uuid
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            self.samples.append((time.perf_counter(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0: float, t1: float):
        rows = [p for t, p in self.samples if t0 - 0.1 <= t <= t1 + 0.1]
        mine = [p for p in rows if self.uuid is None or self.uuid.lower() in p[0].lower()]
        rows = mine or rows
        if not rows:
            rows = [p for _, p in self.samples]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return float("nan")
        sm = [num(p[1]) for p in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for p in rows:
            for name, v in zip(names, p[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.nanmedian(sm)), "sm_max_mhz": num(rows[0][2]), "reasons": sorted(reasons),
                "power_w_max": float(np.nanmax([num(p[3]) for p in rows])), "samples": len(rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profile_figures(kind: str = "cornell") -> dict:
    """Per-launch figures of the traversal kernel from the committed ncu
    summary of the workload: its machine-readable lines `key: number`
    (dram_bytes_per_launch, l2_bytes_per_launch, warp_inst_per_launch,
    issue_active_pct, rays_per_launch)."""
    path = os.path.join(PROFILES, f"trace_closest_{kind}_incoherent.txt")
    out = {}
    if not os.path.exists(path):
        return out
    keys = ("dram_bytes_per_launch", "l2_bytes_per_launch", "warp_inst_per_launch", "issue_active_pct",
            "rays_per_launch")
    for line in open(path):
        k, _, v = line.strip().partition(":")
        if k in keys:
            try:
                out[k] = float(v.split()[0])
            except (ValueError, IndexError):
                pass
    return out


def l2_read_bandwidth() -> dict:
    """L2 read bandwidth of this GPU, measured by probe/l2_read.cu: a
    persistent grid re-reads a 48 MB L2-resident buffer 64 times per launch
    with 16-byte ld.global.cg loads; best of 10 launches (CUDA events)."""
    import ctypes as C
    from foundation_gb300 import _build
    L = C.CDLL(_build.PROBE_PATH)
    L.fnd_probe_l2_read.argtypes = [C.c_uint64, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_uint64)]
    L.fnd_probe_l2_read.restype = C.c_int
    gbs, ms, nb = C.c_double(), C.c_double(), C.c_uint64()
    if L.fnd_probe_l2_read(48 << 20, 64, 10, C.byref(gbs), C.byref(ms), C.byref(nb)) != 0:
        raise RuntimeError("L2 bandwidth probe failed")
    return {"gbs": gbs.value, "ms": ms.value, "bytes_per_launch": nb.value,
            "method": "48 MB buffer re-read 64x per launch, 16 B ld.global.cg, persistent grid, best of 10"}


def algorithmic_bytes_per_ray(sc, rays, sample=1 << 20):
    import oracle
    b = oracle.OracleBVH(sc.verts, sc.idx)
    _, st = b.closest(rays[:sample], with_stats=True)
    n = min(sample, len(rays))
    nodes, tris = st["node_fetches"] / n, st["tri_tests"] / n
    return 32.0 + 8.0 + 32.0 * nodes + 36.0 * tris, nodes, tris


def trace_counters(scene, rd, hd):
    """Per-ray node fetches and triangle tests of the device traversal (the
    counting variant of the kernel, untimed) and the active-lane fraction of
    its node and triangle phases."""
    st = scene.closest(rd, hd, stats=True)
    n = max(1, st["rays"])
    return {"nodes_per_ray": st["node_fetches"] / n, "tris_per_ray": st["tri_tests"] / n,
            "node_lane_util": st["node_fetches"] / max(1, 32 * st["warp_node_steps"]),
            "tri_lane_util": st["tri_tests"] / max(1, 32 * st["warp_tri_steps"])}


def path_tracer_block(fg, torch, stream, local):
    """One 1920x1080, 64-spp frame of the Cornell scene (max depth 8, RR from
    bounce 3, NEE to the area light), timed with CUDA events on the pass's
    stream after a 4-spp warm-up frame."""
    from foundation_gb300 import scenes
    cs = scenes.cornell_scene()
    ctx = fg.Context(local, stream=stream.cuda_stream)
    s = ctx.upload(cs.verts, cs.idx, **CORNELL_BVH)
    s.set_materials(cs.tri_material, scenes.material_records(cs))
    s.set_lights(scenes.light_records(cs))
    out = torch.empty(1920 * 1080 * 3, dtype=torch.float32, device="cuda")
    ctx.render(s, 1920, 1080, 4, scenes.CORNELL_CAMERA, out=out)
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.render(s, 1920, 1080, 64, scenes.CORNELL_CAMERA, out=out)
    e1.record(stream)
    ctx.sync()
    ms = e0.elapsed_time(e1)
    st = ctx.render_stats()
    ctx.close()
    rays = st["extension_rays"] + st["shadow_rays"]
    return {"workload": "cornell200 1920x1080 64 spp, max depth 8, RR from bounce 3, NEE", "frame_ms": ms,
            "paths": st["paths"], "extension_rays": st["extension_rays"], "shadow_rays": st["shadow_rays"],
            "mrays_s_incl_shading": rays / (ms * 1e-3) / 1e6, "waves": st["waves"]}


def incoherent_1m_block(fg, torch, stream, local, n_rays=8_388_608):
    """The 1.5 Grays/s target workload: a 1,048,576-triangle soup in the unit cube
    (edge lengths log-uniform in [1e-3, 0.1], seed 2) and 8,388,608 rays with
    origins uniform in the cube and directions uniform on the sphere. Timed
    on the reference tree (binned SAH, default launch shape) and on the
    best configuration: spatial splits with a split budget of 4 or 8 extra
    references per triangle (at 8 the builder stops on the SAH before the
    budget: about 6.4 references per triangle) and the SAH-optimal collapse,
    launch shape and coherence order picked by the autotuner in set-up (the
    timed launches include the ray-sorting kernels when the tuner chose them)."""
    from foundation_gb300 import scenes
    so = scenes.soup_scene(1 << 20, seed=2)
    rays = scenes.incoherent_rays(n_rays, (0, 0, 0), (1, 1, 1), seed=2)
    ctx = fg.Context(local, stream=stream.cuda_stream)
    rd = torch.from_numpy(rays).to("cuda")
    hd = torch.empty(2 * n_rays, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()

    def time_it(s, reps=20):
        for _ in range(3):
            s.closest(rd, hd)
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            s.closest(rd, hd)
        e1.record(stream)
        ctx.sync()
        return e0.elapsed_time(e1) / reps

    s = ctx.upload(so.verts, so.idx)
    info = s.info()
    ms_ref = time_it(s)
    counters_ref = trace_counters(s, rd, hd)
    s.close()
    best = None
    for budget in (4.0, 8.0):
        s = ctx.upload(so.verts, so.idx, spatial_splits=True, split_budget=budget, sah_collapse=True)
        cfg, _ = ctx.tune(s, rd, reps=2)
        ctx.set_trace_config(**cfg)
        ms = time_it(s)
        sinfo = s.info()
        if best is None or ms < best["kernel_ms"]:
            best = {"kernel_ms": ms, "split_budget": budget, "launch_shape": cfg, "refs": sinfo["num_refs"],
                    "wide_nodes": sinfo["num_wide_nodes"], "node_bytes": sinfo["node_bytes"],
                    "tri_bytes": sinfo["tri_bytes"], "build_ms": sinfo["build_ms"],
                    "device_counters": trace_counters(s, rd, hd)}
        ctx.set_trace_config()
        s.close()
    ctx.close()
    best["mrays_s"] = n_rays / (best["kernel_ms"] * 1e-3) / 1e6
    return {"workload": "soup 1,048,576 tris, 8,388,608 incoherent rays",
            "reference_tree": {"kernel_ms": ms_ref, "mrays_s": n_rays / (ms_ref * 1e-3) / 1e6,
                               "wide_nodes": info["num_wide_nodes"], "wide_depth": info["wide_depth"],
                               "build_ms": info["build_ms"], "device_counters": counters_ref},
            "best": best, "target_mrays_s": 1500.0}


def cache_frames_block(fg, torch, stream, local, frames: int = 8):
    """Radiance-cache frames at 1920x1080 on the Cornell scene with
    CACHE_SETTINGS: `frames` training-only frames, then `frames` 1-spp cache
    frames, each timed with CUDA events (the per-frame costs behind the
    time-to-relMSE block)."""
    from foundation_gb300 import scenes
    cs = scenes.cornell_scene()
    ctx = fg.Context(local, stream=stream.cuda_stream)
    s = ctx.upload(cs.verts, cs.idx, **CORNELL_BVH)
    s.set_materials(cs.tri_material, scenes.material_records(cs))
    s.set_lights(scenes.light_records(cs))
    out = torch.empty(1920 * 1080 * 3, dtype=torch.float32, device="cuda")
    ctx.cache_create(s, seed=1, **CACHE_SETTINGS)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        ctx.sync()
        return e0.elapsed_time(e1)

    cam = scenes.CORNELL_CAMERA
    train = [timed(lambda: ctx.render(s, 1920, 1080, 1, cam, seed=f, cache=True, train_only=True))
             for f in range(frames)]
    render = [timed(lambda: ctx.render(s, 1920, 1080, 1, cam, seed=100 + f, cache=True, accumulate=f > 0, out=out))
              for f in range(frames)]
    st = ctx.render_stats()
    ctx.close()
    c = CACHE_SETTINGS
    return {"workload": f"cornell200 1920x1080, cache frames ({c['train_paths']:,} training paths, "
                        f"{c['train_steps']} x {c['batch']:,}-sample steps, weight average {c['weight_average']})",
            "train_only_ms": float(np.median(train)), "cache_frame_ms": float(np.median(render)),
            "extension_rays_last": st["extension_rays"], "shadow_rays_last": st["shadow_rays"]}


def time_to_relmse_block(fg, torch, stream, local, ref_spp: int = 8192):
    """The second half of the metric: wall time to relMSE 1e-3 at 1920x1080
    on the Cornell scene, radiance cache vs the plain tracer (8 spp per
    frame), both against a plain render of `ref_spp` spp on the same GPU.
    The cache renders 1 spp per frame with CACHE_SETTINGS after CACHE_WARMUP
    training-only frames whose time counts; its figure is the median over
    three training seeds. Also the cache's bias: its relMSE after 512
    accumulated frames."""
    from foundation_gb300 import convergence as CV
    from foundation_gb300 import scenes
    cs = scenes.cornell_scene()
    ctx = fg.Context(local, stream=stream.cuda_stream)
    s = ctx.upload(cs.verts, cs.idx, **CORNELL_BVH)
    s.set_materials(cs.tri_material, scenes.material_records(cs))
    s.set_lights(scenes.light_records(cs))
    W, H, cam = 1920, 1080, scenes.CORNELL_CAMERA
    t0 = time.perf_counter()
    ref = CV.render_reference(ctx, s, W, H, cam, ref_spp, seed=9001)
    ref_s = time.perf_counter() - t0
    half = CV.render_reference(ctx, s, W, H, cam, 1024, seed=4242)
    ref_noise = CV.relmse(half, ref) * 1024 / (ref_spp + 1024)  # relMSE of a 1024-spp image ~ noise(1024)+noise(ref)
    plain = CV.time_to_relmse(ctx, s, ref, W, H, cam, mode="plain", spp_per_frame=8, max_frames=400, stream=stream)
    # the crossing time of the cache depends on its training seed (about
    # +-5%): three seeds, the median is the figure
    runs = []
    for cseed in (1, 3, 5):
        ctx.cache_create(s, seed=cseed, **CACHE_SETTINGS)
        runs.append(CV.time_to_relmse(ctx, s, ref, W, H, cam, mode="cache", warmup=CACHE_WARMUP, max_frames=1200,
                                      stream=stream))
    cache = sorted(runs, key=lambda c: c["time_ms"] if c["reached"] else float("inf"))[1]
    # bias: a fresh cache trained 32 frames, then 512 accumulated frames
    ctx.cache_create(s, seed=2, **CACHE_SETTINGS)
    long = CV.time_to_relmse(ctx, s, ref, W, H, cam, mode="cache", warmup=CACHE_WARMUP,
                             max_frames=CACHE_WARMUP + 512, target=0.0, stream=stream)
    st = ctx.cache_stats()
    ctx.close()
    speedup = plain["time_ms"] / cache["time_ms"] if plain["reached"] and cache["reached"] else None
    return {"workload": "cornell200 1920x1080, max depth 8, RR from bounce 3, NEE; target relMSE 1e-3 "
                        "(eps 1e-2 in the denominator, FP64 reduction)",
            "reference": {"spp": ref_spp, "render_s": ref_s, "est_relmse_noise": ref_noise},
            "plain": {k: plain[k] for k in ("reached", "time_ms", "spp", "relmse")},
            "cache": {k: cache[k] for k in ("reached", "time_ms", "frames", "spp", "relmse")},
            "cache_settings": dict(CACHE_SETTINGS, warmup_frames=CACHE_WARMUP),
            "cache_time_ms_per_seed": {sd: (c["time_ms"] if c["reached"] else None) for sd, c in zip((1, 3, 5), runs)},
            "speedup_cache_vs_plain": speedup, "target_speedup": 3.0,
            "cache_relmse_after_512_frames": long["relmse"],
            "relmse_per_channel": {"plain": plain.get("relmse_rgb"), "cache": cache.get("relmse_rgb")},
            "cache_loss_last": st["loss_last"]}


def batched_block(fg, torch, stream, local, num_scenes: int = 256, reps: int = 5):
    """Batched traversal: 256 triangle soups (log-uniform 1k..500k triangles, seed 2),
    each with a log-uniform 4k..1M ray batch (half camera, half random
    closest-hit rays) and as many any-hit shadow segments, all served by ONE
    persistent launch over the job table, replayed from a CUDA graph, launch
    shape picked by the autotuner. The scenes are generated on the host cores
    (spawned workers, one scene each; identical to the serial generator) and
    built with binned SAH and the SAH-optimal collapse."""
    import concurrent.futures as cf
    import multiprocessing as mp
    from foundation_gb300 import scenes
    t0 = time.perf_counter()
    plan = scenes.batch_plan(num_scenes)
    workers = max(1, min(16, os.cpu_count() or 1))
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        work = list(ex.map(scenes.batch_item, [plan] * num_scenes, range(num_scenes), chunksize=4))
    gen_s = time.perf_counter() - t0
    ctx = fg.Context(local, stream=stream.cuda_stream)
    t0 = time.perf_counter()
    jobs, tris = [], 0
    for w in work:
        s = ctx.upload(w["scene"].verts, w["scene"].idx, sah_collapse=True)
        tris += w["scene"].num_tris
        for kind, rays in ((0, w["closest"]), (1, w["any"])):
            rd = torch.from_numpy(rays).to("cuda")
            out = torch.empty(2 * len(rays) if kind == 0 else len(rays),
                              dtype=torch.int32 if kind == 0 else torch.uint8, device="cuda")
            jobs.append((s, rd, out, kind))
    build_s = time.perf_counter() - t0
    del work
    torch.cuda.synchronize()
    batch = fg.Batch(ctx, jobs)
    best, table = batch.tune(reps=1)
    for _ in range(2):
        batch.launch()
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        batch.launch()
    e1.record(stream)
    ctx.sync()
    ms = e0.elapsed_time(e1) / reps
    total = batch.total_rays
    default_ms = next((e["ms"] for e in table if (e["block"], e["short_stack"], e["refill_min"], e["postpone_min"])
                       == (128, 8, 8, 0)), None)
    batch.close()
    ctx.close()
    return {"workload": f"{num_scenes} soups, {tris} tris, {total} rays (closest + any) per launch",
            "launch_ms": ms, "grays_s": total / (ms * 1e-3) / 1e9, "tuned": best,
            "default_shape_ms": default_ms, "jobs": 2 * num_scenes, "gen_s": gen_s, "build_upload_s": build_s,
            "graph": True}


def large_scene_block(fg, torch, stream, local, spp: int = 16, ref_spp: int = 256, warmup_frames: int = 16):
    """Large scene: heightfield terrain (2237^2 vertices, 8-octave value noise,
    seed 3) plus 4,096 level-4 icospheres, 30,970,912 triangles, lit by a
    directional sun and a constant sky; 3840x2160, max depth 6, RR from
    bounce 3. Reported: the host build (binned SAH, SAH-optimal collapse),
    incoherent closest-hit throughput on the scene and on the trees built on
    the GPU (Karras hierarchy; locally-ordered clustering), the plain tracer's 16-spp
    frame, and the radiance cache
    (training-only warm-up frames, then 1-spp frames) given the same wall
    time; both scored by relMSE against a plain render of `ref_spp` spp."""
    from foundation_gb300 import convergence as CV
    from foundation_gb300 import scenes
    t0 = time.perf_counter()
    tr = scenes.terrain_scene()
    gen_s = time.perf_counter() - t0
    ctx = fg.Context(local, stream=stream.cuda_stream)
    t0 = time.perf_counter()
    s = ctx.upload(tr.verts, tr.idx, sah_collapse=True)
    upload_s = time.perf_counter() - t0
    info = s.info()
    s.set_materials(tr.tri_material, scenes.material_records(tr))
    s.set_lights(scenes.light_records(tr))
    W, H, cam = 3840, 2160, scenes.TERRAIN_CAMERA
    kw = dict(max_depth=6, **scenes.TERRAIN_LIGHTING)
    n_rays = N_RAYS
    rd = torch.from_numpy(scenes.incoherent_rays(n_rays, *tr.bounds, seed=3)).to("cuda")
    hd = torch.empty(2 * n_rays, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        ctx.sync()
        return e0.elapsed_time(e1)

    for _ in range(2):
        s.closest(rd, hd)
    trace_ms = sum(timed(lambda: s.closest(rd, hd)) for _ in range(5)) / 5
    # the same scene built on the GPU (linear BVH + device collapse)
    t0 = time.perf_counter()
    g = ctx.upload(tr.verts, tr.idx, gpu_build=True, sah_collapse=True)
    gpu_upload_s = time.perf_counter() - t0
    ginfo = g.info()
    for _ in range(2):
        g.closest(rd, hd)
    gpu_trace_ms = sum(timed(lambda: g.closest(rd, hd)) for _ in range(5)) / 5
    g.close()
    # built on the GPU by locally-ordered clustering instead
    t0 = time.perf_counter()
    g = ctx.upload(tr.verts, tr.idx, gpu_build=True, sah_collapse=True, cluster=True)
    cl_upload_s = time.perf_counter() - t0
    cinfo = g.info()
    for _ in range(2):
        g.closest(rd, hd)
    cl_trace_ms = sum(timed(lambda: g.closest(rd, hd)) for _ in range(5)) / 5
    g.close()
    s.closest(rd, hd)
    flat_hits = hd.clone()
    ref = CV.render_reference(ctx, s, W, H, cam, ref_spp, chunk=16, seed=9001, **kw)
    inst = instanced_terrain(fg, ctx, tr, W, H, cam, kw, ref, spp, timed, rd, hd, flat_hits)
    del rd, hd, flat_hits
    out = torch.empty(W * H * 3, dtype=torch.float32, device="cuda")
    ctx.render(s, W, H, 1, cam, seed=5, out=out, **kw)  # warm-up (buffers)
    plain_ms = timed(lambda: ctx.render(s, W, H, spp, cam, seed=1, out=out, **kw))
    st = ctx.render_stats()
    r_plain = CV.relmse(out, ref)
    ctx.cache_create(s, seed=1, **CACHE_SETTINGS)
    t_cache, frames = 0.0, 0
    for f in range(warmup_frames):
        t_cache += timed(lambda: ctx.render(s, W, H, 1, cam, seed=100 + f, cache=True, train_only=True, **kw))
    while t_cache < plain_ms and frames < 256:
        t_cache += timed(lambda: ctx.render(s, W, H, 1, cam, seed=1000 + frames, cache=True, accumulate=frames > 0,
                                            out=out, **kw))
        frames += 1
    r_cache = CV.relmse(out, ref)
    # bias floor: the same cache accumulated over 128 more frames
    for f in range(128):
        ctx.render(s, W, H, 1, cam, seed=5000 + f, cache=True, accumulate=True, out=out, **kw)
    ctx.sync()
    r_bias = CV.relmse(out, ref)
    ctx.close()
    return {"workload": f"terrain 2237^2 + 4096 level-4 icospheres ({tr.num_tris} tris), sun + sky, "
                        f"{W}x{H}, max depth 6",
            "gen_s": gen_s, "upload_s": upload_s, "build_ms": info["build_ms"], "collapse_ms": info["collapse_ms"],
            "wide_nodes": info["num_wide_nodes"], "node_bytes": info["node_bytes"], "tri_bytes": info["tri_bytes"],
            "incoherent_mrays_s": n_rays / (trace_ms * 1e-3) / 1e6,
            "gpu_build": {"upload_s": gpu_upload_s, "build_ms": ginfo["build_ms"], "collapse_ms": ginfo["collapse_ms"],
                          "wide_nodes": ginfo["num_wide_nodes"],
                          "incoherent_mrays_s": n_rays / (gpu_trace_ms * 1e-3) / 1e6},
            "gpu_build_clustered": {"upload_s": cl_upload_s, "build_ms": cinfo["build_ms"],
                                    "collapse_ms": cinfo["collapse_ms"], "wide_nodes": cinfo["num_wide_nodes"],
                                    "incoherent_mrays_s": n_rays / (cl_trace_ms * 1e-3) / 1e6},
            "reference_spp": ref_spp, "est_reference_relmse": r_plain * spp / ref_spp,
            "plain": {"spp": spp, "ms": plain_ms, "relmse": r_plain, "extension_rays": st["extension_rays"],
                      "shadow_rays": st["shadow_rays"],
                      "grays_s_incl_shading": (st["extension_rays"] + st["shadow_rays"]) / (plain_ms * 1e-3) / 1e9},
            "cache_same_time": {"ms": t_cache, "warmup_frames": warmup_frames, "frames": frames, "relmse": r_cache},
            "cache_relmse_after_more_frames": {"frames": frames + 128, "relmse": r_bias,
                                               "note": "bias + reference noise floor"},
            "instanced": inst}


def instanced_terrain(fg, ctx, tr, W, H, cam, kw, ref, spp, timed, rd, hd, flat_hits):
    """The large terrain scene as a two-level scene: the terrain (built on the GPU)
    as one instance and the 4,096 spheres as instances of one level-4
    icosphere; set-up time, device memory, the incoherent closest-hit rate on
    the rays of the flattened scene's measurement (and the fraction of rays
    whose hit equals the flattened scene's: the two representations differ
    only at ulp-level ties), and the plain 16-spp frame against the same
    reference as the flattened scene."""
    from foundation_gb300 import convergence as CV
    from foundation_gb300 import scenes
    import torch
    n_inst = 4096
    grid = 2237
    n_terrain = (grid - 1) * (grid - 1) * 2
    sv, sf = scenes.icosphere(4)
    g = scenes.Pcg32Streams(3, np.arange(1 << 32, (1 << 32) + n_inst, dtype=np.uint64))
    cx, cz = g.next_f64(), g.next_f64()
    rad = 0.001 + g.next_f64() * 0.009
    cy = scenes.value_noise(cx, cz, 3) + 0.5 * rad
    t0 = time.perf_counter()
    terrain = ctx.upload(tr.verts[:grid * grid], tr.idx[:n_terrain], gpu_build=True, sah_collapse=True)
    sphere = ctx.upload(sv.astype(np.float32), sf, margin_scale=64)
    inst = [(terrain, np.eye(3, 4, dtype=np.float32), 0)]
    for k in range(n_inst):
        m = np.zeros((3, 4), np.float32)
        m[:, :3] = np.eye(3) * rad[k]
        m[:, 3] = (cx[k], cy[k], cz[k])
        inst.append((sphere, m, n_terrain + k * len(sf)))
    two = ctx.instances(inst)
    two.set_materials(tr.tri_material, scenes.material_records(tr))
    setup_s = time.perf_counter() - t0
    n_rays = rd.shape[0]
    for _ in range(2):
        two.closest(rd, hd)
    trace_ms = sum(timed(lambda: two.closest(rd, hd)) for _ in range(5)) / 5
    same = float((hd.view(-1, 2)[:, 0] == flat_hits.view(-1, 2)[:, 0]).float().mean().item())
    out = torch.empty(W * H * 3, dtype=torch.float32, device="cuda")
    ctx.render(two, W, H, 1, cam, seed=5, out=out, **kw)
    ms = timed(lambda: ctx.render(two, W, H, spp, cam, seed=1, out=out, **kw))
    r = CV.relmse(out, ref)
    mem = sum(x.info()["node_bytes"] + x.info()["tri_bytes"] for x in (terrain, sphere, two))
    two.close()
    return {"setup_s": setup_s, "device_bvh_bytes": mem, "incoherent_mrays_s": n_rays / (trace_ms * 1e-3) / 1e6,
            "same_hit_as_flattened": same, "plain": {"spp": spp, "ms": ms, "relmse": r}}


def cpu_baseline(sc, rays):
    import oracle
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    b = oracle.OracleBVH(sc.verts, sc.idx)
    build_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    b.closest(rays, threads=cores)
    dt = time.perf_counter() - t0
    n1 = min(len(rays), 1 << 18)
    t0 = time.perf_counter()
    b.closest(rays[:n1], threads=1)
    dt1 = time.perf_counter() - t0
    # the integrator: the FP64 oracle path tracer on a crop of the 1080p frame
    integ = None
    if hasattr(sc, "materials") and sc.materials is not None:
        from foundation_gb300 import scenes
        crop, spp = (896, 476, 128, 128), 16
        t0 = time.perf_counter()
        oracle.pt_render(b, sc.tri_material, scenes.material_records(sc), scenes.light_records(sc),
                         scenes.CORNELL_CAMERA, 1920, 1080, spp, crop=crop, threads=cores)
        dt2 = time.perf_counter() - t0
        integ = {"paths_per_s": crop[2] * crop[3] * spp / dt2, "sample": f"{crop[2]}x{crop[3]} crop x {spp} spp of "
                 "the 1920x1080 Cornell frame, FP64 path tracer, max depth 8", "cores": cores}
    return {"value": len(rays) / dt / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"all {len(rays)} rays of one step, scalar C++ oracle on {cores} threads",
            "single_core_mrays_s": n1 / dt1 / 1e6, "bvh_build_s": build_s, "integrator": integ}


def target_figures(blocks: dict) -> dict:
    """The headline figure of each measured block as a scalar key of the
    contract line (the blocks themselves are on the line before)."""
    out = {}
    b = blocks.get("incoherent_1m_tris")
    if b:
        out["target_soup1m_mrays_s"] = b["best"]["mrays_s"]
        out["target_soup1m_goal_mrays_s"] = b["target_mrays_s"]
    b = blocks.get("time_to_relmse_1080p")
    if b:
        out["target_cache_speedup_to_relmse_1e3"] = b["speedup_cache_vs_plain"]
        out["target_cache_speedup_goal"] = b["target_speedup"]
    b = blocks.get("path_tracer")
    if b:
        out["path_tracer_1080p_64spp_ms"] = b["frame_ms"]
    b = blocks.get("batched_256_scenes")
    if b:
        out["batched_256_scenes_grays_s"] = b["grays_s"]
    b = blocks.get("large_scene_4k")
    if b and "incoherent_mrays_s" in b:
        out["large_scene_incoherent_mrays_s"] = b["incoherent_mrays_s"]
        if "gpu_build_clustered" in b:
            out["large_scene_gpu_built_mrays_s"] = b["gpu_build_clustered"]["incoherent_mrays_s"]
        if "incoherent_mrays_s" in b.get("instanced", {}):
            out["large_scene_two_level_mrays_s"] = b["instanced"]["incoherent_mrays_s"]
    return out


# ---------------------------------------------------------------------------
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    sc, rays = workload(0, args.rays, args.workload)
    b = oracle.OracleBVH(sc.verts, sc.idx)
    cores = os.cpu_count() or 1
    # every step traces the whole step's rays, like the GPU arm
    for i in range(args.warmup):
        b.closest(rays, threads=cores)
    times = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        b.closest(rays, threads=cores)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = len(rays) * args.steps / tot / 1e6
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_block(sc, args.rays, 1, args.workload), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"all {len(rays)} rays of the workload per step, scalar C++ oracle on "
                                       f"{cores} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "mos9527/Foundation has no ray tracer; its arm is the CPU restatement of the path"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    import foundation_gb300 as fg
    from foundation_gb300 import replicas
    fg.load()  # fails loudly when the native library is missing
    sc, rays = workload(rank, args.rays, args.workload)
    n = len(rays)
    stream = torch.cuda.Stream()
    ctx = fg.Context(local, stream=stream.cuda_stream)
    bvh = dict(spatial_splits=True, split_budget=args.split_budget) if args.bvh == "spatial" else {}
    bvh["sah_collapse"] = args.collapse == "sah"
    scene = ctx.upload(sc.verts, sc.idx, **bvh)
    info = scene.info()
    rd = torch.from_numpy(rays).to("cuda")
    hd = torch.empty(2 * n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()

    try:
        uuid = torch.cuda.get_device_properties(local).uuid
        uuid = str(uuid)
    except Exception:
        uuid = None
    clocks = ClockSampler(uuid)
    clocks.start()
    for _ in range(args.warmup):
        scene.closest(rd, hd)
    ctx.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            ev[i][0].record(stream)
            scene.closest(rd, hd)
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    t_wall1 = time.perf_counter()
    ctx.sync()
    if world > 1:
        dist.barrier()
    per_step = [s.elapsed_time(e) for s, e in ev]
    total_ms = ev[0][0].elapsed_time(ev[-1][1])
    clk = clocks.summary(t_wall0, t_wall1)
    total_ms = replicas.max_over_ranks(total_ms, dist, "cuda")
    value = replicas.job_rate(n, args.steps, world, total_ms * 1e-3)

    # end to end through the C ABI with pinned host buffers
    pin_in = fg.PinnedBuffer(n * 32)
    pin_out = fg.PinnedBuffer(n * 8)
    hr = pin_in.view(np.float32, (n, 8))
    hr[:] = rays
    ho = pin_out.view(fg.HIT_DTYPE, (n,))
    for _ in range(max(1, args.warmup // 2)):
        scene.closest(hr, ho)
    if world > 1:
        dist.barrier()
    e2e_steps = max(3, args.steps // 4)
    per_call = []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        scene.closest(hr, ho)
        per_call.append(time.perf_counter() - t1)
    e2e_s = time.perf_counter() - t0
    e2e_value = replicas.job_rate(n, e2e_steps, world, replicas.max_over_ranks(e2e_s, dist, "cuda"))
    # spot-check the end-to-end result against the device result
    dev_hits = hd.cpu().numpy().view(np.uint32)
    e2e_ok = bool(np.array_equal(dev_hits[0::2], ho["prim"]))
    clocks.stop()
    counters = trace_counters(scene, rd, hd)

    if rank == 0:
        peaks, peak_kind = measured_peaks()
        bpr, nodes, tris = algorithmic_bytes_per_ray(sc, rays)
        kern_ms = float(np.mean(per_step))
        kern_s = kern_ms * 1e-3
        prof = profile_figures(args.workload)
        l2 = l2_read_bandwidth()
        # issue bound: 4 warp schedulers per SM, one instruction per cycle each
        sm_mhz = clk.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        issue_peak = 4 * sms * sm_mhz * 1e6 / 1e9  # G warp instructions / s
        prof_rays = prof.get("rays_per_launch", float(n))
        inst_per_ray = prof["warp_inst_per_launch"] / prof_rays if "warp_inst_per_launch" in prof else None
        issue_achieved = inst_per_ray * n / kern_s / 1e9 if inst_per_ray else None
        l2_bpr = prof["l2_bytes_per_launch"] / prof_rays if "l2_bytes_per_launch" in prof else None
        traffic = prof["dram_bytes_per_launch"] * n / prof_rays if "dram_bytes_per_launch" in prof else None
        algo_gbs = bpr * n / kern_s / 1e9
        roofline = {
            "bound": "issue", "achieved": issue_achieved, "peak": issue_peak, "unit": "G warp-inst/s",
            "frac": issue_achieved / issue_peak if issue_achieved else None, "traffic": traffic,
            "warp_inst_per_ray": inst_per_ray, "issue_active_ncu": prof.get("issue_active_pct"),
            "peak_source": f"4 warp-inst/cycle/SM x {sms} SMs x {sm_mhz:g} MHz (median SM clock, timed steps)",
            "kernel_ms_avg": kern_ms,
            "l2_bytes_per_ray": l2_bpr, "l2_gbs": l2_bpr * n / kern_s / 1e9 if l2_bpr else None,
            "l2_peak_gbs": l2["gbs"], "l2_frac": (l2_bpr * n / kern_s / 1e9) / l2["gbs"] if l2_bpr else None,
            "hbm_gbs": traffic / kern_s / 1e9 if traffic else None, "hbm_peak_gbs": peaks["hbm_gbs"],
            "hbm_frac": traffic / kern_s / 1e9 / peaks["hbm_gbs"] if traffic else None,
            "hbm_peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)",
            "accounting_bytes_per_ray": bpr, "accounting_gbs": algo_gbs,
            "accounting_frac_of_hbm": algo_gbs / peaks["hbm_gbs"],
            "profile": f"profiles/trace_closest_{args.workload}_incoherent.txt",
        }
        blocks_out = {
            "bvh": ("binned SAH 32 bins, <=4 tris/leaf" +
                    (f", spatial splits (split budget {args.split_budget:g})" if args.bvh == "spatial" else "") +
                    (", SAH-optimal collapse" if args.collapse == "sah" else ", greedy collapse") +
                    " to 8-wide compressed nodes"),
            "scene_info": {k: info[k] for k in ("num_wide_nodes", "num_refs", "wide_depth", "node_bytes", "tri_bytes",
                                                "build_ms", "collapse_ms")},
            "roofline_detail": {"oracle_nodes_per_ray": nodes, "oracle_tris_per_ray": tris,
                                "device_counters": counters, "l2_probe": l2, "profile_figures": prof,
                                "accounting_note": "algorithmic bytes of the binary reference tree (32 B per "
                                "binary node visit, 36 B per triangle test, 40 B of ray and hit); the wide tree "
                                "fetches fewer bytes, from L1 and L2, so this figure is an accounting unit and "
                                "not a position against HBM"},
            "e2e_ms_per_call": {"min": 1e3 * min(per_call), "median": 1e3 * float(np.median(per_call)),
                                "max": 1e3 * max(per_call)},
        }
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_block(sc, n, world, args.workload),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 32, "d2h_bytes_per_step": n * 8,
                    "steps": e2e_steps, "matches_device_result": e2e_ok},
            "gpu_launches": args.steps,
            "roofline": roofline,
            "clocks": clk,
        }
        if not args.no_extra:
            blocks = {"path_tracer": path_tracer_block, "incoherent_1m_tris": incoherent_1m_block,
                      "time_to_relmse_1080p": time_to_relmse_block, "batched_256_scenes": batched_block,
                      "large_scene_4k": large_scene_block, "cache_frames": cache_frames_block}
            for name in [x for x in args.extra.split(",") if x]:
                blocks_out[name] = blocks[name](fg, torch, stream, local)
            line.update(target_figures(blocks_out))
        if not args.no_cpu_baseline and world == 1:
            cb = cpu_baseline(sc, rays)
            blocks_out["cpu_baseline_detail"] = cb
            line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        print(json.dumps({"bench_blocks": blocks_out}), flush=True)
        print(json.dumps(line), flush=True)
    scene.close()
    ctx.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
