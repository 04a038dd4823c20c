"""Tuned launch shapes of the traversal kernels, keyed by workload class.

The native tuner (fnd_rt_tune / fnd_rt_batch_tune) times every launch shape
(block 64/128/256 x shared short stack 4/8/16 x refill threshold
4/8/16/24 x triangle postponement off/8) on a ray batch, and for single
scenes then the best shape with each coherence-order key width (9..21 bits,
sort time included). This module runs it on representative workloads
and keeps the winners in a JSON file keyed by

    "<scene size bucket>:<coherence>:<query kind>"

where the size bucket is floor(log2(triangles)), coherence is "coherent"
(camera rays) or "incoherent", and the kind is "closest" or "any".
`apply` selects the entry of the nearest size bucket for a workload.

`tune_node_width` adds the node-width dimension: the scene is built with
nodes of at most 4, 6 and 8 children, the launch shapes are tuned on each,
and the entry keeps the fastest width (read back by `upload_options`).

The path tracer's queue widths — paths in flight per wave and the queue
length below which the tail megakernel finishes a wave — are tuned per image
size and mode by `tune_render` (key "render:<w>x<h>:<plain|cache>") and read
back with `render_options`.
"""
from __future__ import annotations

import json
import math
import os
import time

from . import rt


def size_bucket(num_tris: int) -> int:
    return int(math.floor(math.log2(max(1, num_tris))))


def key(num_tris: int, coherence: str, kind: int) -> str:
    return f"{size_bucket(num_tris)}:{coherence}:{'any' if kind == rt.QUERY_ANY else 'closest'}"


class TuneTable:
    def __init__(self, entries: dict | None = None):
        self.entries = dict(entries or {})

    @classmethod
    def load(cls, path: str) -> "TuneTable":
        if not os.path.exists(path):
            return cls()
        with open(path) as f:
            return cls(json.load(f).get("entries", {}))

    def save(self, path: str) -> None:
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump({"version": 1, "entries": self.entries}, f, indent=1, sort_keys=True)
        os.replace(tmp, path)

    def record(self, num_tris: int, coherence: str, kind: int, best: dict, table: list) -> dict:
        ms = min(e["ms"] for e in table) if table else None
        default = next((e["ms"] for e in table if (e["block"], e["short_stack"], e["refill_min"],
                                                    e.get("postpone_min", 0), e.get("sort_bits", 0)) ==
                        (128, 8, 8, 0, 0)), None)
        entry = dict(best, ms=ms, default_ms=default)
        self.entries[key(num_tris, coherence, kind)] = entry
        return entry

    def lookup(self, num_tris: int, coherence: str, kind: int) -> dict | None:
        want = size_bucket(num_tris)
        suffix = f":{coherence}:{'any' if kind == rt.QUERY_ANY else 'closest'}"
        cands = [(abs(int(k.split(':')[0]) - want), k) for k in self.entries if k.endswith(suffix)]
        if not cands:
            return None
        return self.entries[min(cands)[1]]

    def apply(self, ctx: "rt.Context", num_tris: int, coherence: str, kind: int = rt.QUERY_CLOSEST) -> dict:
        e = self.lookup(num_tris, coherence, kind)
        cfg = dict(block=128, short_stack=8, refill_min=8, postpone_min=0, sort_bits=0) if e is None else \
            dict(block=e["block"], short_stack=e["short_stack"], refill_min=e["refill_min"],
                 postpone_min=e.get("postpone_min", 0), sort_bits=e.get("sort_bits", 0))
        ctx.set_trace_config(**cfg)
        return cfg


def tune_workload(ctx: "rt.Context", table: TuneTable, scene: "rt.Scene", rays_dev, coherence: str,
                  kind: int = rt.QUERY_CLOSEST, reps: int = 3) -> dict:
    best, entries = ctx.tune(scene, rays_dev, kind=kind, reps=reps)
    return table.record(scene.info()["num_tris"], coherence, kind, best, entries)


def tune_node_width(ctx: "rt.Context", table: TuneTable, verts, idx, rays_dev, coherence: str,
                    kind: int = rt.QUERY_CLOSEST, widths=(4, 6, 8), reps: int = 3, **upload_kw) -> dict:
    """The node-width dimension: builds the scene with nodes of at most w
    children for every w in `widths` (upload_kw as for Context.upload), runs
    the launch-shape tuner on each and records the width whose best shape is
    the fastest, with that shape, under the workload's key. The entry's
    "width_ms" holds every width's best time."""
    results = []
    num_tris = 0
    for w in widths:
        s = ctx.upload(verts, idx, node_width=w, **upload_kw)
        try:
            num_tris = s.info()["num_tris"]
            best, entries = ctx.tune(s, rays_dev, kind=kind, reps=reps)
        finally:
            s.close()
        results.append(dict(node_width=w, ms=min(e["ms"] for e in entries), best=best, entries=entries))
    win = min(results, key=lambda r: r["ms"])
    entry = table.record(num_tris, coherence, kind, win["best"], win["entries"])
    entry["node_width"] = win["node_width"]
    entry["width_ms"] = {str(r["node_width"]): r["ms"] for r in results}
    return entry


def upload_options(table: TuneTable, num_tris: int, coherence: str, kind: int = rt.QUERY_CLOSEST) -> dict:
    """Keyword arguments for Context.upload from the nearest tuned entry: the
    node width, if the entry was tuned over widths ({} otherwise)."""
    e = table.lookup(num_tris, coherence, kind)
    return {} if e is None or "node_width" not in e else dict(node_width=e["node_width"])


def render_key(width: int, height: int, cache: bool) -> str:
    return f"render:{width}x{height}:{'cache' if cache else 'plain'}"


def tune_render(ctx: "rt.Context", table: TuneTable, scene: "rt.Scene", width: int, height: int, camera: dict, *,
                spp: int = 2, cache: bool = False, waves=(1 << 20, 1 << 21, 1 << 22, 1 << 23),
                tails=(0, 1 << 16, 1 << 18, 1 << 20), reps: int = 2, **render_kw) -> dict:
    """Times `reps` render calls of `spp` samples per pixel for every wave
    size x tail threshold (0: automatic) and records the fastest. With
    cache=True the calls render with the radiance cache (the cache must
    exist)."""
    results = []
    for w in waves:
        for tp in tails:
            ctx.render(scene, width, height, spp, camera, wave_paths=w, tail_paths=tp, cache=cache, **render_kw)
            ctx.sync()
            best = math.inf
            for _ in range(reps):
                t0 = time.perf_counter()
                ctx.render(scene, width, height, spp, camera, wave_paths=w, tail_paths=tp, cache=cache, **render_kw)
                ctx.sync()
                best = min(best, (time.perf_counter() - t0) * 1e3)
            results.append(dict(wave_paths=w, tail_paths=tp, ms=best))
    win = min(results, key=lambda e: e["ms"])
    default = next((e["ms"] for e in results if e["wave_paths"] == (1 << 22) and e["tail_paths"] == 0), None)
    entry = dict(win, default_ms=default, spp=spp)
    table.entries[render_key(width, height, cache)] = entry
    return entry


def render_options(table: TuneTable, width: int, height: int, cache: bool = False) -> dict:
    """Keyword arguments for Context.render from a tuned entry ({} if none)."""
    e = table.entries.get(render_key(width, height, cache))
    return {} if e is None else dict(wave_paths=e["wave_paths"], tail_paths=e["tail_paths"])
