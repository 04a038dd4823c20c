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
"""
from __future__ import annotations

import json
import math
import os

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
