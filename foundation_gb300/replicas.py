"""Replicated traversal across ranks: one process per GPU, no data exchange.

Rays are independent and scenes are read-only, so the traversal shards by
rays: every rank holds its own copy of the scene and traces its own ray batch.
Nothing on the data path crosses ranks. The ranks meet only at a barrier on
each side of the timed region and in one max-reduction of the elapsed time,
so the job's rate is (rays of all ranks) / (slowest rank's time), per-rank work
fixed as the rank count grows (weak scaling).

Rank r's rays are rays [r n, (r + 1) n) of one seeded stream (PCG32 streams
numbered from 2^40), so the union over ranks is the same batch a single
process would draw for world x n rays.
"""
from __future__ import annotations

STREAM_BASE = 1 << 40


def stream_base(rank: int, n_rays: int) -> int:
    """First PCG32 stream of rank `rank`'s rays."""
    return STREAM_BASE + rank * n_rays


def shard_workload(kind: str, rank: int, n_rays: int):
    """(scene, rays) of one rank. kind: "cornell" (Cornell box + 200 level-3
    icospheres, rays uniform in the box) or "soup1m" (1,048,576-triangle soup
    in the unit cube, rays uniform in the cube); directions uniform on S^2."""
    from . import scenes
    if kind == "soup1m":
        sc = scenes.soup_scene(1 << 20, seed=2)
        return sc, scenes.incoherent_rays(n_rays, (0, 0, 0), (1, 1, 1), seed=2,
                                          stream_base=stream_base(rank, n_rays))
    if kind == "cornell":
        sc = scenes.cornell_scene()
        return sc, scenes.incoherent_rays(n_rays, *sc.bounds, seed=1, stream_base=stream_base(rank, n_rays))
    raise ValueError(f"unknown workload {kind!r}")


def max_over_ranks(x: float, dist=None, device=None) -> float:
    """The largest of every rank's x (x itself on one rank). dist is
    torch.distributed with an initialised group, or None."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(rays_per_rank: int, steps: int, world: int, max_seconds: float) -> float:
    """Whole-job throughput in Mrays/s: every rank's rays over the slowest
    rank's time."""
    if max_seconds <= 0.0:
        raise ValueError("elapsed time must be positive")
    return rays_per_rank * steps * world / max_seconds / 1e6
