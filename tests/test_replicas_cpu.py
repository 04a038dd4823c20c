"""The multi-rank (replicas) path on the CPU: two gloo ranks, each tracing its
own shard of the Cornell incoherent workload with the oracle, then one
all_gather to compare with a single process tracing the union; and the
max-over-ranks timing the bench reports. The GPU traversal is the same per
rank, so what crosses ranks (ray sharding, the time reduction, the job rate)
is what is tested here."""
import os
import socket
from datetime import timedelta

import numpy as np
import pytest

N_RAYS = 4096
WORLD = 2


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=120))
    import oracle
    from foundation_gb300 import replicas
    sc, rays = replicas.shard_workload("cornell", rank, N_RAYS)
    hits = oracle.OracleBVH(sc.verts, sc.idx).closest(rays)
    prim = torch.from_numpy(hits["prim"].astype(np.int64))
    tbits = torch.from_numpy(hits["t"].view(np.uint32).astype(np.int64))
    gp = [torch.empty_like(prim) for _ in range(world)]
    gt = [torch.empty_like(tbits) for _ in range(world)]
    dist.all_gather(gp, prim)
    dist.all_gather(gt, tbits)
    # each rank reports its own elapsed time; every rank sees the slowest
    slowest = replicas.max_over_ranks(0.25 * (rank + 1), dist)
    if rank == 0:
        np.savez(out_path, prim=torch.cat(gp).numpy(), tbits=torch.cat(gt).numpy(), slowest=slowest,
                 first=rays[:4])
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_match_one_process(built, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import oracle
    from foundation_gb300 import replicas, scenes
    out = str(tmp_path / "gathered.npz")
    mp.start_processes(_rank_main, args=(WORLD, _free_port(), out), nprocs=WORLD, join=True, start_method="spawn")
    g = np.load(out)
    # the shards are consecutive pieces of one ray stream
    sc = scenes.cornell_scene()
    union = scenes.incoherent_rays(WORLD * N_RAYS, *sc.bounds, seed=1, stream_base=replicas.STREAM_BASE)
    assert np.array_equal(union[:4], g["first"])
    _, r1 = replicas.shard_workload("cornell", 1, N_RAYS)
    assert np.array_equal(union[N_RAYS:], r1)
    ref = oracle.OracleBVH(sc.verts, sc.idx).closest(union)
    assert np.array_equal(g["prim"], ref["prim"].astype(np.int64))
    assert np.array_equal(g["tbits"], ref["t"].view(np.uint32).astype(np.int64))
    # the job's time is the slowest rank's
    assert g["slowest"] == 0.5


def test_job_rate_and_single_rank_reduction():
    from foundation_gb300 import replicas
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.job_rate(8_388_608, 10, 2, 0.05) == pytest.approx(8_388_608 * 20 / 0.05 / 1e6)
    with pytest.raises(ValueError):
        replicas.job_rate(1, 1, 1, 0.0)
    with pytest.raises(ValueError):
        replicas.shard_workload("sponza", 0, 16)
    assert replicas.stream_base(3, 100) == replicas.STREAM_BASE + 300
