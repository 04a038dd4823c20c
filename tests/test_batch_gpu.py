"""Batched multi-scene traversal (one persistent launch over a job table,
replayed from a CUDA graph) and the launch-shape autotuner: results must
equal the CPU oracle exactly under every launch shape."""
import numpy as np
import pytest

import oracle as O
from foundation_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built):
    import foundation_gb300 as fg
    c = fg.Context(0)
    yield c
    c.close()


def check_job(sc, rays, out, kind, bvh=None):
    b = bvh or O.OracleBVH(sc.verts, sc.idx)
    if kind == 0:
        h = out.cpu().numpy().view(np.uint32)
        ref = b.closest(rays)
        assert np.array_equal(h[0::2], ref["prim"])
        assert np.array_equal(h[1::2], ref["t"].view(np.uint32))
    else:
        assert np.array_equal(out.cpu().numpy(), b.any(rays))


def make_jobs(ctx, work):
    import torch
    jobs, meta = [], []
    for w in work:
        s = ctx.upload(w["scene"].verts, w["scene"].idx)
        for kind, rays in ((0, w["closest"]), (1, w["any"])):
            rd = torch.from_numpy(rays).cuda()
            out = torch.empty(2 * len(rays) if kind == 0 else len(rays), dtype=torch.int32 if kind == 0 else
                              torch.uint8, device="cuda")
            jobs.append((s, rd, out, kind))
            meta.append((w["scene"], rays, out, kind))
    return jobs, meta


def test_batch_matches_oracle_with_graph_and_tuning(ctx):
    import torch
    import foundation_gb300 as fg
    work = S.batch_workload(12, tris=(1000, 20000), rays=(1000, 8000))
    jobs, meta = make_jobs(ctx, work)
    # an empty scene and an empty job ride along
    empty = ctx.upload(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    er = torch.from_numpy(S.cube_camera_rays(100)).cuda()
    eo = torch.full((200,), 7, dtype=torch.int32, device="cuda")
    jobs.append((empty, er, eo, 0))
    zr = torch.empty((0, 8), dtype=torch.float32, device="cuda")
    jobs.append((jobs[0][0], zr, torch.empty(0, dtype=torch.int32, device="cuda"), 0))
    torch.cuda.synchronize()
    batch = fg.Batch(ctx, jobs)
    assert batch.total_rays == sum(len(m[1]) for m in meta) + 100
    batch.launch()
    batch.launch()  # graph replay
    ctx.sync()
    bvhs = {}
    for sc, rays, out, kind in meta:
        key = id(sc)
        bvhs.setdefault(key, O.OracleBVH(sc.verts, sc.idx))
        check_job(sc, rays, out, kind, bvhs[key])
    eh = eo.cpu().numpy().view(np.uint32)
    assert (eh[0::2] == fg.INVALID_ID).all() and np.isinf(eh[1::2].view(np.float32)).all()
    best, table = batch.tune(reps=1)
    assert len(table) == 72 and best["block"] in (64, 128, 256)
    for _, _, out, _ in jobs[:-2]:
        out.zero_()
    batch.launch()
    ctx.sync()
    for sc, rays, out, kind in meta:
        check_job(sc, rays, out, kind, bvhs[id(sc)])
    batch.close()
    nog = fg.Batch(ctx, jobs[:4], graph=False)
    nog.launch()
    ctx.sync()
    for sc, rays, out, kind in meta[:4]:
        check_job(sc, rays, out, kind, bvhs[id(sc)])
    nog.close()


def test_tuner_and_launch_shapes_keep_parity(ctx):
    import torch
    import foundation_gb300 as fg
    cs = S.cornell_scene()
    s = ctx.upload(cs.verts, cs.idx)
    rays = S.incoherent_rays(1 << 18, *cs.bounds, seed=31)
    rd = torch.from_numpy(rays).cuda()
    best, table = ctx.tune(s, rd, reps=1)
    # 72 launch shapes, then the best one with 5 coherence-order key widths
    assert len(table) == 77 and all(e["ms"] > 0 for e in table)
    assert [e["sort_bits"] for e in table[72:]] == [9, 12, 15, 18, 21]
    ref = O.OracleBVH(cs.verts, cs.idx).closest(rays)
    for cfg in (best, dict(block=64, short_stack=4, refill_min=1, postpone_min=0, sort_bits=0),
                dict(block=256, short_stack=16, refill_min=32, postpone_min=8, sort_bits=6),
                dict(block=128, short_stack=4, refill_min=8, postpone_min=32, sort_bits=21),
                dict(block=128, short_stack=8, refill_min=8, postpone_min=0, sort_bits=15)):
        ctx.set_trace_config(**cfg)
        assert ctx.trace_config() == cfg
        h = s.closest(rays)
        assert np.array_equal(h["prim"], ref["prim"])
        assert np.array_equal(h["t"].view(np.uint32), ref["t"].view(np.uint32))
    with pytest.raises(fg.FndError):
        ctx.set_trace_config(block=96)
    for bad in (3, 10, 24):
        with pytest.raises(fg.FndError):
            ctx.set_trace_config(sort_bits=bad)
    ctx.set_trace_config()
    s.close()
