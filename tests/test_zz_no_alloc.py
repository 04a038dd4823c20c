"""The no-allocation closest-hit entry point (fnd_rt_trace_closest_noalloc).

It serves callers that cannot call cudaMalloc when they trace (for example a
plugin running inside a host application's frame callback, where device
allocations are forbidden or all device memory was handed out up front): it
stages rays and hits through a fixed device array instead of allocating.
These tests call it through the C ABI, twice in a row, and require results
identical to fnd_rt_trace_closest's (ids exact, t bit-identical: the same
tolerance as every other traversal test). This file is collected last so a
run that stops at the first failure has run every other test already.
"""
import ctypes as C

import numpy as np
import pytest

from foundation_gb300 import scenes as S

pytestmark = pytest.mark.gpu

MAX_RAYS = 65536


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def test_noalloc_matches_trace_closest_on_two_calls(built):
    import torch
    import foundation_gb300 as fg
    from foundation_gb300 import rt
    lib = rt.load()
    with fg.Context(0) as ctx:
        cs = S.cornell_scene()
        scene = ctx.upload(cs.verts, cs.idx)
        rays1 = S.incoherent_rays(MAX_RAYS, *cs.bounds, seed=21)
        rays2 = S.camera_rays(200, 150, **S.CORNELL_CAMERA)  # 30,000 rays: fewer than the first call
        ref1 = scene.closest(rays1)
        ref2 = scene.closest(rays2)
        out1 = np.empty(len(rays1), fg.HIT_DTYPE)
        out2 = np.empty(len(rays2), fg.HIT_DTYPE)
        rc1 = lib.fnd_rt_trace_closest_noalloc(scene.handle, _p(rays1), len(rays1), _p(out1), None)
        free_after_first = torch.cuda.mem_get_info(0)[0]
        rc2 = lib.fnd_rt_trace_closest_noalloc(scene.handle, _p(rays2), len(rays2), _p(out2), None)
        free_after_second = torch.cuda.mem_get_info(0)[0]
        assert rc1 == 0, lib.fnd_rt_last_error(ctx.handle)
        assert rc2 == 0, lib.fnd_rt_last_error(ctx.handle)
        for out, ref in ((out1, ref1), (out2, ref2)):
            assert np.array_equal(out["prim"], ref["prim"])
            assert np.array_equal(out["t"].view(np.uint32), ref["t"].view(np.uint32))
        # the second call allocated no device memory
        assert free_after_second == free_after_first
        scene.close()


def test_noalloc_rejects_batches_over_the_limit(built):
    import foundation_gb300 as fg
    from foundation_gb300 import rt
    lib = rt.load()
    with fg.Context(0) as ctx:
        v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
        scene = ctx.upload(v, np.array([[0, 1, 2]], np.uint32))
        big = np.zeros((MAX_RAYS + 1, 8), np.float32)
        out = np.empty(MAX_RAYS + 1, fg.HIT_DTYPE)
        rc = lib.fnd_rt_trace_closest_noalloc(scene.handle, _p(big), len(big), _p(out), None)
        assert rc == -1
        assert b"no-allocation limit" in lib.fnd_rt_last_error(ctx.handle)
        # the context stays usable, and a batch at the limit is accepted
        ok = np.zeros((MAX_RAYS, 8), np.float32)
        ok[:, 0:3] = [0.2, 0.2, 1.0]
        ok[:, 6] = -1.0
        ok[:, 7] = np.inf
        out_ok = np.empty(MAX_RAYS, fg.HIT_DTYPE)
        assert lib.fnd_rt_trace_closest_noalloc(scene.handle, _p(ok), len(ok), _p(out_ok), None) == 0
        assert (out_ok["prim"] == 0).all() and (out_ok["t"] == 1.0).all()
        scene.close()


def test_noalloc_on_a_caller_stream_and_empty_batch(built):
    """A caller-supplied stream (not the context's) under a non-default
    launch shape gives the same hits, and n == 0 returns success without
    touching the buffers."""
    import torch
    import foundation_gb300 as fg
    from foundation_gb300 import rt
    lib = rt.load()
    with fg.Context(0) as ctx:
        cs = S.cornell_scene()
        scene = ctx.upload(cs.verts, cs.idx, spatial_splits=True, split_budget=8.0, sah_collapse=True)
        rays = S.incoherent_rays(40000, *cs.bounds, seed=5)
        ref = scene.closest(rays)
        # a launch shape other than the default (64-thread blocks, short stack 4)
        ctx.set_trace_config(block=64, short_stack=4, refill_min=16)
        side = torch.cuda.Stream(device=0)
        out = np.empty(len(rays), fg.HIT_DTYPE)
        rc = lib.fnd_rt_trace_closest_noalloc(scene.handle, _p(rays), len(rays), _p(out), C.c_void_p(side.cuda_stream))
        assert rc == 0, lib.fnd_rt_last_error(ctx.handle)
        assert np.array_equal(out["prim"], ref["prim"])
        assert np.array_equal(out["t"].view(np.uint32), ref["t"].view(np.uint32))
        empty = np.empty(1, fg.HIT_DTYPE)
        empty["prim"] = 7
        assert lib.fnd_rt_trace_closest_noalloc(scene.handle, None, 0, _p(empty), None) == 0
        assert empty["prim"][0] == 7
        scene.close()
