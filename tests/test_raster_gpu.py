"""The raster pass on the GPU (fnd_rt_raster_draw) against its scalar
restatement (oracle/raster_oracle.cpp): every byte equal, for the reference
renderer's quad and uniforms at several times at 1920x1080, for a random
triangle list without culling, and through a device output buffer."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def texture(seed=1, w=256, h=192):
    rng = np.random.default_rng(seed)
    t = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    t[..., 3] = 255
    return t


def test_reference_quad_matches_oracle(built):
    import foundation_gb300 as fg
    from foundation_gb300 import rt
    tex = texture()
    quad = rt.REFERENCE_QUAD.view(np.float32).reshape(4, 7)
    with fg.Context(0) as ctx:
        for t in (0.0, 0.37, 1.5, 3.99):
            m, v, p = rt.raster_uniforms(t, 1920 / 1080)
            got = ctx.raster_draw(1920, 1080, m, v, p, tex)
            want = O.raster_draw(1920, 1080, m, v, p, tex, quad, rt.REFERENCE_QUAD_INDICES)
            assert np.array_equal(got, want), (t, int((got != want).any(-1).sum()))
            assert (got[..., :3].sum(-1) > 0).mean() > 0.02


def test_triangle_list_and_device_output(built):
    import torch
    import foundation_gb300 as fg
    from foundation_gb300 import rt
    rng = np.random.default_rng(7)
    n = 60
    verts = np.zeros(3 * n, rt.RASTER_VERTEX_DTYPE)
    verts["pos"] = rng.uniform(-1.3, 1.3, (3 * n, 2))
    verts["color"] = rng.uniform(0, 1, (3 * n, 3))
    verts["uv"] = rng.uniform(-2, 3, (3 * n, 2))
    idx = np.arange(3 * n, dtype=np.uint16)
    eye = np.eye(4, dtype=np.float32).ravel(order="F")
    persp = eye.copy()
    persp[3] = 0.2  # w = 1 + 0.2 x: a perspective divide with w != 1
    tex = texture(3, 64, 64)
    with fg.Context(0) as ctx:
        got = ctx.raster_draw(333, 177, eye, eye, persp, tex, verts, idx, clear=(0.1, 0.2, 0.3, 0.0), cull_back=False)
        want = O.raster_draw(333, 177, eye, eye, persp, tex, verts.view(np.float32).reshape(-1, 7), idx,
                             clear=(0.1, 0.2, 0.3, 0.0), cull_back=False)
        assert np.array_equal(got, want), int((got != want).any(-1).sum())
        dev = torch.empty(333 * 177 * 4, dtype=torch.uint8, device="cuda")
        ctx.raster_draw(333, 177, eye, eye, persp, tex, verts, idx, clear=(0.1, 0.2, 0.3, 0.0), cull_back=False,
                        out=dev)
        ctx.sync()
        assert np.array_equal(dev.cpu().numpy().reshape(177, 333, 4), got)
        with pytest.raises(fg.FndError):
            ctx.raster_draw(64, 64, eye, eye, eye, tex, verts, np.array([0, 1, 999], np.uint16))
