"""Raster-pass restatement on the CPU: the reference's per-frame uniforms
(fnd_rt_raster_uniforms, host code of the library) against a float32
restatement of the glm formulas, and the scalar raster oracle's rules:
gap-free coverage of shared edges, back-face culling, the reference quad."""
import math

import numpy as np
import pytest

import oracle as O

W, H = 160, 90


def glm_uniforms(t, aspect):
    f32 = np.float32
    deg = f32(0.01745329251994329576923690768489)
    ang = f32(t) * (f32(90.0) * deg)
    c, s = f32(math.cos(ang)), f32(math.sin(ang))
    M = np.zeros(16, np.float32)
    M[[0, 1, 4, 5, 10, 15]] = [c, s, -s, c, c + (f32(1) - c), 1]
    eye, up = np.array([2, 2, 2], np.float32), np.array([0, 0, 1], np.float32)
    norm = lambda v: v * (f32(1) / np.sqrt(np.float32(v @ v)))  # noqa: E731
    fwd = norm(-eye)
    sv = norm(np.cross(fwd, up).astype(np.float32))
    u = np.cross(sv, fwd).astype(np.float32)
    V = np.zeros(16, np.float32)
    V[[0, 4, 8]], V[[1, 5, 9]], V[[2, 6, 10]] = sv, u, -fwd
    V[12], V[13], V[14], V[15] = -(sv @ eye), -(u @ eye), fwd @ eye, 1
    rng = f32(math.tan(f32(45.0) * deg / f32(2))) * f32(0.1)
    P = np.zeros(16, np.float32)
    P[0] = f32(0.2) / (rng * f32(aspect) * 2)
    P[5] = -(f32(0.2) / (rng * 2))
    P[10], P[11], P[14] = -1, -1, f32(-0.2)
    return M, V, P


def test_reference_uniforms(built):
    from foundation_gb300 import rt
    for t in (0.0, 0.25, 1.7, 12.0):
        got = rt.raster_uniforms(t, 1920 / 1080)
        want = glm_uniforms(t, 1920 / 1080)
        for g, w in zip(got, want):
            np.testing.assert_allclose(g, w, rtol=2e-6, atol=1e-7)
    with pytest.raises(rt.FndError):
        rt.raster_uniforms(0.0, -1.0)


def ident():
    return np.eye(4, dtype=np.float32).ravel(order="F")


def flat_texture(v=255):
    return np.full((4, 4, 4), v, np.uint8)


def quad_verts(corners, colors):
    return np.array([[x, y, *c, 0.0, 0.0] for (x, y), c in zip(corners, colors)], np.float32)


def test_shared_edges_leave_no_gaps(built):
    # a fan of 7 triangles around an off-centre point covering the whole NDC square
    rng = np.random.default_rng(3)
    ring = [(-1, -1), (0.3, -1), (1, -1), (1, 0.2), (1, 1), (-0.4, 1), (-1, 1), (-1, -0.1)]
    centre = (0.137, -0.071)
    verts = [[*centre, 1, 1, 1, 0, 0]] + [[x, y, *rng.uniform(0.2, 1, 3), 0, 0] for x, y in ring]
    idx = []
    for i in range(len(ring)):
        a, b = 1 + i, 1 + (i + 1) % len(ring)
        idx += [0, a, b]
    out = O.raster_draw(W, H, ident(), ident(), ident(), flat_texture(), np.array(verts, np.float32),
                        np.array(idx, np.uint16), clear=(0, 0, 0, 0), cull_back=False)
    assert (out[..., 3] == 255).all(), "uncovered pixels along shared edges"


def test_back_faces_culled(built):
    # NDC y runs down the framebuffer (Vulkan), so (-.5,-.5) -> (.5,.5) -> (.5,-.5)
    # is counter-clockwise on screen (front-facing) and its mirror clockwise
    ccw = quad_verts([(-0.5, -0.5), (0.5, 0.5), (0.5, -0.5)], [(1, 0, 0)] * 3)
    cw = ccw[[0, 2, 1]]
    idx = np.array([0, 1, 2], np.uint16)
    a = O.raster_draw(W, H, ident(), ident(), ident(), flat_texture(), ccw, idx)
    b = O.raster_draw(W, H, ident(), ident(), ident(), flat_texture(), cw, idx)
    c = O.raster_draw(W, H, ident(), ident(), ident(), flat_texture(), cw, idx, cull_back=False)
    covered = lambda img: int((img[..., 0] > 0).sum())  # noqa: E731
    assert covered(a) > 0 and covered(b) == 0 and covered(c) == covered(a)


def test_reference_quad_frame(built):
    from foundation_gb300 import rt
    m, v, p = rt.raster_uniforms(0.5, W / H)
    tex = np.zeros((8, 8, 4), np.uint8)
    tex[...] = 255
    out = O.raster_draw(W, H, m, v, p, tex, rt.REFERENCE_QUAD.view(np.float32).reshape(4, 7), rt.REFERENCE_QUAD_INDICES)
    lit = out[..., :3].sum(-1) > 0
    assert 0.02 < lit.mean() < 0.6, lit.mean()
    assert (out[~lit] == [0, 0, 0, 255]).all()  # clear colour elsewhere
    ys, xs = np.nonzero(lit)
    assert abs(xs.mean() - W / 2) < W / 8 and abs(ys.mean() - H / 2) < H / 8
