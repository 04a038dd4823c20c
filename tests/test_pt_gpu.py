"""GPU wavefront path tracer against the FP64 oracle: exact furnace values,
GGX furnace means, and the Cornell box against the committed 4096-spp FP64
render (relMSE = mean((I - R)^2 / (R^2 + 1e-2)))."""
import os

import numpy as np
import pytest

import oracle as O
from foundation_gb300 import scenes as S

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FURNACE_CAM = dict(eye=(0.0, 0.0, 4.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), vfov_deg=45.0)


def relmse(img, ref, eps=1e-2):
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + eps)))


@pytest.fixture(scope="module")
def ctx(built):
    import foundation_gb300 as fg
    c = fg.Context(0)
    yield c
    c.close()


def upload(ctx, sc):
    s = ctx.upload(sc.verts, sc.idx)
    s.set_materials(sc.tri_material, S.material_records(sc))
    s.set_lights(S.light_records(sc))
    return s


def test_lambert_furnace_exact(ctx):
    sc = S.sphere_scene(4, 1.0)
    s = upload(ctx, sc)
    img = ctx.render(s, 64, 64, 16, FURNACE_CAM, sky=(1, 1, 1))
    assert np.all(img[24:40, 24:40] == 0.5)
    assert img.min() >= 0.5 - 1e-6 and img.max() <= 1.0 + 1e-6
    assert np.all(img[0, 0] == 1.0)
    s.close()


def test_ggx_furnace_matches_oracle(ctx):
    sc = S.sphere_scene(4, 1.0, material=(1, 1.0, 1.0, 1.0, 0.5, 0, 0, 0))
    s = upload(ctx, sc)
    img = ctx.render(s, 48, 48, 2048, FURNACE_CAM, sky=(1, 1, 1))
    b = O.OracleBVH(sc.verts, sc.idx)
    ref = O.pt_render(b, sc.tri_material, S.material_records(sc), S.light_records(sc), FURNACE_CAM, 48, 48, 1024,
                      sky=(1, 1, 1))
    m = slice(16, 32)
    g, r = img[m, m].mean(), ref[m, m].mean()
    assert 0.5 < r < 1.0
    assert abs(g / r - 1.0) < 5e-3, (g, r)
    s.close()


def test_cornell_matches_fp64_oracle(ctx):
    g = np.load(os.path.join(GOLDEN, "cornell_fp64_96x54.npz"))
    ref = g["image"]
    cs = S.cornell_scene()
    s = upload(ctx, cs)
    a = ctx.render(s, 96, 54, 4096, S.CORNELL_CAMERA, seed=1)
    b = ctx.render(s, 96, 54, 4096, S.CORNELL_CAMERA, seed=2)
    r_ab = relmse(a, b)
    r = relmse(a, ref)
    # both sides carry sampling noise only: without bias relMSE(a, ref) ~ r_ab
    assert r < 1.5 * r_ab + 1e-5, (r, r_ab)
    assert abs(a.mean() / ref.mean() - 1.0) < 0.01
    st = ctx.render_stats()
    assert st["paths"] == 96 * 54 * 4096
    assert st["extension_rays"] >= st["paths"] and st["shadow_rays"] > 0
    s.close()


def test_accumulate(ctx):
    cs = S.cornell_scene(num_spheres=20, level=2)
    s = upload(ctx, cs)
    one = ctx.render(s, 64, 36, 8, S.CORNELL_CAMERA, seed=3)
    two = ctx.render(s, 64, 36, 8, S.CORNELL_CAMERA, seed=3, accumulate=True)
    assert ctx.render_stats()["samples_accumulated"] == 16
    assert not np.array_equal(one, two)
    full = ctx.render(s, 64, 36, 1024, S.CORNELL_CAMERA, seed=9)
    assert relmse(two, full) < relmse(one, full) * 1.2
    s.close()


def test_render_argument_errors(ctx):
    import foundation_gb300 as fg
    cs = S.cornell_scene(num_spheres=2, level=1)
    s = upload(ctx, cs)
    with pytest.raises(fg.FndError):
        ctx.render(s, 0, 10, 1, S.CORNELL_CAMERA)
    with pytest.raises(fg.FndError):
        ctx.render(s, 8, 8, 1, dict(eye=(0, 0, 0), target=(0, 0, 0)))
    with pytest.raises(fg.FndError):
        s.set_materials(np.zeros(3, np.uint32), S.material_records(cs))
    bad = S.material_records(cs)
    bad[0]["type"] = 7
    with pytest.raises(fg.FndError):
        s.set_materials(cs.tri_material, bad)
    img = ctx.render(s, 8, 8, 1, S.CORNELL_CAMERA)  # context still usable
    assert np.isfinite(img).all()
    s.close()


@pytest.mark.parametrize("cache", [False, True])
def test_tail_megakernel_matches_wavefront(ctx, cache):
    """The tail megakernel runs the same paths as the wavefront stages: the
    same extension and shadow ray counts, and images equal up to the order of
    the frame-buffer additions. Thresholds: never (wavefront), everything
    from the second interaction on, and the automatic one; and the wavefront
    with coherence-ordered secondary and shadow rays."""
    cs = S.cornell_scene()
    s = upload(ctx, cs)
    kw = dict(seed=5, sky=(0.05, 0.06, 0.08), sun_dir=(0.3, 1.0, 0.2), sun_irradiance=(0.5, 0.5, 0.4))
    if cache:
        ctx.cache_create(s, train_paths=4096, train_steps=0, batch=1024, seed=3)
    imgs, stats = [], []
    # the last variant also puts secondary and shadow rays in coherence order
    for opts, bits in ((dict(wavefront=True), 0), (dict(tail_paths=1 << 28), 0), (dict(), 0),
                       (dict(wavefront=True), 15)):
        ctx.set_trace_config(sort_bits=bits)
        imgs.append(ctx.render(s, 96, 54, 64, S.CORNELL_CAMERA, cache=cache, **kw, **opts))
        st = ctx.render_stats()
        stats.append((st["extension_rays"], st["shadow_rays"]))
    ctx.set_trace_config()
    assert len(set(stats)) == 1, stats
    assert stats[0][0] > 96 * 54 * 64
    for img in imgs[1:]:
        np.testing.assert_allclose(img, imgs[0], rtol=1e-4, atol=1e-6)
    if cache:
        ctx.cache_destroy()
    s.close()


def test_render_does_not_depend_on_the_tree(ctx):
    """Closest and any hits do not depend on the tree, so neither do the
    paths: the binned-SAH tree, the spatial-split tree (split budget 8) and
    the GPU-built tree give the same extension and shadow ray counts and
    images equal up to the order of the frame-buffer additions."""
    cs = S.cornell_scene(num_spheres=60)
    kw = dict(seed=11, sky=(0.05, 0.06, 0.08))
    imgs, stats = [], []
    for bvh in (dict(), dict(spatial_splits=True, split_budget=8.0), dict(gpu_build=True)):
        s = ctx.upload(cs.verts, cs.idx, **bvh)
        s.set_materials(cs.tri_material, S.material_records(cs))
        s.set_lights(S.light_records(cs))
        imgs.append(ctx.render(s, 96, 54, 32, S.CORNELL_CAMERA, **kw))
        st = ctx.render_stats()
        stats.append((st["extension_rays"], st["shadow_rays"]))
        s.close()
    assert len(set(stats)) == 1, stats
    for img in imgs[1:]:
        np.testing.assert_allclose(img, imgs[0], rtol=1e-4, atol=1e-6)


def test_time_to_relmse_reference_matches_fp64_oracle_on_1080p_crops(ctx):
    """The time-to-relMSE reference is the GPU's own plain render
    (convergence.render_reference, 8192 spp in the bench). Checked here at
    its full 1920x1080 geometry: three 24x24 crops of a 1024-spp reference
    render (centre, the brightest block, a block of median brightness)
    against the FP64 oracle's path tracer at 4096 spp over the same crops.
    Without bias the reference render's relMSE against the oracle is about
    0.6x the relMSE between two reference renders of different seeds; the bar
    is 1.5x, and the crop means agree within 2%."""
    from foundation_gb300 import convergence as CV
    cs = S.cornell_scene()
    s = upload(ctx, cs)
    W, H, cam = 1920, 1080, S.CORNELL_CAMERA
    a = CV.render_reference(ctx, s, W, H, cam, 1024, seed=9001).cpu().numpy().reshape(H, W, 3)
    b = CV.render_reference(ctx, s, W, H, cam, 1024, seed=4242).cpu().numpy().reshape(H, W, 3)
    s.close()
    bvh = O.OracleBVH(cs.verts, cs.idx)
    # the centre, the brightest 24x24 block of a 120-pixel grid (the light)
    # and the lit block of median brightness
    means = {(x, y): float(a[y:y + 24, x:x + 24].mean()) for x in range(0, W - 24, 120) for y in range(0, H - 24, 120)}
    lit = sorted((m, xy) for xy, m in means.items() if m > 0.0)
    picks = [(948, 528), lit[-1][1], lit[len(lit) // 2][1]]
    for x0, y0 in picks:
        crop = (x0, y0, 24, 24)
        ref = O.pt_render(bvh, cs.tri_material, S.material_records(cs), S.light_records(cs), cam, W, H, 4096,
                          crop=crop, seed=77)
        ga = a[y0:y0 + 24, x0:x0 + 24].astype(np.float64)
        gb = b[y0:y0 + 24, x0:x0 + 24].astype(np.float64)
        r_ab = relmse(ga, gb)
        r = relmse(ga, ref)
        assert r < 1.5 * r_ab + 1e-6, (crop, r, r_ab)
        assert abs(ga.mean() / ref.mean() - 1.0) < 0.02, (crop, ga.mean(), ref.mean())
