"""FP64 path-tracing oracle on the CPU: furnace known answer and the
committed FP64 Cornell fixture."""
import os

import numpy as np

import oracle as O
from foundation_gb300 import scenes as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FURNACE_CAM = dict(eye=(0.0, 0.0, 4.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), vfov_deg=45.0)


def relmse(img, ref, eps=1e-2):
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + eps)))


def test_lambert_furnace_is_exact():
    # convex Lambertian sphere of albedo 0.5 under a white sky: every path
    # that hits it scatters once and escapes, so the pixel is exactly 0.5
    sc = S.sphere_scene(4, 1.0)
    b = O.OracleBVH(sc.verts, sc.idx)
    img = O.pt_render(b, sc.tri_material, S.material_records(sc), S.light_records(sc), FURNACE_CAM, 32, 32, 8,
                      sky=(1, 1, 1))
    assert np.allclose(img[12:20, 12:20], 0.5, atol=1e-12)
    assert img.min() >= 0.5 - 1e-12 and img.max() <= 1.0 + 1e-12
    assert np.allclose(img[0, 0], 1.0)


def test_cornell_fixture_regression():
    g = np.load(os.path.join(GOLDEN, "cornell_fp64_96x54.npz"))
    cs = S.cornell_scene()
    b = O.OracleBVH(cs.verts, cs.idx)
    img = O.pt_render(b, cs.tri_material, S.material_records(cs), S.light_records(cs), S.CORNELL_CAMERA, 96, 54,
                      256, seed=11)
    # 256 spp against the 4096 spp fixture: only sampling noise, no bias
    assert relmse(img, g["image"]) < 0.05
    assert abs(img.mean() / g["image"].mean() - 1.0) < 0.02
