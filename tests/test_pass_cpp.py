"""The C++ path-tracer pass (foundation_gb300/renderer): OBJ/MTL loading on
the CPU, and a headless render through PathTracerPass on the GPU compared
with the same scene rendered through the Python binding."""
import os
import subprocess

import numpy as np
import pytest

from foundation_gb300 import scenes as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DEMO = os.path.join(ROOT, "foundation_gb300", "lib", "fnd_pass_demo")


def read_pfm(path):
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = map(int, f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), dtype="<f4" if scale < 0 else ">f4")
    return data.reshape(h, w, 3)[::-1]


def test_obj_round_trip(built, tmp_path):
    cs = S.cornell_scene(num_spheres=4, level=1)
    p = str(tmp_path / "scene.obj")
    S.write_obj(cs, p)
    out = subprocess.run([DEMO, "--parse", p], capture_output=True, text=True, check=True).stdout.splitlines()
    assert out[0] == f"verts {len(cs.verts)} tris {cs.num_tris} materials {len(cs.materials)} lights 1"
    mats = [ln for ln in out[1:] if ln.startswith("material")]
    assert "type 2" in mats[3] and "light 0" in mats[3]
    assert sum("type 1" in m for m in mats) == int((cs.materials[:, 0] == 1).sum())


def test_obj_errors(built, tmp_path):
    p = tmp_path / "bad.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nf 1 2 7\n")
    r = subprocess.run([DEMO, "--parse", str(p)], capture_output=True, text=True)
    assert r.returncode == 1 and "out of range" in r.stderr
    r = subprocess.run([DEMO, "--parse", str(tmp_path / "missing.obj")], capture_output=True, text=True)
    assert r.returncode == 1


@pytest.mark.gpu
def test_cpp_pass_matches_python_binding(built, tmp_path):
    import foundation_gb300 as fg
    cs = S.cornell_scene(num_spheres=30, level=2)
    p = str(tmp_path / "cornell.obj")
    S.write_obj(cs, p)
    cam = S.CORNELL_CAMERA
    pfm = str(tmp_path / "out.pfm")
    r = subprocess.run([DEMO, p, pfm, "64", "36", "64", "4", *map(str, cam["eye"]), *map(str, cam["target"]),
                        str(cam["vfov_deg"])], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    assert "host memory still allocated: 0 bytes" in r.stdout
    img = read_pfm(pfm)
    with fg.Context(0) as ctx:
        s = ctx.upload(cs.verts, cs.idx)
        s.set_materials(cs.tri_material, S.material_records(cs))
        s.set_lights(S.light_records(cs))
        ref = ctx.render(s, 64, 36, 4096, cam, seed=5)
        s.close()
    assert img.shape == (36, 64, 3)
    rel = np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2))
    assert rel < 0.05 and abs(img.mean() / ref.mean() - 1) < 0.03


@pytest.mark.gpu
def test_cpp_pass_png_output(built, tmp_path):
    """The pass's display readback (PathTracerPass::ReadbackRGBA8 ->
    fnd_rt_tonemap) written as PNG equals the display encoding of its own
    PFM frame, computed by the oracle (one code of slack for powf)."""
    import oracle as O
    from foundation_gb300 import image
    cs = S.cornell_scene(num_spheres=10, level=1)
    p = str(tmp_path / "cornell.obj")
    S.write_obj(cs, p)
    cam = S.CORNELL_CAMERA
    args = ["48", "27", "16", "2", *map(str, cam["eye"]), *map(str, cam["target"]), str(cam["vfov_deg"])]
    for out in ("out.pfm", "out.png"):
        r = subprocess.run([DEMO, p, str(tmp_path / out), *args], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr + r.stdout
    png = image.read_png(str(tmp_path / "out.png"))
    want = O.tonemap_rgba8(image.read_pfm(str(tmp_path / "out.pfm")), 1.0, 2)
    assert png.shape == (27, 48, 4)
    assert np.abs(png.astype(int) - want.astype(int)).max() <= 1
