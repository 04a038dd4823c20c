"""Headless image output on the CPU: the C++ PNG encoder of the pass
(renderer/ImageIO.cpp, driven through fnd_pass_demo --write-test-png), the
Python PNG / PFM helpers, and the display-encoding oracle's known values."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from foundation_gb300 import image

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DEMO = os.path.join(ROOT, "foundation_gb300", "lib", "fnd_pass_demo")


def test_cpp_png_encoder(built, tmp_path):
    p = str(tmp_path / "g.png")
    subprocess.run([DEMO, "--write-test-png", p], check=True, timeout=60)
    img = image.read_png(p)
    y, x = np.mgrid[0:23, 0:37]
    want = np.stack([(7 * x) & 255, (11 * y) & 255, x ^ y, 255 - x - y], -1).astype(np.uint8)
    assert img.shape == (23, 37, 4) and np.array_equal(img, want)


def test_python_png_and_pfm_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    a = rng.integers(0, 256, (19, 41, 4), dtype=np.uint8)
    image.write_png(str(tmp_path / "a.png"), a)
    assert np.array_equal(image.read_png(str(tmp_path / "a.png")), a)
    f = rng.standard_normal((7, 5, 3)).astype(np.float32)
    image.write_pfm(str(tmp_path / "a.pfm"), f)
    assert np.array_equal(image.read_pfm(str(tmp_path / "a.pfm")), f)


def test_tonemap_oracle_known_values():
    rgb = np.array([[[0.0, -1.0, np.nan], [1.0, 2.0, 0.0031308], [1e-3, 0.5, 1e9]]], np.float32)
    c = O.tonemap_rgba8(rgb, 1.0, 0)  # clamp curve
    assert c.shape == (1, 3, 4) and (c[..., 3] == 255).all()
    assert list(c[0, 0, :3]) == [0, 0, 0]
    assert list(c[0, 1, :3]) == [255, 255, 10]  # 12.92 * 0.0031308 * 255 = 10.3
    assert c[0, 2, 0] == round(12.92 * 1e-3 * 255) and c[0, 2, 2] == 255
    assert abs(int(c[0, 2, 1]) - 188) <= 1  # sRGB(0.5) = 0.7354
    r = O.tonemap_rgba8(np.full((1, 1, 3), 1.0, np.float32), 1.0, 1)  # Reinhard: 0.5
    assert abs(int(r[0, 0, 0]) - 188) <= 1
    a = O.tonemap_rgba8(np.full((1, 1, 3), 1e6, np.float32), 1.0, 2)  # ACES saturates
    assert a[0, 0, 0] == 255
