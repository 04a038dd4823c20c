"""The operations the traversal's child-box test is built from, checked on
the GPU against their host definitions (tests/native/minmax_check.cu):
three-input max.f32 / min.f32 must drop NaN operands like nested
fmaxf / fminf (a NaN plane must not cull a child), __fmaf_rd /
__fmaf_ru must be the exact product-sum rounded down / up, and the packed
fma.rm / fma.rp .f32x2 must give, lane by lane, the scalar __fmaf_rd /
__fmaf_ru bits."""
import ctypes as C
import itertools
import os
from fractions import Fraction

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _round_dir(v: Fraction, up: bool) -> float:
    f = np.float32(float(v))
    inf = np.float32(np.inf)
    if not up:
        while Fraction(float(f)) > v:
            f = np.nextafter(f, -inf)
        while Fraction(float(np.nextafter(f, inf))) <= v:
            f = np.nextafter(f, inf)
    else:
        while Fraction(float(f)) < v:
            f = np.nextafter(f, inf)
        while Fraction(float(np.nextafter(f, -inf))) >= v:
            f = np.nextafter(f, -inf)
    return float(f)


def test_minmax3_and_directed_fma(built):
    L = C.CDLL(os.path.join(HERE, "_build", "libminmax_check.so"))
    P = C.c_void_p
    L.minmax_check.argtypes = [P, P, P, C.c_uint32, P]
    special = [np.nan, np.inf, -np.inf, 0.0, -0.0, 1.0, -1.0, 3.5, 1e30, -1e-30, 1e-40]
    trip = np.array(list(itertools.product(special, repeat=3)), np.float32)
    rng = np.random.default_rng(7)
    finite = (rng.standard_normal((4000, 3)) * np.exp2(rng.integers(-20, 20, (4000, 3)))).astype(np.float32)
    x = np.concatenate([trip, finite], 0)
    a, b, c = (np.ascontiguousarray(x[:, k]) for k in range(3))
    out = np.zeros((len(x), 4), np.float32)
    assert L.minmax_check(a.ctypes.data_as(P), b.ctypes.data_as(P), c.ctypes.data_as(P), len(x),
                          out.ctypes.data_as(P)) == 0
    with np.errstate(invalid="ignore"):
        mx = np.fmax(np.fmax(a, b), c)
        mn = np.fmin(np.fmin(a, b), c)
    same = lambda u, v: (u == v) | (np.isnan(u) & np.isnan(v))
    assert same(out[:, 0], mx).all(), x[~same(out[:, 0], mx)][:5]
    assert same(out[:, 1], mn).all(), x[~same(out[:, 1], mn)][:5]
    for i in range(len(trip), len(x)):
        v = Fraction(float(a[i])) * Fraction(float(b[i])) + Fraction(float(c[i]))
        assert out[i, 2] == _round_dir(v, False), (a[i], b[i], c[i])
        assert out[i, 3] == _round_dir(v, True), (a[i], b[i], c[i])


def test_packed_directed_fma_equals_scalar(built):
    L = C.CDLL(os.path.join(HERE, "_build", "libminmax_check.so"))
    P = C.c_void_p
    L.fma2_check.argtypes = [P, P, P, C.c_uint32, P]
    special = [np.nan, np.inf, -np.inf, 0.0, -0.0, 1.0, -1.0, 3.5, 1e30, -1e-30, 1e-40, 1024.0, 1279.0]
    trip = np.array(list(itertools.product(special, repeat=3)), np.float32)
    rng = np.random.default_rng(11)
    finite = (rng.standard_normal((20000, 3)) * np.exp2(rng.integers(-30, 30, (20000, 3)))).astype(np.float32)
    x = np.concatenate([trip, finite], 0)
    a, b, c = (np.ascontiguousarray(x[:, k]) for k in range(3))
    out = np.zeros((len(x), 8), np.float32)
    assert L.fma2_check(a.ctypes.data_as(P), b.ctypes.data_as(P), c.ctypes.data_as(P), len(x),
                        out.ctypes.data_as(P)) == 0
    bits = out.view(np.uint32)
    nan = np.isnan(out)
    for packed, scalar in ((0, 4), (1, 5), (2, 6), (3, 7)):
        same = (bits[:, packed] == bits[:, scalar]) | (nan[:, packed] & nan[:, scalar])
        assert same.all(), x[~same][:5]
    for i in range(len(trip), len(trip) + 2000):
        v = Fraction(float(b[i])) * Fraction(float(c[i])) + Fraction(float(a[i]))
        assert out[i, 1] == _round_dir(v, False) and out[i, 3] == _round_dir(v, True), (a[i], b[i], c[i])
