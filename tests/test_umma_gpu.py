"""The fifth-generation tensor-core primitives the radiance cache trains with
(foundation_gb300/csrc/nrc/umma.cuh: tensor-memory allocation, shared-memory
descriptors of the row-group-major operand layout, tcgen05.mma kind::f16,
commit, tensor-memory loads), run on the GPU by tests/native/umma_check.cu.

Inputs are small integers in BF16, so every product and sum is exact in FP32
and the device result must equal the host's bit for bit: a wrong descriptor
stride, operand major-ness or tensor-memory lane mapping shows up as a
mismatch, not as a rounding difference."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _bf16_bits(x):
    """float32 values exactly representable in BF16 -> their 16-bit patterns"""
    return (np.ascontiguousarray(x, np.float32).view(np.uint32) >> 16).astype(np.uint16)


def _run(mode, a, b, k_or_f, n):
    L = C.CDLL(os.path.join(HERE, "_build", "libumma_check.so"))
    P = C.c_void_p
    L.umma_check.argtypes = [C.c_int, P, P, C.c_uint32, C.c_uint32, P]
    L.umma_check.restype = C.c_int
    ab, bb = _bf16_bits(a), _bf16_bits(b)
    d = np.zeros((128, n), np.float32)
    p = lambda x: x.ctypes.data_as(P)  # noqa: E731
    rc = L.umma_check(mode, p(ab), p(bb), k_or_f, n, p(d))
    assert rc == 0, f"umma_check returned {rc}"
    return d


@pytest.mark.parametrize("k,n", [(96, 64), (64, 64), (64, 16), (16, 16), (128, 32)])
def test_kmajor_product_exact(built, k, n):
    rng = np.random.default_rng(k * 100 + n)
    a = rng.integers(-4, 5, (128, k)).astype(np.float32)
    b = rng.integers(-4, 5, (n, k)).astype(np.float32)
    d = _run(0, a, b, k, n)
    assert np.array_equal(d, (a.astype(np.float64) @ b.T.astype(np.float64)).astype(np.float32))


@pytest.mark.parametrize("f,n", [(64, 64), (96, 64), (64, 16), (16, 16)])
def test_mnmajor_weight_gradient_exact(built, f, n):
    rng = np.random.default_rng(f * 100 + n + 7)
    h = rng.integers(-3, 4, (128, f)).astype(np.float32)
    g = rng.integers(-3, 4, (128, n)).astype(np.float32)
    d = _run(1, h, g, f, n)
    want = (h.T.astype(np.float64) @ g.astype(np.float64)).astype(np.float32)
    assert np.array_equal(d[:f], want)
