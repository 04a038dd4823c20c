"""The device PCG32 (foundation_gb300/csrc/pt/pt_math.cuh) run on the GPU
through tests/native/pcg_check.cu and compared word for word with the
oracle's generator (oracle/oracle_common.hpp, itself pinned against a
big-integer restatement of O'Neill's recurrence in test_oracle.py).

Integer work is bit-exact: every 32-bit output must equal the oracle's, for
plain (seed, sequence) pairs, for the integrator's per-pixel camera-path
seeding (with the stream saved to and restored from its path record after
every draw, as between wavefront stages) and for the radiance cache's
training-path seeding. uniform() must be the top 24 bits of the same word
scaled by 2^-24."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
MASK64 = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15
TRAIN_MUL = 0x5851F42D4C957F2D
N = 96


def _lib():
    L = C.CDLL(os.path.join(HERE, "_build", "libpcg_check.so"))
    P = C.c_void_p
    L.pcg_check.argtypes = [C.c_int, P, P, P, P, C.c_uint32, C.c_uint32, P, P]
    L.pcg_check.restype = C.c_int
    return L


def _run(mode, a, b, c, d):
    m = len(a)
    a = np.ascontiguousarray(a, np.uint64)
    b = np.ascontiguousarray(b, np.uint64)
    c = np.ascontiguousarray(c, np.uint32)
    d = np.ascontiguousarray(d, np.uint32)
    words = np.zeros((m, N), np.uint32)
    uni = np.zeros((m, N), np.float32)
    p = lambda x: x.ctypes.data_as(C.c_void_p)  # noqa: E731
    assert _lib().pcg_check(mode, p(a), p(b), p(c), p(d), m, N, p(words), p(uni)) == 0
    return words, uni


def _check(words, uni, streams):
    for j, (initstate, seq) in enumerate(streams):
        ref = O.pcg32(initstate & MASK64, seq & MASK64, N)
        assert np.array_equal(words[j], ref), f"stream {j} (initstate {initstate:#x}, sequence {seq:#x})"
        # uniform(): (word >> 8) * 2^-24, exact in FP32
        assert np.array_equal(uni[j], (ref >> np.uint32(8)).astype(np.float32) * np.float32(2.0 ** -24))


def test_pcg32_plain_streams_bit_exact(built):
    pairs = [(42, 54), (0, 0), (2**63 + 5, 7), (123456789, 2**40), (MASK64, MASK64 >> 1), (1, 2**62 + 3)]
    a = [s for s, _ in pairs]
    b = [q for _, q in pairs]
    zeros = np.zeros(len(pairs), np.uint32)
    words, uni = _run(0, a, b, zeros, zeros)
    _check(words, uni, pairs)


def test_pcg32_camera_path_seeding_bit_exact(built):
    """initstate = frame_seed * 0x9E3779B97F4A7C15 + pixel, sequence = sample;
    the stream survives the path record's save / restore."""
    rng = np.random.default_rng(7)
    frame_seeds = [0, 1, 12345, 2**40 + 17] + [int(x) for x in rng.integers(0, 2**63, 4, dtype=np.uint64)]
    pixels = [0, 1, 1920 * 1080 - 1, 1037, 77, 2**31, 5, 2**32 - 1]
    samples = [0, 63, 1, 2**20, 4095, 7, 2**31 - 1, 2**32 - 1]
    words, uni = _run(1, frame_seeds, np.zeros(8, np.uint64), pixels, samples)
    streams = [((fs * GOLDEN + px) & MASK64, sm) for fs, px, sm in zip(frame_seeds, pixels, samples)]
    _check(words, uni, streams)


def test_pcg32_training_path_seeding_bit_exact(built):
    """initstate = frame_seed * 0x9E3779B97F4A7C15 + pixel + 0x5851F42D4C957F2D * (i + 1),
    sequence = 2^30 + (round_seed mod 2^30)."""
    frame_seeds = [0, 3, 2**50 + 9, 99]
    rounds = [0, 1, 2**30 + 5, 2**32 - 1]
    pixels = [0, 4242, 1920 * 1080 - 1, 17]
    paths = [0, 65535, 12, 2**32 - 1]
    words, uni = _run(2, frame_seeds, rounds, pixels, paths)
    streams = [((fs * GOLDEN + px + TRAIN_MUL * (i + 1)) & MASK64, 0x40000000 + (r & 0x3FFFFFFF))
               for fs, r, px, i in zip(frame_seeds, rounds, pixels, paths)]
    _check(words, uni, streams)
