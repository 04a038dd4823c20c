"""The device status word: the traversal's own checks turn a corrupt tree
into a latched status bit and an fnd_status code, never an out-of-range
access or a fault.

Scenes are written node by node here (80-byte wide nodes, foundation_gb300/
csrc/bvh/wide_bvh.hpp) and cover:
  * a child index past the node array           -> kStatusBadIndex (4)
  * a leaf whose triangle range passes the end   -> kStatusBadIndex (4)
  * a chain of 80 nested nodes, each leaving one
    sibling on the stack (deeper than its 64 entries) -> kStatusStackOverflow (1)
  * a chain of 40 (within the stack) ending in a triangle: no status, the hit
The chain's siblings are empty nodes, so every scene is traversed in a
number of steps linear in its size whatever the checks do.

CPU: the product's RT::trace_single compiled on the host
(tests/native/wide_emu.cpp), and the status-to-code mapping every entry
point uses (RT::StatusCode). GPU: the same per-thread traversal and the
persistent closest- and any-hit kernels (tests/native/status_check.cu).
Counterpart in the reference: CHECK -> BugCheck (src/Core/Core.hpp:17,
src/Core/Core.cpp:7-10), which terminates; here the failure is reported.
"""
import ctypes as C
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

BAD_INDEX = 4
STACK_OVERFLOW = 1
TIMEOUT = 2
FND_OK, FND_ERR_CUDA, FND_ERR_INVALID_SCENE, FND_ERR_STACK_OVERFLOW, FND_ERR_TIMEOUT = 0, -3, -5, -6, -7

NODE = np.dtype([("p", "<f4", 3), ("e", "u1", 3), ("imask", "u1"), ("child_base", "<u4"), ("tri_base", "<u4"),
                 ("meta", "u1", 8), ("qlo", "u1", (3, 8)), ("qhi", "u1", (3, 8))])
assert NODE.itemsize == 80
TRI_ID = 7


def _node(imask=0, child_base=0, tri_base=0, leaf_slot0=0):
    """Every used slot's box is [-1, -1 + 255 / 64] on each axis; slots set in
    imask are internal; leaf_slot0 = k puts a leaf of k triangles in slot 0."""
    n = np.zeros(1, NODE)
    n["p"] = -1.0
    n["e"] = 127 - 6
    n["imask"] = imask
    n["child_base"] = child_base
    n["tri_base"] = tri_base
    meta = np.zeros(8, np.uint8)
    used = imask
    for s in range(8):
        if imask >> s & 1:
            meta[s] = 0x01
    if leaf_slot0:
        meta[0] = 0x80 | (leaf_slot0 - 1) << 5
        used |= 1
    n["meta"] = meta
    q = np.zeros((3, 8), np.uint8)
    q[:, [s for s in range(8) if used >> s & 1]] = 255
    n["qhi"] = q
    return n


def _chain(depth, tail_tris=0):
    """C_k at 2k with internal children C_{k+1} (slot 0) and the empty T_{k+1}
    (slot 1) at 2k + 2, 2k + 3; the last C holds a leaf of tail_tris."""
    nodes = []
    for k in range(depth):
        if k < depth - 1:
            nodes.append(_node(imask=0b11, child_base=2 * k + 2))
        else:
            nodes.append(_node(leaf_slot0=tail_tris))
        nodes.append(_node())  # T_k (T_0 is never referenced)
    return np.concatenate(nodes)


def _planes(ntri):
    """ntri copies of the triangle (3,0,0), (0,3,0), (0,0,3), id TRI_ID."""
    v = np.zeros((3, max(ntri, 1), 4), np.float32)
    v[0, :, 0] = 3.0
    v[1, :, 1] = 3.0
    v[2, :, 2] = 3.0
    v[0, :, 3] = np.array([TRI_ID], np.uint32).view(np.float32)[0]
    return v[:, :ntri].copy()


def _rays(n=64):
    """Origins inside the boxes, directions in the positive octant (slot 0 is
    visited first, slot 1 waits on the stack)."""
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = [0.1, 0.2, 0.3]
    r[:, 3] = 0.0
    r[:, 4:7] = [1.0, 1.1, 1.2]
    r[:, 4] += np.linspace(0, 0.05, n, dtype=np.float32)
    r[:, 7] = np.inf
    return r


CASES = {
    # name: (nodes, planes, status, hit expected)
    "bad_child": (lambda: _node(imask=0b1, child_base=5), lambda: _planes(0), BAD_INDEX, False),
    "bad_triangle_range": (lambda: _node(leaf_slot0=4), lambda: _planes(2), BAD_INDEX, False),
    "stack_overflow": (lambda: _chain(80), lambda: _planes(0), STACK_OVERFLOW, False),
    "deep_but_fits": (lambda: _chain(40, tail_tris=1), lambda: _planes(1), 0, True),
}
CODES = {BAD_INDEX: FND_ERR_INVALID_SCENE, STACK_OVERFLOW: FND_ERR_STACK_OVERFLOW, 0: FND_OK}


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.fixture(scope="module")
def emu(built):
    L = C.CDLL(os.path.join(HERE, "_build", "libwide_emu.so"))
    P = C.c_void_p
    L.emu_trace_single_raw.argtypes = [P, C.c_uint32, P, C.c_uint32, P, C.c_uint64, P, P]
    L.emu_status_code.argtypes = [C.c_uint32]
    L.emu_status_code.restype = C.c_int
    return L


def _expect_hits(hits, hit):
    if hit:
        assert (hits[:, 0] == TRI_ID).all()
        t = hits[:, 1].view(np.float32)
        # (0.1 + 0.2 + 0.3) + t (1 + dx + 1.1 + 1.2) = 3 on the triangle's plane
        assert np.allclose(t[0], 2.4 / 3.3, rtol=1e-6)
    else:
        assert (hits[:, 0] == 0xFFFFFFFF).all()


@pytest.mark.parametrize("case", sorted(CASES))
def test_status_word_emulated(emu, case):
    mk_nodes, mk_planes, status, hit = CASES[case]
    nodes, planes, rays = mk_nodes(), mk_planes(), _rays()
    hits = np.zeros((len(rays), 2), np.uint32)
    st = np.zeros(1, np.uint32)
    emu.emu_trace_single_raw(_p(nodes), len(nodes), _p(planes), planes.shape[1], _p(rays), len(rays), _p(hits),
                             _p(st))
    assert int(st[0]) == status
    _expect_hits(hits, hit)
    assert emu.emu_status_code(int(st[0])) == CODES[status]


def test_status_code_mapping(emu):
    """Overflow outranks a timeout, which outranks a bad index; unknown bits
    are reported as a CUDA failure."""
    assert emu.emu_status_code(0) == FND_OK
    assert emu.emu_status_code(BAD_INDEX) == FND_ERR_INVALID_SCENE
    assert emu.emu_status_code(STACK_OVERFLOW) == FND_ERR_STACK_OVERFLOW
    assert emu.emu_status_code(TIMEOUT) == FND_ERR_TIMEOUT
    assert emu.emu_status_code(BAD_INDEX | STACK_OVERFLOW) == FND_ERR_STACK_OVERFLOW
    assert emu.emu_status_code(BAD_INDEX | TIMEOUT) == FND_ERR_TIMEOUT
    assert emu.emu_status_code(8) == FND_ERR_CUDA


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1, 2], ids=["per_thread", "persistent_closest", "persistent_any"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_status_word_on_gpu(built, emu, case, mode):
    L = C.CDLL(os.path.join(HERE, "_build", "libstatus_check.so"))
    P = C.c_void_p
    L.status_trace.argtypes = [C.c_int, P, C.c_uint32, P, C.c_uint32, P, C.c_uint32, P, P]
    L.status_trace.restype = C.c_int
    mk_nodes, mk_planes, status, hit = CASES[case]
    nodes, planes, rays = mk_nodes(), mk_planes(), _rays(256)
    hits = np.zeros((len(rays), 2), np.uint32)
    st = np.zeros(1, np.uint32)
    assert L.status_trace(mode, _p(nodes), len(nodes), _p(planes), planes.shape[1], _p(rays), len(rays), _p(hits),
                          _p(st)) == 0
    assert int(st[0]) == status
    if mode == 2:
        assert (hits[:, 0] == (1 if hit else 0)).all()
        return
    _expect_hits(hits, hit)
    # same hits, t bit for bit, as the host compilation of the same code
    ref = np.zeros_like(hits)
    st_ref = np.zeros(1, np.uint32)
    emu.emu_trace_single_raw(_p(nodes), len(nodes), _p(planes), planes.shape[1], _p(rays), len(rays), _p(ref),
                             _p(st_ref))
    assert np.array_equal(hits, ref)
