"""Product BVH (binned SAH -> compressed 8-wide) checked on the CPU through
the host emulation of the kernel's per-ray logic (tests/native/wide_emu.cpp
compiles the product's traverse.cuh with host intrinsics)."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O
from foundation_gb300 import scenes as S

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def emu(built):
    L = C.CDLL(os.path.join(HERE, "_build", "libwide_emu.so"))
    P = C.c_void_p
    L.emu_build.restype = P
    L.emu_build.argtypes = [P, C.c_uint32, P, C.c_uint32, C.c_uint32]
    L.emu_trace.argtypes = [P, P, C.c_uint64, P, C.c_int, P]
    L.emu_stats.argtypes = [P, P, P, P]
    L.emu_free.argtypes = [P]
    L.emu_trace_single.argtypes = [P, P, C.c_uint64, P, C.c_int]
    L.emu_build_sbvh.restype = P
    L.emu_build_sbvh.argtypes = [P, C.c_uint32, P, C.c_uint32, C.c_float]
    L.emu_num_refs.restype = C.c_uint64
    L.emu_num_refs.argtypes = [P]
    L.emu_build_sah_collapse.restype = P
    L.emu_build_sah_collapse.argtypes = [P, C.c_uint32, P, C.c_uint32, C.c_int, C.c_double]
    L.emu_build_width.restype = P
    L.emu_build_width.argtypes = [P, C.c_uint32, P, C.c_uint32, C.c_int, C.c_uint32]
    L.emu_nodes.restype = C.c_uint32
    L.emu_nodes.argtypes = [P, P]
    L.emu_binary_hash.restype = C.c_uint64
    L.emu_binary_hash.argtypes = [P, P, C.c_uint32, C.c_uint32]
    L.emu_collapse_hash.restype = C.c_uint64
    L.emu_collapse_hash.argtypes = [P, P, P, C.c_uint32, C.c_int, C.c_uint32]
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Emu:
    def __init__(self, L, verts, idx):
        self.L = L
        self.v = np.ascontiguousarray(verts, np.float32)
        self.f = np.ascontiguousarray(idx, np.uint32)
        self.h = L.emu_build(_p(self.v), len(self.v), _p(self.f), len(self.f), 0)

    def stats(self):
        st = np.zeros(6, np.uint64)
        sah, mg = C.c_double(), C.c_float()
        self.L.emu_stats(self.h, _p(st), C.byref(sah), C.byref(mg))
        return dict(nodes=int(st[0]), leaves=int(st[1]), depth=int(st[2]), wide_nodes=int(st[3]),
                    wide_depth=int(st[4]), wide_leaves=int(st[5]), sah=sah.value, margin=mg.value)

    def trace(self, rays, any_hit=False):
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.zeros(2 * len(rays), np.uint32)
        st = np.zeros(4, np.uint64)
        self.L.emu_trace(self.h, _p(rays), len(rays), _p(out), int(any_hit), _p(st))
        return out[0::2], out[1::2], st

    def __del__(self):
        self.L.emu_free(self.h)


CASES = {
    "icosphere_camera": lambda: (S.icosphere_scene(), S.camera_rays(128, 128)),
    "cornell_incoherent": lambda: (S.cornell_scene(), S.incoherent_rays(20000, (-1, 0, -1), (1, 2, 1), seed=1)),
    "cornell_camera": lambda: (S.cornell_scene(), S.camera_rays(160, 90, **S.CORNELL_CAMERA)),
    "soup": lambda: (S.soup_scene(50000), S.incoherent_rays(20000, (0, 0, 0), (1, 1, 1), seed=2)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_emulated_wide_traversal_matches_oracle(emu, case):
    sc, rays = CASES[case]()
    e = Emu(emu, sc.verts, sc.idx)
    b = O.OracleBVH(sc.verts, sc.idx)
    es, os_ = e.stats(), b.stats()
    # the product builder reproduces the oracle's tree exactly
    assert (es["nodes"], es["leaves"], es["depth"]) == (os_["nodes"], os_["leaves"], os_["depth"])
    assert es["sah"] == pytest.approx(os_["sah"], rel=1e-9)
    assert es["wide_leaves"] == os_["leaves"]
    assert es["wide_depth"] <= 32
    prim, tbits, st = e.trace(rays)
    ref = b.closest(rays)
    assert np.array_equal(prim, ref["prim"])
    assert np.array_equal(tbits, ref["t"].view(np.uint32))
    assert int(st[2]) <= 64
    prim_a, _, _ = e.trace(rays, any_hit=True)
    assert np.array_equal((prim_a != 0xFFFFFFFF).astype(np.uint8), b.any(rays))
    # the single-ray traversal of the training-path megakernel
    out = np.zeros(2 * len(rays), np.uint32)
    emu.emu_trace_single(e.h, _p(np.ascontiguousarray(rays, np.float32)), len(rays), _p(out), 0)
    assert np.array_equal(out[0::2], ref["prim"])
    assert np.array_equal(out[1::2], ref["t"].view(np.uint32))
    emu.emu_trace_single(e.h, _p(np.ascontiguousarray(rays, np.float32)), len(rays), _p(out), 1)
    assert np.array_equal((out[0::2] != 0xFFFFFFFF).astype(np.uint8), b.any(rays))


def test_emulated_edge_cases(emu):
    # single triangle, duplicates, a degenerate (zero-area) triangle, far origins
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [2, 2, 2]], np.float32)
    f = np.array([[0, 1, 2], [0, 1, 2], [3, 3, 3], [0, 2, 1]], np.uint32)
    rays = np.array([
        [0.2, 0.2, 1, 0, 0, 0, -1, np.inf],
        [0.2, 0.2, -1, 0, 0, 0, 1, np.inf],
        [0.2, 0.2, 1, 0, 0, 0, -1, 0.5],
        [0.5, 0.0, 1, 0, 0, 0, -1, np.inf],      # on an edge
        [0.2, 0.2, 1, 0, 0, 0, 1, np.inf],       # pointing away
        [50.2, 0.2, 1, 0, -1, 0, -0.02, np.inf],  # far origin, grazing direction
        [0.2, 0.2, 0, 0, 0, 0, 0, np.inf],       # zero direction
    ], np.float32)
    e = Emu(emu, v, f)
    prim, tbits, _ = e.trace(rays)
    ref = O.brute_closest(v, f, rays)
    assert np.array_equal(prim, ref["prim"])
    assert np.array_equal(tbits, ref["t"].view(np.uint32))
    assert prim[0] == 0 and prim[1] == 0 and prim[2] == 0xFFFFFFFF


def test_emulated_axis_aligned_walls(emu):
    # flat boxes (Cornell walls) hit by rays parallel to an axis and by rays
    # grazing the box faces
    sc = S.cornell_scene(num_spheres=0)
    g = S.Pcg32Streams(5, np.arange(4000, dtype=np.uint64))
    o = np.stack([g.next_f64() * 2 - 1, g.next_f64() * 2, g.next_f64() * 2 - 1], 1)
    d = np.zeros((4000, 3))
    axis = (g.next_u32() % 3).astype(int)
    sign = np.where(g.next_u32() & 1, 1.0, -1.0)
    d[np.arange(4000), axis] = sign
    rays = np.zeros((4000, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 4:7] = d
    rays[:, 7] = np.inf
    e = Emu(emu, sc.verts, sc.idx)
    prim, tbits, _ = e.trace(rays)
    ref = O.brute_closest(sc.verts, sc.idx, rays)
    assert np.array_equal(prim, ref["prim"])
    assert np.array_equal(tbits, ref["t"].view(np.uint32))


@pytest.mark.parametrize("budget", [2.0, 8.0])
@pytest.mark.parametrize("case", ["soup", "cornell_incoherent"])
def test_emulated_spatial_split_bvh_matches_oracle(emu, case, budget):
    """Binned SAH with spatial splits: leaves hold clipped references, some
    of them to the same triangle; closest and any hits equal the oracle's
    (which uses no splits), and the reference count stays within the split
    budget (extra references per triangle)."""
    sc, rays = CASES[case]()
    v = np.ascontiguousarray(sc.verts, np.float32)
    f = np.ascontiguousarray(sc.idx, np.uint32)
    e = Emu.__new__(Emu)
    e.L, e.v, e.f = emu, v, f
    e.h = emu.emu_build_sbvh(_p(v), len(v), _p(f), len(f), budget)
    refs = emu.emu_num_refs(e.h)
    assert len(f) < refs <= (1.0 + budget) * len(f) + 64
    b = O.OracleBVH(sc.verts, sc.idx)
    st = e.stats()
    assert st["wide_depth"] <= 32
    prim, tbits, _ = e.trace(rays)
    ref = b.closest(rays)
    assert np.array_equal(prim, ref["prim"])
    assert np.array_equal(tbits, ref["t"].view(np.uint32))
    prim_a, _, _ = e.trace(rays, any_hit=True)
    assert np.array_equal((prim_a != 0xFFFFFFFF).astype(np.uint8), b.any(rays))


@pytest.mark.parametrize("spatial", [0, 1])
@pytest.mark.parametrize("case", ["soup", "cornell_incoherent"])
def test_emulated_sah_collapse_matches_oracle(emu, case, spatial):
    """The SAH-optimal collapse (fuller wide nodes, small subtrees merged into
    leaf slots of up to 4 triangles) gives the oracle's hits, with fewer wide
    nodes than the greedy collapse."""
    sc, rays = CASES[case]()
    v = np.ascontiguousarray(sc.verts, np.float32)
    f = np.ascontiguousarray(sc.idx, np.uint32)
    e = Emu.__new__(Emu)
    e.L, e.v, e.f = emu, v, f
    e.h = emu.emu_build_sah_collapse(_p(v), len(v), _p(f), len(f), spatial, 0.3)
    st = e.stats()
    assert st["wide_depth"] <= 32
    greedy = Emu(emu, sc.verts, sc.idx).stats() if not spatial else None
    if greedy:
        assert st["wide_nodes"] < greedy["wide_nodes"]
    b = O.OracleBVH(sc.verts, sc.idx)
    prim, tbits, _ = e.trace(rays)
    ref = b.closest(rays)
    assert np.array_equal(prim, ref["prim"])
    assert np.array_equal(tbits, ref["t"].view(np.uint32))
    prim_a, _, _ = e.trace(rays, any_hit=True)
    assert np.array_equal((prim_a != 0xFFFFFFFF).astype(np.uint8), b.any(rays))


def test_emulated_sah_collapse_small_and_degenerate(emu):
    """The SAH-optimal collapse on trees of 1 to 33 triangles (a root that is
    one leaf, leaves merged into the root), duplicates, a zero-area triangle
    and coincident centroids: the oracle's hits."""
    rng = np.random.default_rng(7)
    cases = []
    for n in (1, 2, 3, 4, 5, 9, 17, 33):
        v = rng.uniform(-1, 1, (3 * n, 3)).astype(np.float32)
        cases.append((v, np.arange(3 * n, dtype=np.uint32).reshape(n, 3)))
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, 0.5, 0], [0.5, 0.5, 0], [0.5, 0.5, 0]], np.float32)
    cases.append((v, np.array([[0, 1, 2]] * 40 + [[3, 4, 5]] * 3, np.uint32)))
    for v, f in cases:
        rays = np.concatenate([S.incoherent_rays(2048, (-1, -1, -1), (1, 1, 1), seed=len(f)),
                               S.camera_rays(32, 32, eye=(0.3, 0.3, 2.0), target=(0.3, 0.3, 0.0))])
        for spatial in (0, 1):
            e = Emu.__new__(Emu)
            e.L, e.v, e.f = emu, v, f
            e.h = emu.emu_build_sah_collapse(_p(v), len(v), _p(f), len(f), spatial, 0.3)
            prim, tbits, _ = e.trace(rays)
            ref = O.brute_closest(v, f, rays)
            assert np.array_equal(prim, ref["prim"]), (len(f), spatial)
            assert np.array_equal(tbits, ref["t"].view(np.uint32))


@pytest.mark.parametrize("scene", ["soup", "cornell"])
def test_collapse_independent_of_threads(emu, scene):
    """The wide tree's bytes (nodes and triangle planes) are the same on 1, 2,
    3 and 8 collapse threads, for both collapse rules and both builders: the
    collapse lays the nodes out a level at a time, in the breadth-first order
    of a one-by-one queue, and solves the SAH-optimal costs of independent
    subtrees in parallel."""
    sc = S.soup_scene(60000) if scene == "soup" else S.cornell_scene(num_spheres=40)
    v = np.ascontiguousarray(sc.verts, np.float32)
    f = np.ascontiguousarray(sc.idx, np.uint32)
    for spatial in (0, 1):
        h = emu.emu_build_sah_collapse(_p(v), len(v), _p(f), len(f), spatial, 0.3)
        try:
            for sah in (0, 1):
                hashes = {emu.emu_collapse_hash(h, _p(v), _p(f), len(f), sah, t) for t in (1, 2, 3, 8)}
                assert len(hashes) == 1, (scene, spatial, sah)
        finally:
            emu.emu_free(h)


@pytest.mark.parametrize("sah", [0, 1])
def test_emulated_node_width(emu, sah):
    """Nodes of at most 2, 4 and 6 children (the autotuner's node-width
    dimension; the record keeps its 8 slots): no node uses more slots than
    the width, narrower trees have more nodes, and the hits are the oracle's,
    on Cornell rays and on the small and degenerate trees."""
    sc, rays = CASES["cornell_incoherent"]()
    v = np.ascontiguousarray(sc.verts, np.float32)
    f = np.ascontiguousarray(sc.idx, np.uint32)
    ref = O.OracleBVH(sc.verts, sc.idx).closest(rays)
    counts = {}
    for width in (2, 4, 6, 8):
        e = Emu.__new__(Emu)
        e.L, e.v, e.f = emu, v, f
        e.h = emu.emu_build_width(_p(v), len(v), _p(f), len(f), sah, width)
        n = emu.emu_nodes(e.h, None)
        raw = np.zeros((n, 80), np.uint8)
        emu.emu_nodes(e.h, _p(raw))
        used = (raw[:, 24:32] != 0).sum(1)
        assert used.max() <= width and used.min() >= 1
        counts[width] = n
        prim, tbits, _ = e.trace(rays)
        assert np.array_equal(prim, ref["prim"]), width
        assert np.array_equal(tbits, ref["t"].view(np.uint32))
    assert counts[2] > counts[4] > counts[6] > counts[8]
    rng = np.random.default_rng(11)
    for n in (1, 2, 3, 5, 9, 33):
        vv = rng.uniform(-1, 1, (3 * n, 3)).astype(np.float32)
        ff = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
        rr = S.incoherent_rays(2048, (-1, -1, -1), (1, 1, 1), seed=n)
        want = O.brute_closest(vv, ff, rr)
        for width in (2, 3):
            e = Emu.__new__(Emu)
            e.L, e.v, e.f = emu, vv, ff
            e.h = emu.emu_build_width(_p(vv), len(vv), _p(ff), len(ff), sah, width)
            prim, tbits, _ = e.trace(rr)
            assert np.array_equal(prim, want["prim"]), (n, width)
            assert np.array_equal(tbits, want["t"].view(np.uint32))


@pytest.mark.parametrize("scene", ["soup", "identical"])
def test_binary_build_independent_of_threads(emu, scene):
    """The binned-SAH tree (boxes, counts, leaf triangles in depth-first
    order) is the same on 1, 2, 3 and 8 build threads: large nodes are split
    with every thread (bins merged, stable partition through per-chunk
    offsets), the rest one node per thread. The identical-triangles case
    takes the index-median split in both phases."""
    if scene == "soup":
        sc = S.soup_scene(300000, seed=6)
        v, f = np.ascontiguousarray(sc.verts, np.float32), np.ascontiguousarray(sc.idx, np.uint32)
    else:
        v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
        f = np.zeros((150000, 3), np.uint32) + np.arange(3, dtype=np.uint32)
    hashes = {emu.emu_binary_hash(_p(v), _p(f), len(f), t) for t in (1, 2, 3, 8)}
    assert len(hashes) == 1
