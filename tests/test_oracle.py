"""CPU oracle: hand-derived known-answer tests, PCG32 cross-checks, BVH
invariants, brute-force agreement and the committed golden fixtures."""
import hashlib
import os

import numpy as np
import pytest

import oracle as O
from foundation_gb300 import scenes as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TRI = [0, 0, 0, 1, 0, 0, 0, 1, 0]  # unit right triangle in z = 0


def ray(o, d, tmin=0.0, tmax=np.inf):
    return [*o, tmin, *d, tmax]


# ---- watertight intersection, answers derived by hand -------------------

def test_kat_interior_hit_exact_t():
    h, t, _ = O.intersect1(ray((0.25, 0.25, 1.0), (0, 0, -1)), TRI)
    assert h and t == 1.0


def test_kat_barycentrics():
    # point (0.25, 0.5): weights of v1, v2 are 0.25 and 0.5, of v0 0.25
    h, t, uvwd = O.intersect1(ray((0.25, 0.5, 2.0), (0, 0, -1)), TRI)
    U, V, W, det = uvwd
    assert h and t == 2.0
    w = np.array([U, V, W]) / det
    assert sorted(np.round(w, 6).tolist()) == [0.25, 0.25, 0.5]


def test_kat_outside_miss():
    assert not O.intersect1(ray((0.75, 0.75, 1.0), (0, 0, -1)), TRI)[0]
    assert not O.intersect1(ray((-0.01, 0.5, 1.0), (0, 0, -1)), TRI)[0]


@pytest.mark.parametrize("xy", [(0.5, 0.0), (0.0, 0.5), (0.5, 0.5), (0.0, 0.0), (1.0, 0.0), (0.0, 1.0)])
def test_kat_edges_and_vertices_hit(xy):
    h, t, _ = O.intersect1(ray((xy[0], xy[1], 1.0), (0, 0, -1)), TRI)
    assert h and t == 1.0


def test_kat_parallel_in_plane_misses():
    assert not O.intersect1(ray((-1.0, 0.25, 0.0), (1, 0, 0)), TRI)[0]


def test_kat_backface_hit_non_culling():
    h, t, _ = O.intersect1(ray((0.25, 0.25, -3.0), (0, 0, 1)), TRI)
    assert h and t == 3.0


def test_kat_interval_clipping_inclusive():
    assert not O.intersect1(ray((0.25, 0.25, 1.0), (0, 0, -1), tmax=0.5), TRI)[0]
    assert not O.intersect1(ray((0.25, 0.25, 1.0), (0, 0, -1), tmin=1.5), TRI)[0]
    assert O.intersect1(ray((0.25, 0.25, 1.0), (0, 0, -1), tmax=1.0), TRI)[0]
    assert O.intersect1(ray((0.25, 0.25, 1.0), (0, 0, -1), tmin=1.0), TRI)[0]


def test_kat_unnormalised_direction_scales_t():
    h, t, _ = O.intersect1(ray((0.25, 0.25, 1.0), (0, 0, -4)), TRI)
    assert h and t == 0.25


def test_kat_degenerate_and_nan_triangles_miss():
    assert not O.intersect1(ray((0.0, 0.0, 1.0), (0, 0, -1)), [0, 0, 0, 1, 1, 0, 2, 2, 0])[0]
    assert not O.intersect1(ray((0.2, 0.2, 1.0), (0, 0, -1)), [np.nan, 0, 0, 1, 0, 0, 0, 1, 0])[0]


def test_tie_breaks_to_lowest_id():
    # triangles 0..2 are the same triangle; 3 is coplanar and overlapping
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [-1, -1, 0], [2, -1, 0], [-1, 2, 0]], np.float32)
    f = np.array([[3, 4, 5], [0, 1, 2], [0, 2, 1], [1, 2, 0]], np.uint32)
    r = np.array([ray((0.2, 0.2, 1.0), (0, 0, -1)), ray((1.5, -0.5, 1.0), (0, 0, -1))], np.float32)
    hb = O.brute_closest(v, f, r)
    assert hb["prim"].tolist() == [0, 0] and hb["t"].tolist() == [1.0, 1.0]
    f2 = f[[1, 2, 3, 0]]  # the big triangle now has id 3
    hb2 = O.brute_closest(v, f2, r)
    assert hb2["prim"].tolist() == [0, 3]
    b = O.OracleBVH(v, f2)
    assert b.closest(r)["prim"].tolist() == [0, 3]


def test_watertight_closed_mesh_from_inside():
    # every ray from the centre of a closed icosphere hits it, including rays
    # aimed exactly at its vertices and edge midpoints
    v, f = S.icosphere(2)
    v = v.astype(np.float32)
    dirs = np.concatenate([v, (v[f[:, 0]] + v[f[:, 1]]) * 0.5, (v[f[:, 1]] + v[f[:, 2]]) * 0.5], 0)
    rays = np.zeros((len(dirs), 8), np.float32)
    rays[:, 4:7] = dirs
    rays[:, 7] = np.inf
    hb = O.brute_closest(v, f, rays)
    assert (hb["prim"] != 0xFFFFFFFF).all()


# ---- PCG32 -------------------------------------------------------------

def _pcg32_bigint(seed, seq, n):
    """The published PCG-XSH-RR 64/32 recurrence in Python integers."""
    M = 6364136223846793005
    mask = (1 << 64) - 1
    inc = ((seq << 1) | 1) & mask
    state = 0
    out = []

    def step(s):
        return (s * M + inc) & mask

    state = step(state)
    state = (state + seed) & mask
    state = step(state)
    for _ in range(n):
        old = state
        state = step(old)
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        out.append(((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF)
    return out


@pytest.mark.parametrize("seed,seq", [(42, 54), (0, 0), (2**63 + 5, 7), (123456789, 2**40)])
def test_pcg32_matches_bigint_recurrence(seed, seq):
    assert O.pcg32(seed, seq, 64).tolist() == _pcg32_bigint(seed, seq, 64)


def test_pcg32_numpy_streams_match():
    g = S.Pcg32Streams(42, np.array([54, 0, 9], np.uint64))
    got = np.stack([g.next_u32() for _ in range(16)], 1)
    for j, seq in enumerate([54, 0, 9]):
        assert got[j].tolist() == O.pcg32(42, seq, 16).tolist()


# ---- BVH -----------------------------------------------------------------

@pytest.mark.parametrize("name", ["ico", "soup", "cornell_small"])
def test_bvh_invariants(name):
    sc = {"ico": S.icosphere_scene, "soup": lambda: S.soup_scene(20000),
          "cornell_small": lambda: S.cornell_scene(num_spheres=10, level=2)}[name]()
    b = O.OracleBVH(sc.verts, sc.idx)
    assert b.validate() == 0
    st = b.stats()
    assert st["max_leaf"] <= 4 and st["leaves"] * 2 - 1 == st["nodes"]


def test_bvh_equals_brute_force_on_random_rays():
    sc = S.soup_scene(3000, seed=11)
    rays = S.incoherent_rays(3000, (-0.2, -0.2, -0.2), (1.2, 1.2, 1.2), seed=3)
    b = O.OracleBVH(sc.verts, sc.idx)
    h = b.closest(rays)
    hb = O.brute_closest(sc.verts, sc.idx, rays)
    assert np.array_equal(h["prim"], hb["prim"])
    assert np.array_equal(h["t"].view(np.uint32), hb["t"].view(np.uint32))
    assert np.array_equal(b.any(rays), O.brute_any(sc.verts, sc.idx, rays))


def test_bvh_degenerate_inputs():
    # all triangles identical (coincident centroids -> median splits)
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    f = np.zeros((37, 3), np.uint32)
    f[:] = [0, 1, 2]
    b = O.OracleBVH(v, f)
    assert b.validate() == 0
    r = np.array([ray((0.2, 0.2, 1.0), (0, 0, -1))], np.float32)
    assert b.closest(r)["prim"][0] == 0


# ---- golden fixtures --------------------------------------------------------

def _sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_golden_soup():
    g = np.load(os.path.join(GOLDEN, "soup1k.npz"))
    b = O.OracleBVH(g["verts"], g["idx"])
    h = b.closest(g["rays"])
    assert np.array_equal(h["prim"], g["prim"])
    assert np.array_equal(h["t"].view(np.uint32), g["t"].view(np.uint32))
    assert np.array_equal(b.any(g["rays"]), g["occluded"])


def test_golden_generators_are_pinned():
    g = np.load(os.path.join(GOLDEN, "icosphere_rows.npz"))
    ico = S.icosphere_scene()
    assert _sha(ico.verts, ico.idx) == str(g["scene_sha256"])
    assert _sha(S.camera_rays(1024, 1024)) == str(g["rays_sha256"])
    gc = np.load(os.path.join(GOLDEN, "cornell_rows.npz"))
    cs = S.cornell_scene()
    assert _sha(cs.verts, cs.idx, cs.tri_material, cs.materials) == str(gc["scene_sha256"])
    assert cs.num_tris == 256012 and ico.num_tris == 82944


def test_golden_icosphere_rows():
    g = np.load(os.path.join(GOLDEN, "icosphere_rows.npz"))
    ico = S.icosphere_scene()
    h = O.OracleBVH(ico.verts, ico.idx).closest(g["rays"])
    assert np.array_equal(h["prim"], g["prim"])
    assert np.array_equal(h["t"].view(np.uint32), g["t"].view(np.uint32))
