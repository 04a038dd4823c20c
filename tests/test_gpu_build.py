"""BVH built on the GPU (FND_BVH_GPU_BUILD: linear BVH or, with
FND_BVH_GPU_CLUSTER, locally-ordered clustering, then SAH leaf merging and the
device collapse to the 8-wide format): every hit equals the CPU oracle's
(ids exact, t bit-identical), for tiny, degenerate and large scenes; bad
input fails cleanly; a path-traced image equals the host-built scene's."""
import os

import numpy as np
import pytest

import oracle as O
from foundation_gb300 import scenes as S

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx(built):
    import foundation_gb300 as fg
    c = fg.Context(0)
    yield c
    c.close()


def assert_same(h, ref):
    bad = np.nonzero(h["prim"] != ref["prim"])[0]
    assert len(bad) == 0, f"{len(bad)} id mismatches, first {bad[:5]}"
    assert np.array_equal(h["t"].view(np.uint32), ref["t"].view(np.uint32))


@pytest.mark.parametrize("case", ["ico", "cornell", "soup"])
def test_gpu_built_scene_matches_oracle(ctx, case):
    if case == "ico":
        sc, rays = S.icosphere_scene(), S.camera_rays(512, 512)
    elif case == "cornell":
        sc = S.cornell_scene()
        rays = np.concatenate([S.incoherent_rays(1 << 19, *sc.bounds, seed=1),
                               S.camera_rays(320, 180, **S.CORNELL_CAMERA)])
    else:
        sc = S.soup_scene(1 << 20)
        rays = S.incoherent_rays(1 << 18, (0, 0, 0), (1, 1, 1), seed=2)
    b = O.OracleBVH(sc.verts, sc.idx)
    ref_closest, ref_any = b.closest(rays), b.any(rays)
    lo, hi = sc.verts[sc.idx.ravel()].min(0), sc.verts[sc.idx.ravel()].max(0)
    sah = {}
    for cluster in (False, True):
        g = ctx.upload(sc.verts, sc.idx, gpu_build=True, cluster=cluster)
        info = g.info()
        sah[cluster] = info["sah_cost"]
        assert info["num_refs"] == sc.num_tris and 1 <= info["wide_depth"] <= 32
        assert info["num_wide_nodes"] >= 1 and info["num_leaves"] >= 1
        assert np.array_equal(np.array(info["bounds_lo"], np.float32), lo)
        assert np.array_equal(np.array(info["bounds_hi"], np.float32), hi)
        assert_same(g.closest(rays), ref_closest)
        assert np.array_equal(g.any(rays), ref_any)
        # the SAH-optimal collapse on the device: fuller nodes, the same hits
        gs = ctx.upload(sc.verts, sc.idx, gpu_build=True, sah_collapse=True, cluster=cluster)
        si = gs.info()
        assert 1 <= si["wide_depth"] <= 32 and si["num_refs"] == sc.num_tris
        assert si["num_wide_nodes"] < info["num_wide_nodes"]
        assert_same(gs.closest(rays), ref_closest)
        assert np.array_equal(gs.any(rays), ref_any)
        gs.close()
        g.close()
    # clustering gives the lower-cost binary tree
    assert sah[True] < sah[False], sah


@pytest.mark.parametrize("radius", [1, 2, 64])
def test_clustered_build_at_radius_limits(ctx, radius):
    """Radius 1 merges only neighbours in the array (the slowest progress),
    64 is the widest window; the tree is deterministic, hits exact."""
    sc = S.soup_scene(1 << 16)
    rays = S.incoherent_rays(1 << 16, (0, 0, 0), (1, 1, 1), seed=5)
    ref = O.OracleBVH(sc.verts, sc.idx).closest(rays)
    infos = []
    for _ in range(2):
        g = ctx.upload(sc.verts, sc.idx, gpu_build=True, sah_collapse=True, cluster=True, cluster_radius=radius)
        assert_same(g.closest(rays), ref)
        infos.append({k: v for k, v in g.info().items() if not k.endswith("_ms")})
        g.close()
    assert infos[0] == infos[1]


def test_gpu_build_tiny_and_degenerate(ctx):
    rng = np.random.default_rng(3)
    for n in (1, 2, 3, 4, 5, 9, 33):
        v = rng.uniform(-1, 1, (3 * n, 3)).astype(np.float32)
        f = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
        rays = S.incoherent_rays(4096, (-1, -1, -1), (1, 1, 1), seed=n)
        ref = O.OracleBVH(v, f).closest(rays)
        for sah in (False, True):
            for cluster in (False, True):
                g = ctx.upload(v, f, gpu_build=True, sah_collapse=sah, cluster=cluster)
                assert_same(g.closest(rays), ref)
                g.close()
    # duplicates, a degenerate (zero-area) triangle, all centroids equal
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, 0.5, 0], [0.5, 0.5, 0], [0.5, 0.5, 0]], np.float32)
    f = np.array([[0, 1, 2]] * 40 + [[3, 4, 5]] * 3, np.uint32)
    rays = S.camera_rays(64, 64, eye=(0.3, 0.3, 2.0), target=(0.3, 0.3, 0.0))
    ref = O.OracleBVH(v, f).closest(rays)
    for sah in (False, True):
        for cluster in (False, True):
            g = ctx.upload(v, f, gpu_build=True, sah_collapse=sah, cluster=cluster, cluster_radius=3 if cluster else 0)
            assert_same(g.closest(rays), ref)
            g.close()


def test_gpu_build_rejects_bad_input(ctx):
    import foundation_gb300 as fg
    v = np.zeros((3, 3), np.float32)
    with pytest.raises(fg.FndError):
        ctx.upload(v, np.array([[0, 1, 3]], np.uint32), gpu_build=True)
    v2 = v.copy()
    v2[1, 0] = np.nan
    with pytest.raises(fg.FndError):
        ctx.upload(v2, np.array([[0, 1, 2]], np.uint32), gpu_build=True)
    with pytest.raises(fg.FndError):
        ctx.upload(v, np.array([[0, 1, 2]], np.uint32), gpu_build=True, spatial_splits=True)
    with pytest.raises(fg.FndError):  # clustering on the host build
        ctx.upload(v, np.array([[0, 1, 2]], np.uint32), cluster=True)
    with pytest.raises(fg.FndError):  # radius above 64
        ctx.upload(v, np.array([[0, 1, 2]], np.uint32), gpu_build=True, cluster=True, cluster_radius=65)
    with pytest.raises(fg.FndError):  # a radius without clustering
        ctx.upload(v, np.array([[0, 1, 2]], np.uint32), gpu_build=True, cluster_radius=8)
    g = ctx.upload(v, np.zeros((0, 3), np.uint32), gpu_build=True)  # empty scene still works
    assert (g.closest(S.cube_camera_rays(10))["prim"] == fg.INVALID_ID).all()
    g.close()


def test_gpu_built_scene_renders_like_host_built(ctx):
    cs = S.cornell_scene()
    imgs, stats = [], []
    for gpu in (False, True):
        s = ctx.upload(cs.verts, cs.idx, gpu_build=gpu)
        s.set_materials(cs.tri_material, S.material_records(cs))
        s.set_lights(S.light_records(cs))
        imgs.append(ctx.render(s, 96, 54, 32, S.CORNELL_CAMERA, seed=4))
        st = ctx.render_stats()
        stats.append((st["extension_rays"], st["shadow_rays"]))
        s.close()
    assert stats[0] == stats[1]
    np.testing.assert_allclose(imgs[1], imgs[0], rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("gpu", [False, True], ids=["host_build", "gpu_build"])
def test_node_width(ctx, gpu):
    """Nodes of at most 2, 4 and 6 children (FND_BVH_NODE_WIDTH), greedy and
    SAH-optimal collapse, host and GPU builds: the oracle's hits, and more
    wide nodes the narrower they are."""
    import foundation_gb300 as fg
    sc = S.cornell_scene(num_spheres=40)
    rays = S.incoherent_rays(1 << 17, *sc.bounds, seed=4)
    ref = O.OracleBVH(sc.verts, sc.idx).closest(rays)
    for sah in (False, True):
        nodes = []
        for width in (2, 4, 6, 8):
            g = ctx.upload(sc.verts, sc.idx, gpu_build=gpu, cluster=gpu, sah_collapse=sah, node_width=width)
            assert_same(g.closest(rays), ref)
            nodes.append(g.info()["num_wide_nodes"])
            g.close()
        assert nodes == sorted(nodes, reverse=True) and nodes[0] > nodes[-1], nodes
    for bad in (1, 9):
        with pytest.raises(fg.FndError):
            ctx.upload(sc.verts[:3], sc.idx[:1] * 0 + np.arange(3, dtype=np.uint32), node_width=bad)
