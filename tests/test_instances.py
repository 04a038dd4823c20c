"""Two-level scenes (fnd_rt_instances_upload). CPU: the oracle's instanced
brute force against the same geometry flattened into world space (same ids;
t equal up to the rounding of the ray transform; bit-equal for identity
instances). GPU: device hits equal the oracle's exactly (ids and t bits),
closest and any; the bottom-level margin check; lifetime rules."""
import numpy as np
import pytest

import oracle as O
from foundation_gb300 import scenes as S


def random_instances(n, n_levels, seed=4, scale=(0.05, 0.3)):
    rng = np.random.default_rng(seed)
    out = []
    off = 0
    for i in range(n):
        q = rng.standard_normal(4)
        q /= np.linalg.norm(q)
        a, b, c, d = q
        rot = np.array([[a*a+b*b-c*c-d*d, 2*(b*c-a*d), 2*(b*d+a*c)],
                        [2*(b*c+a*d), a*a-b*b+c*c-d*d, 2*(c*d-a*b)],
                        [2*(b*d-a*c), 2*(c*d+a*b), a*a-b*b-c*c+d*d]])
        s = rng.uniform(*scale)
        m = np.zeros((3, 4), np.float32)
        m[:, :3] = rot * s
        m[:, 3] = rng.uniform(-1.6, 1.6, 3)
        lv = int(rng.integers(0, n_levels))
        out.append((lv, m, off))
        off += 10000
    return out


def levels():
    sv, sf = S.icosphere(2)
    soup = S.soup_scene(150, seed=9)
    return [(sv.astype(np.float32), sf), (soup.verts - 0.5, soup.idx)]


def test_oracle_instances_match_flattened_geometry(built):
    lv = levels()
    inst = random_instances(12, 2)
    rays = S.incoherent_rays(3000, (-2, -2, -2), (2, 2, 2), seed=5)
    verts, idx, ids = [], [], []
    base = 0
    for l, m, off in inst:
        v, f = lv[l]
        w = (np.asarray(v, np.float64) @ m[:, :3].T.astype(np.float64) + m[:, 3]).astype(np.float32)
        verts.append(w)
        idx.append(np.asarray(f, np.uint32) + base)
        ids.append(off + np.arange(len(f), dtype=np.uint32))
        base += len(w)
    flat = O.brute_closest(np.concatenate(verts), np.concatenate(idx), rays)
    ids = np.concatenate(ids)
    hi = O.instances_trace(lv, inst, rays)
    hit = flat["prim"] != 0xFFFFFFFF
    # the same triangle away from silhouettes, t to within the transform's rounding
    agree = np.mean(np.where(hit, ids[np.minimum(flat["prim"], len(ids) - 1)] == hi["prim"], hi["prim"] == 0xFFFFFFFF))
    assert agree > 0.995, agree
    both = hit & (ids[np.minimum(flat["prim"], len(ids) - 1)] == hi["prim"])
    np.testing.assert_allclose(hi["t"][both], flat["t"][both], rtol=1e-4)
    # identity instances are the flat scene, bit for bit
    eye = np.eye(3, 4, dtype=np.float32)
    v, f = lv[0]
    a = O.instances_trace([lv[0]], [(0, eye, 0)], rays)
    b = O.brute_closest(v, f, rays)
    assert np.array_equal(a["prim"], b["prim"]) and np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))
    occ = O.instances_trace(lv, inst, rays, any_hit=True)
    assert np.array_equal(occ.astype(bool), hi["prim"] != 0xFFFFFFFF)


@pytest.mark.gpu
def test_instances_match_oracle_on_gpu(built):
    import foundation_gb300 as fg
    lv = levels()
    inst = random_instances(40, 2)
    rays = np.concatenate([S.incoherent_rays(1 << 15, (-2, -2, -2), (2, 2, 2), seed=6),
                           S.camera_rays(128, 96, eye=(0, 0, 6), target=(0, 0, 0))])
    with fg.Context(0) as ctx:
        small = [ctx.upload(v, f) for v, f in lv]
        with pytest.raises(fg.FndError, match="margin_scale"):
            ctx.instances([(small[l], m, off) for l, m, off in inst])
        blas = [ctx.upload(v, f, margin_scale=64) for v, f in lv]
        sc = ctx.instances([(blas[l], m, off) for l, m, off in inst])
        got = sc.closest(rays)
        want = O.instances_trace(lv, inst, rays)
        bad = np.nonzero(got["prim"] != want["prim"])[0]
        assert len(bad) == 0, (len(bad), bad[:5])
        assert np.array_equal(got["t"].view(np.uint32), want["t"].view(np.uint32))
        assert np.array_equal(sc.any(rays), O.instances_trace(lv, inst, rays, any_hit=True))
        assert (got["prim"] != 0xFFFFFFFF).mean() > 0.05
        with pytest.raises(fg.FndError):
            blas[0].close()  # still instanced
        img = ctx.render(sc, 8, 8, 1, dict(eye=(0, 0, 5), target=(0, 0, 0)), sky=(1, 1, 1))
        assert np.isfinite(img).all()
        empty = ctx.instances([])
        assert (empty.closest(rays[:100])["prim"] == fg.INVALID_ID).all()
        sc.close()
        blas[0].close()  # released with its two-level scene


@pytest.mark.gpu
def test_instanced_scene_renders_like_flattened(built):
    """A Cornell box whose spheres are instances of one unit icosphere renders
    like the same geometry flattened: same ray counts to within the few paths
    that ulp-level hit differences send elsewhere, images within noise."""
    import foundation_gb300 as fg
    cs = S.cornell_scene(num_spheres=0)
    sv, sf = S.icosphere(2)
    rng = np.random.default_rng(2)
    n = 24
    centres = np.stack([rng.uniform(-0.8, 0.8, n), rng.uniform(0.2, 1.8, n), rng.uniform(-0.8, 0.8, n)], 1)
    radii = rng.uniform(0.08, 0.2, n)
    mats = list(cs.materials)
    inst_mat = []
    for k in range(n):
        mats.append([k % 2, *rng.uniform(0.2, 0.9, 3), 0.3 if k % 2 else 1.0, 0, 0, 0])
        inst_mat.append(len(mats) - 1)
    mats = np.array(mats, np.float32)
    walls_n = cs.num_tris
    # flattened geometry and per-triangle materials in global-id order
    flat_v = [cs.verts]
    flat_f = [cs.idx]
    tri_mat = [cs.tri_material]
    base = len(cs.verts)
    transforms = []
    for k in range(n):
        m = np.zeros((3, 4), np.float32)
        m[:, :3] = np.eye(3) * radii[k]
        m[:, 3] = centres[k]
        transforms.append(m)
        w = (sv.astype(np.float64) @ m[:, :3].T.astype(np.float64) + m[:, 3]).astype(np.float32)
        flat_v.append(w)
        flat_f.append(sf + base)
        base += len(w)
        tri_mat.append(np.full(len(sf), inst_mat[k], np.uint32))
    flat_v = np.concatenate(flat_v).astype(np.float32)
    flat_f = np.concatenate(flat_f).astype(np.uint32)
    tri_mat = np.concatenate(tri_mat).astype(np.uint32)
    sc_mats = S.Scene(flat_v, flat_f, tri_material=tri_mat, materials=mats, lights=cs.lights)
    recs, lights = S.material_records(sc_mats), S.light_records(sc_mats)
    kw = dict(seed=3)
    with fg.Context(0) as ctx:
        flat = ctx.upload(flat_v, flat_f)
        flat.set_materials(tri_mat, recs)
        flat.set_lights(lights)
        a = ctx.render(flat, 64, 36, 256, S.CORNELL_CAMERA, **kw)
        sa = ctx.render_stats()
        walls = ctx.upload(cs.verts, cs.idx)
        sphere = ctx.upload(sv.astype(np.float32), sf)
        inst = [(walls, np.eye(3, 4, dtype=np.float32), 0)]
        inst += [(sphere, transforms[k], walls_n + k * len(sf)) for k in range(n)]
        two = ctx.instances(inst)
        two.set_materials(tri_mat, recs)
        two.set_lights(lights)
        b = ctx.render(two, 64, 36, 256, S.CORNELL_CAMERA, **kw)
        sb = ctx.render_stats()
        assert abs(sb["extension_rays"] / sa["extension_rays"] - 1) < 1e-3
        rel = float(np.mean((a - b) ** 2 / (a ** 2 + 1e-2)))
        assert rel < 2e-3 and abs(b.mean() / a.mean() - 1) < 0.01, (rel, a.mean(), b.mean())
        ctx.cache_create(two, train_paths=4096, train_steps=2, batch=1024, seed=1)
        c = ctx.render(two, 64, 36, 4, S.CORNELL_CAMERA, cache=True)
        assert np.isfinite(c).all() and c.mean() > 0
        two.close()


def test_emulated_two_level_traversal_matches_oracle(built):
    """The per-thread two-level traversal of the path-tracing megakernels
    (traverse.cuh trace_two_level, compiled for the host) over the product's
    host-side top level (bvh/instances.cpp): ids and t equal the oracle's."""
    import ctypes as C
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    L = C.CDLL(os.path.join(here, "_build", "libwide_emu.so"))
    P = C.c_void_p
    L.emu_build4.restype = P
    L.emu_build4.argtypes = [P, C.c_uint32, P, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_float]
    L.emu_instances.restype = P
    L.emu_instances.argtypes = [P, P, P, C.c_uint32]
    L.emu_instances_trace.argtypes = [P, P, C.c_uint64, P, C.c_int]
    L.emu_instance_reach.restype = C.c_double
    L.emu_instance_reach.argtypes = [P, C.c_uint32]
    L.emu_instances_free.argtypes = [P]
    L.emu_free.argtypes = [P]
    ptr = lambda a: a.ctypes.data_as(P)  # noqa: E731
    lv = levels()
    inst = random_instances(30, 2, seed=11)
    keep = [(np.ascontiguousarray(v, np.float32), np.ascontiguousarray(f, np.uint32)) for v, f in lv]
    blas = [L.emu_build4(ptr(v), len(v), ptr(f), len(f), 0, 0, 1.0, 64.0) for v, f in keep]
    arr = (P * len(inst))(*[blas[l] for l, _, _ in inst])
    tr = np.ascontiguousarray(np.stack([m.reshape(12) for _, m, _ in inst]), np.float32)
    off = np.asarray([o for _, _, o in inst], np.uint32)
    two = L.emu_instances(arr, ptr(tr), ptr(off), len(inst))
    assert max(L.emu_instance_reach(two, i) for i in range(len(inst))) < 32 * 64  # margin_scale 64 covers it
    rays = np.ascontiguousarray(np.concatenate([S.incoherent_rays(6000, (-2, -2, -2), (2, 2, 2), seed=8),
                                                S.camera_rays(48, 48, eye=(0, 0, 6), target=(0, 0, 0))]), np.float32)
    out = np.zeros(2 * len(rays), np.uint32)
    L.emu_instances_trace(two, ptr(rays), len(rays), ptr(out), 0)
    want = O.instances_trace(lv, inst, rays)
    assert np.array_equal(out[0::2], want["prim"])
    assert np.array_equal(out[1::2], want["t"].view(np.uint32))
    assert (want["prim"] != 0xFFFFFFFF).mean() > 0.05
    L.emu_instances_trace(two, ptr(rays), len(rays), ptr(out), 1)
    assert np.array_equal((out[0::2] != 0xFFFFFFFF).astype(np.uint8), O.instances_trace(lv, inst, rays, any_hit=True))
    L.emu_instances_free(two)
    for b in blas:
        L.emu_free(b)
