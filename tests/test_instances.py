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
        with pytest.raises(fg.FndError):
            ctx.render(sc, 8, 8, 1, dict(eye=(0, 0, 5), target=(0, 0, 0)))
        empty = ctx.instances([])
        assert (empty.closest(rays[:100])["prim"] == fg.INVALID_ID).all()
        sc.close()
        blas[0].close()  # released with its two-level scene
