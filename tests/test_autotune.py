"""Tuned-parameter table: keys, nearest-bucket lookup, persistence (CPU),
and one tuning pass on the GPU."""
import numpy as np
import pytest

from foundation_gb300 import autotune as AT


def test_table_keys_lookup_and_persistence(tmp_path):
    t = AT.TuneTable()
    table = [dict(block=128, short_stack=8, refill_min=8, ms=2.0), dict(block=64, short_stack=4, refill_min=16, ms=1.5)]
    e = t.record(256012, "incoherent", 0, dict(block=64, short_stack=4, refill_min=16), table)
    assert e["ms"] == 1.5 and e["default_ms"] == 2.0
    assert AT.key(256012, "incoherent", 0) == "17:incoherent:closest"
    assert t.lookup(300000, "incoherent", 0)["block"] == 64     # same bucket
    assert t.lookup(5_000_000, "incoherent", 0)["block"] == 64  # nearest bucket
    assert t.lookup(1000, "coherent", 0) is None
    p = str(tmp_path / "tune.json")
    t.save(p)
    t2 = AT.TuneTable.load(p)
    assert t2.entries == t.entries
    assert AT.TuneTable.load(str(tmp_path / "missing.json")).entries == {}


@pytest.mark.gpu
def test_tune_pass_on_gpu(built, tmp_path):
    import torch
    import foundation_gb300 as fg
    from foundation_gb300 import scenes as S
    cs = S.cornell_scene(num_spheres=50)
    with fg.Context(0) as ctx:
        s = ctx.upload(cs.verts, cs.idx)
        rays = torch.from_numpy(S.incoherent_rays(1 << 17, *cs.bounds, seed=5)).cuda()
        t = AT.TuneTable()
        e = AT.tune_workload(ctx, t, s, rays, "incoherent", reps=1)
        assert e["ms"] <= e["default_ms"] + 1e-6
        cfg = t.apply(ctx, s.info()["num_tris"], "incoherent")
        assert ctx.trace_config() == cfg
        t.save(str(tmp_path / "t.json"))


@pytest.mark.gpu
def test_node_width_tuned(built, tmp_path):
    """The tuner's node-width dimension: every width is built and tuned, the
    recorded width is the fastest, and upload_options gives it back."""
    import torch
    import foundation_gb300 as fg
    from foundation_gb300 import scenes as S
    cs = S.cornell_scene(num_spheres=50)
    with fg.Context(0) as ctx:
        rays = torch.from_numpy(S.incoherent_rays(1 << 17, *cs.bounds, seed=6)).cuda()
        t = AT.TuneTable()
        e = AT.tune_node_width(ctx, t, cs.verts, cs.idx, rays, "incoherent", widths=(4, 8), reps=1,
                               sah_collapse=True)
        assert set(e["width_ms"]) == {"4", "8"}
        assert e["width_ms"][str(e["node_width"])] == min(e["width_ms"].values())
        opts = AT.upload_options(t, cs.num_tris, "incoherent")
        assert opts == dict(node_width=e["node_width"])
        s = ctx.upload(cs.verts, cs.idx, sah_collapse=True, **opts)
        assert s.info()["num_tris"] == cs.num_tris
        s.close()
        p = str(tmp_path / "t.json")
        t.save(p)
        assert AT.TuneTable.load(p).entries == t.entries


@pytest.mark.gpu
def test_render_queue_widths_tuned(built, tmp_path):
    import foundation_gb300 as fg
    from foundation_gb300 import scenes as S
    cs = S.cornell_scene(num_spheres=30, level=2)
    with fg.Context(0) as ctx:
        s = ctx.upload(cs.verts, cs.idx)
        s.set_materials(cs.tri_material, S.material_records(cs))
        s.set_lights(S.light_records(cs))
        t = AT.TuneTable()
        e = AT.tune_render(ctx, t, s, 320, 180, S.CORNELL_CAMERA, spp=4, waves=(1 << 16, 1 << 18), tails=(0, 4096),
                           reps=1)
        assert e["ms"] <= e["default_ms"] if e["default_ms"] else True
        opts = AT.render_options(t, 320, 180)
        assert opts == dict(wave_paths=e["wave_paths"], tail_paths=e["tail_paths"])
        img = ctx.render(s, 320, 180, 4, S.CORNELL_CAMERA, **opts)
        assert np.isfinite(img).all()
        p = str(tmp_path / "t.json")
        t.save(p)
        assert AT.render_options(AT.TuneTable.load(p), 320, 180) == opts
        assert AT.render_options(t, 64, 64) == {}
