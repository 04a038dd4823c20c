"""bench.py on the CPU: the reference arm's JSON line (the oracle timed on the
host cores) and the workload description shared with the GPU arm."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _run(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                          capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)


@pytest.mark.parametrize("workload", ["cornell", "soup1m"])
def test_reference_arm_line(workload):
    r = _run({}, "--steps", "2", "--warmup", "1", "--rays", "65536", "--workload", workload)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "Mrays/s closest-hit" and d["unit"] == "Mrays/s"
    assert d["higher_is_better"] is True and d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "all 65536 rays" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cfg = d["config"]
    assert cfg["rays_per_step_per_gpu"] == 65536
    assert cfg["workload"].startswith("cornell200" if workload == "cornell" else "soup1m")
    assert cfg["l2"].startswith("inputs within L2")


def test_reference_arm_other_ranks_silent():
    r = _run({"RANK": "1", "WORLD_SIZE": "2"}, "--steps", "1", "--warmup", "0", "--rays", "4096")
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_l2_note():
    import bench
    assert bench.l2_note(bench.N_RAYS) == "inputs larger than L2: 268 MB of rays streamed per step per GPU"
    assert bench.l2_note(1 << 20).startswith("inputs within L2: 33.6 MB")


def test_target_figures_are_scalars():
    import bench
    blocks = {"incoherent_1m_tris": {"best": {"mrays_s": 2100.0}, "target_mrays_s": 1500.0},
              "time_to_relmse_1080p": {"speedup_cache_vs_plain": 3.2, "target_speedup": 3.0},
              "path_tracer": {"frame_ms": 139.0}, "batched_256_scenes": {"grays_s": 1.9},
              "large_scene_4k": {"incoherent_mrays_s": 3800.0}}
    t = bench.target_figures(blocks)
    assert t["target_soup1m_mrays_s"] == 2100.0 and t["target_cache_speedup_to_relmse_1e3"] == 3.2
    assert all(isinstance(v, float) for v in t.values())
    assert bench.target_figures({}) == {}


def test_profile_figures_parse(tmp_path, monkeypatch):
    import bench
    (tmp_path / "trace_closest_cornell_incoherent.txt").write_text(
        "header\ndram_bytes_per_launch: 324571136\nwarp_inst_per_launch: 2.141e9   (255 per ray)\n"
        "issue_active_pct: 84.6\nother: 3\n")
    monkeypatch.setattr(bench, "PROFILES", str(tmp_path))
    f = bench.profile_figures("cornell")
    assert f == {"dram_bytes_per_launch": 324571136.0, "warp_inst_per_launch": 2.141e9, "issue_active_pct": 84.6}
