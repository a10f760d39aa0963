"""bench.py's reference arm on the CPU (the oracle on the host cores): one
JSON line with the contract's keys, and under torchrun only rank 0 prints."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--dim", "2",
        "--dr", "0.05", "--steps", "1", "--warmup", "1"]


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    r = subprocess.run(ARGS, capture_output=True, text=True, env=env, cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stderr
    return [ln for ln in r.stdout.splitlines() if ln.strip()]


def test_reference_arm_line():
    lines = _run({"RANK": "0", "WORLD_SIZE": "1"})
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]


def test_reference_arm_other_ranks_silent():
    assert _run({"RANK": "1", "WORLD_SIZE": "2"}) == []


def test_pair_once_flops_below_per_hit_count():
    """The FP64 count is per unordered pair plus per-target accumulation, so
    one fluid-fluid pair (two directed hits) costs less than two mixed hits,
    each of which is evaluated in full."""
    sys.path.insert(0, ROOT)
    import bench
    cats = dict(density=200, wall=10, force_fluid=180, force_wall=10, force_av=60)
    for dim in (2, 3):
        f64 = bench.pass_flops(cats, dim, False)
        f32 = bench.pass_flops(cats, dim, True)
        assert 0 < f64["force"] < f32["force"]
        assert 0 < f64["density"] < f32["density"]
        F = bench.FP64_FLOPS[dim]
        assert f64["force"] == (90 * F["ff_pair"] + 30 * F["av_pair"] + 10 * F["fw_pair"]
                                + 180 * (F["acc_a"] + F["acc_x"]) + 10 * F["acc_a"])
