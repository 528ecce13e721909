"""The reference arm of bench.py (the oracle, the CPU restatement of the
reference, on the host cores) prints exactly one contract line; a tiny sample
keeps the CPU suite fast."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--cpu-rays", "16"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["metric"] == "ray-steps/s" and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "ray-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_curvature_cpu_leg(orc):
    """The config-4 CPU baseline times the oracle with the reference's call
    graph (Riemann again inside every call) and with Riemann once; the former
    forms Riemann 34 times per point (2 for the Einstein tensor, 2 per vector)."""
    sys.path.insert(0, ROOT)
    import bench
    from geon_gb300.curvature import grid_points
    pts = grid_points((-4, -4, -4), (4, 4, 4), (32, 32, 32))
    r = bench.curvature_cpu_leg(orc, [2.0, 0.125, 0.5, 0.0], pts, orc.hardware_threads(), budget_s=0.3)
    assert set(r) == {"reference_call_graph", "riemann_once"}
    for v in r.values():
        assert v["value"] > 0 and 256 <= v["points"] <= len(pts) and v["seconds"] > 0
    assert r["riemann_once"]["value"] > 3 * r["reference_call_graph"]["value"]


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun (N > 1) rank 0 alone runs and prints the reference arm."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--cpu-rays", "16"], capture_output=True, text=True, timeout=600, cwd=ROOT,
                         env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    assert not [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
