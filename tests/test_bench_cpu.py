"""CPU checks of bench.py's contract: argument defaults and the reference arm's
JSON line (the reference arm runs the oracle on host cores only)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                       cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def test_default_steps_follow_the_workloads():
    sys.path.insert(0, ROOT)
    import bench
    saved = sys.argv
    try:
        sys.argv = ["bench.py"]
        assert bench.parse().steps == 50  # the anisotropic workload runs 50 Lloyd iterations
        sys.argv = ["bench.py", "--workload", "bisector"]
        assert bench.parse().steps == 20
        sys.argv = ["bench.py", "--steps", "7"]
        assert bench.parse().steps == 7
    finally:
        sys.argv = saved


@pytest.mark.timeout(600)
def test_reference_arm_line():
    out = _bench("--impl", "reference", "--scale", "0.005", "--steps", "2", "--warmup", "1")
    assert out["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "config",
                "cpu_baseline", "e2e"):
        assert key in out, key
    assert out["unit"] == "iters/s" and out["higher_is_better"] is True and out["value"] > 0
    assert out["cpu_baseline"]["kind"] == "port" and out["cpu_baseline"]["value"] == out["value"]
    assert out["e2e"]["value"] == out["value"]
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["e2e"]["d2h_bytes_per_step"] == 0
    assert out["config"]["workload"] == "anisotropic_1024x128"
