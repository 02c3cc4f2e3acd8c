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
    # the steps together are one full Lloyd iteration over every row, measured
    assert out["config"]["n"] == 20000 and "one full Lloyd iteration over all 20000 rows" in out["cpu_baseline"]["sample"]
    assert abs(out["ms_per_step"] * out["steps"] / 1e3 - 1.0 / out["value"]) < 1e-6 / out["value"]
    assert out["cpu_baseline"]["cpu_model"]


def test_both_arms_share_the_workload_config():
    sys.path.insert(0, ROOT)
    import bench
    from ferrolearn_gb300 import workloads as W
    w = W.anisotropic_1024x128(scale=0.002)
    cfg = bench.workload_config(w)
    assert cfg == {"workload": "anisotropic_1024x128", "n": 8000, "d": 128, "k": 1024, "X": "f32",
                   "init": "first k rows of a seeded permutation", "tol": 0.0,
                   "l2": "inputs larger than L2 (X 0.00 GB)", "parallelism": "replicas"}


def test_tensor_peak_follows_the_sampled_clock():
    sys.path.insert(0, ROOT)
    import bench
    peaks = {"bf16": 1911.1, "bf16s": 1715.8, "sm_max": 2070.0, "src": "measured"}
    assert bench.pick_tensor_peak(peaks, {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0})[0] == 1911.1
    assert bench.pick_tensor_peak(peaks, {"sm_mhz": 1462.0, "sm_max_mhz": 2070.0})[0] == 1715.8
    assert bench.pick_tensor_peak(peaks, {"sm_mhz": None, "sm_max_mhz": None})[0] == 1715.8


_RANK_SCRIPT = r"""
import os, sys, json
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method="env://")
rank, world = dist.get_rank(), dist.get_world_size()
ms = 100.0 + 50.0 * rank  # rank 1 is the slower replica
slowest = bench.max_over_ranks(ms, "cpu")
print(json.dumps({"rank": rank, "slowest": slowest, "rate": bench.job_rate(50, slowest, world)}))
dist.destroy_process_group()
"""


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.timeout(300)
def test_replicas_time_the_slowest_rank_gloo_world_2():
    # the N > 1 path: replicas, no data-path collective, one all-reduce (MAX)
    # of the timed region, whole-job rate = all ranks' iterations over it
    port = str(_free_port())
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=port)
        procs.append(subprocess.Popen([sys.executable, "-c", _RANK_SCRIPT, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True, cwd=ROOT))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=240)
        assert p.returncode == 0, e[-2000:]
        outs.append(json.loads([ln for ln in o.splitlines() if ln.startswith("{")][0]))
    for o in outs:
        assert o["slowest"] == 150.0
        assert abs(o["rate"] - 2 * 50 / 0.150) < 1e-9


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, "cpu") == 12.5
    assert bench.job_rate(50, 100.0, 1) == 500.0


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale", "0.005",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
