"""bench.py's reference arm on the CPU: one JSON line with the contract's keys, and
silence on ranks other than 0 (the arm times the oracle, which needs no GPU)."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
        "restriction", "--steps", "1", "--warmup", "3", "--ref-units", "2e5"]


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run(ARGS, capture_output=True, text=True, env=env, timeout=600, cwd=ROOT)


def test_reference_arm_prints_one_contract_line():
    p = _run({"RANK": "0", "WORLD_SIZE": "1"})
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert key in out, key
    assert out["value"] > 0 and out["higher_is_better"] is True
    assert out["cpu_baseline"]["value"] == out["value"]
    assert out["cpu_baseline"]["kind"] in ("port", "reference") and out["cpu_baseline"]["cores"] >= 1
    assert out["e2e"]["value"] == out["value"] and out["e2e"]["unit"] == out["unit"]
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["e2e"]["d2h_bytes_per_step"] == 0
    assert out["config"]["workload"] == "restriction"


def test_reference_arm_other_ranks_exit_quietly():
    p = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""


def test_cpu_legs_share_one_sample():
    """The reference arm and the GPU arm's cpu_baseline time the oracle on the same
    windows: one per instance, at a fixed stride through the workload, up to the
    unit budget."""
    sys.path.insert(0, ROOT)
    import bench
    from mcphylo_gb300 import simulate
    insts = [simulate.restriction_small(seed=s) for s in range(5)]
    per = insts[0].units()
    w = bench.oracle_windows(insts, 3 * per - 1)
    assert len(w) == 3 and [x[2].parent is insts[i].parent for i, x in enumerate(w)] == [True] * 3
    w2 = bench.oracle_windows(insts, 3 * per - 1)
    assert all(np.array_equal(a[2].codes, b[2].codes) for a, b in zip(w, w2))
    one = bench.oracle_windows([simulate.restriction_small()], 1e12, window=300)
    assert len(one) == 4 and sum(x[2].codes.shape[1] for x in one) == 1000


def test_gpu_arm_cpu_leg_is_the_reference_arm():
    """The GPU arm's cpu_baseline leg runs the reference arm in a child process and
    reports its line."""
    import argparse
    sys.path.insert(0, ROOT)
    import bench
    a = argparse.Namespace(workload="restriction", cpu_steps=1, ref_units=2e5)
    out = bench.cpu_leg(a)
    assert out["impl"] == "reference" and out["steps"] == 1 and out["value"] > 0
    assert out["config"]["workload"] == "restriction"
