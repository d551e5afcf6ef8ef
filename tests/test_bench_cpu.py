"""bench.py's reference arm (the oracle timed on the host cores) needs no GPU:
its JSON line is checked here on an 8 x 8 x 4 grid, and so is the rule that
under torchrun only rank 0 runs it and the other ranks exit 0 without work."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--ni", "8", "--nj", "8", "--nk", "4", "--steps", "2", "--warmup", "1"]


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *ARGS], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=300)


def test_reference_arm_line():
    r = _run({"RANK": "0", "WORLD_SIZE": "1"})
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["metric"] == d["unit"] == "cell-Newton-steps/s"
    assert d["steps"] == 2 and d["warmup"] == 1 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["config"]["cells"] == 256
    # the converged Newton loop of the GPU line: at least one iteration per step
    assert d["newton_iterations"] >= 2 and d["linear_iterations"] > 0
    assert set(d["config"]) == {"workload", "cells", "pattern_nnz", "dt_s", "seed"}
    assert "first K steps from the initial state" in d["config"]["workload"]
    assert "java" in d["jvm"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] == 1
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_sweep_bytes():
    """Algorithmic bytes of the ILU(0) level walks that the roofline divides
    by: 12 B per strictly lower (upper) entry, 16 (24) B per row."""
    import numpy as np

    import bench

    rp = np.array([0, 2, 5, 7], np.int32)  # 3 x 3 tridiagonal
    col = np.array([0, 1, 0, 1, 2, 1, 2], np.int32)
    assert bench.sweep_bytes(rp, col) == (12 * 2 + 16 * 3, 12 * 2 + 24 * 3)


def test_both_arms_describe_the_same_workload():
    """The GPU line and the reference line build their config from one
    function, so the driver sees the same workload on both."""
    import argparse

    import bench

    a = argparse.Namespace(ni=128, nj=128, nk=32, rtol=1e-8, seed=1)
    assert bench.config_of(a, 13716856, 8640.0) == bench.config_of(a, 13716856, 8640.0)
    src = open(os.path.join(ROOT, "bench.py")).read()
    assert src.count('"config": config_of(args, len(col)') == 2
