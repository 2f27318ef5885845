"""bench.py's reference arm runs on the host alone: one JSON line with the contract's keys
(the CPU restatement of the reference's OpenMP algorithm, timed on a small sample)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    return json.loads(lines[0])


def test_reference_arm_pencil_line():
    d = _run("--impl", "reference", "--n", "2000", "--cpu-sample-n", "150", "--steps", "1", "--warmup", "1")
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == "s" and d["higher_is_better"] is False
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]


def test_reference_arm_batch_line():
    d = _run("--impl", "reference", "--workload", "batch4096", "--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference" and d["unit"] == "pencils/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and "n log-U" not in d["config"]["workload"]


def test_reference_arm_states_its_extrapolation():
    d = _run("--impl", "reference", "--n", "1200", "--cpu-sample-n", "200", "--steps", "3", "--warmup", "0")
    assert d["sample_n"] == 200 and d["extrapolated"] is True
    assert 1 <= d["steps"] <= 3 and d["steps_requested"] == 3
    assert abs(d["value"] - d["ms_per_step"] / 1e3 * (1200 / 200) ** 3) < 1e-9 * d["value"]


def test_budget_plan():
    sys.path.insert(0, ROOT)
    import bench

    # the first step always runs; later ones only while a step plus the reserve fits the budget
    assert bench.budget_plan(100.0, 99.0, 50.0, 0, 20, 10.0)
    assert bench.budget_plan(1500.0, 400.0, 150.0, 2, 20, 300.0)
    assert not bench.budget_plan(1500.0, 1100.0, 150.0, 3, 20, 300.0)
    assert not bench.budget_plan(1500.0, 10.0, 1.0, 20, 20, 0.0)  # all requested steps done
    args = bench.parse(["--steps", "20", "--warmup", "5"])
    assert args.budget_s + 0 <= 1700 and args.n == 16000 and args.fp64_params == "32,4,16"


def test_eig_mismatch_greedy_matching():
    import numpy as np

    sys.path.insert(0, ROOT)
    import bench

    assert bench.eig_mismatch([1.0, 2.0, np.inf], [2.0, np.inf, 1.0]) == 0.0
    assert abs(bench.eig_mismatch([1.0, 200.0], [1.0, 202.0]) - 0.01) < 1e-15  # relative to |lambda|
    assert bench.eig_mismatch([0.5], [0.6]) == pytest.approx(0.1)           # absolute below |lambda| = 1
    assert bench.eig_mismatch([1.0, np.inf], [1.0, 2.0]) == float("inf")    # an infinite one unmatched
    assert bench.eig_mismatch([1.0], [1.0, 2.0]) == float("inf")


def test_reference_arm_qz_line():
    """--workload qz1216: DHGEQZ on every host core over the whole batch of 1216 pencils."""
    d = _run("--workload", "qz1216", "--impl", "reference", "--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference" and d["unit"] == "pencils/s" and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert d["value"] > 0 and cb["value"] == d["value"] and cb["cores"] == (os.cpu_count() or 1)
    assert 0 < cb["one_core"] <= d["value"] * 1.5
