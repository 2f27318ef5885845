"""Autotuner table lookup (host logic, no GPU)."""
import json

from paraht_gb300 import tune


def test_pick_nearest_size_on_log_scale(tmp_path):
    table = {"split": [[1000, 16, 4, 16], [4000, 32, 2, 16]], "fp64": [[1000, 16, 4, 8]], "batch": [[256, 8, 4, 8]]}
    p = tmp_path / "t.json"
    p.write_text(json.dumps(table))
    t = tune.load_table(str(p))
    assert tune.pick(900, "split", t) == (16, 4, 16)
    assert tune.pick(2100, "split", t) == (32, 2, 16)  # log-nearest: 2100 is closer to 4000 than to 1000
    assert tune.pick(16000, "split", t) == (32, 2, 16)
    assert tune.pick(5000, "fp64", t) == (16, 4, 8)
    assert tune.pick(40, "batch", t) == (8, 4, 8)


def test_pick_clamps_bandwidth_for_tiny_pencils():
    t = {"split": [[1000, 16, 4, 16]], "fp64": [[1000, 16, 4, 16]], "batch": [[256, 16, 4, 16]]}
    r, p, nq = tune.pick(5, "batch", t)
    assert r == 4 and nq == 4 and p == 4


def test_missing_table_falls_back(tmp_path):
    t = tune.load_table(str(tmp_path / "absent.json"))
    assert set(t) == {"split", "fp64", "batch"}
    r, p, nq = tune.pick(16000, "split", t)
    assert 1 <= nq <= r and p >= 2


def test_stage2_variant_per_mode(tmp_path):
    table = {"split": [[1000, 16, 4, 16]], "fp64": [[1000, 32, 4, 16]], "batch": [[256, 16, 4, 16]],
             "stage2": {"split": "givens", "fp64": "householder"}}
    assert tune.stage2("split", 16, 16, table) == "givens"
    assert tune.stage2("fp64", 32, 16, table) == "householder"
    assert tune.stage2("batch", 16, 16, table) == "householder"  # the persistent kernel chases with reflectors
    assert tune.stage2("split", 48, 8, table) == "householder"   # the Givens variant needs r <= 32
    assert tune.stage2("split", 32, 40, table) == "householder"  # ... and r + nq <= 64
    assert tune.stage2("split", 16, 16, {}) == "givens"          # no table entry: the measured default
    assert tune.stage2("split", 16, 16) in ("givens", "householder")  # the shipped table
