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
