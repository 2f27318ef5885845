"""Pencil files (stage-1 output saved for a stage-2-only run): round trip, header, mapping and
corrupt-file errors.  Host logic only; the stage split itself is exercised against the oracle on
the CPU (stage 1 saved, reloaded, stage 2 run on it gives the two-stage result bit for bit)."""
import numpy as np
import pytest

from paraht_gb300 import pencilio
from paraht_gb300.generate import identity, pencil


def test_round_trip_and_header(tmp_path):
    A, B = pencil(37, "std", seed=3)
    Q, Z = identity(37), identity(37)
    Q[0, 1] = 0.5
    p = str(tmp_path / "p.pht")
    pencilio.save_pencil(p, A, B, Q, Z, stage=1, r=4, p=3)
    head = pencilio.read_header(p)
    assert head["n"] == 37 and head["stage"] == 1 and head["r"] == 4 and head["matrices"] == ["A", "B", "Q", "Z"]
    for mm in (False, True):
        h2, mats = pencilio.load_pencil(p, mmap=mm)
        for k, X in zip("ABQZ", (A, B, Q, Z)):
            assert np.array_equal(mats[k], X) and mats[k].flags.f_contiguous


def test_optional_transforms_and_errors(tmp_path):
    A, B = pencil(8, "std", seed=4)
    p = str(tmp_path / "ab.pht")
    pencilio.save_pencil(p, A, B)
    head, mats = pencilio.load_pencil(p)
    assert set(mats) == {"A", "B"}
    with open(p, "ab") as f:
        f.write(b"x")
    with pytest.raises(ValueError):
        pencilio.load_pencil(p)
    bad = tmp_path / "bad.pht"
    bad.write_bytes(b"NOTAPENC" + bytes(16))
    with pytest.raises(ValueError):
        pencilio.read_header(str(bad))
    with pytest.raises(ValueError):
        pencilio.save_pencil(str(tmp_path / "x.pht"), A, B[:4, :4])


def test_stage_split_through_a_file_matches_two_stages(tmp_path, oracle):
    n, r, p, nq = 60, 4, 3, 4
    A0, B0 = pencil(n, "std", seed=9)
    A, B, Q, Z = A0.copy(order="F"), B0.copy(order="F"), identity(n), identity(n)
    oracle.ab2rht_simple(A, B, Q, Z, r, p)
    f = str(tmp_path / "s1.pht")
    pencilio.save_pencil(f, A, B, Q, Z, stage=1, r=r, p=p)
    _, m = pencilio.load_pencil(f)
    A1, B1, Q1, Z1 = (np.array(m[k], order="F") for k in "ABQZ")
    oracle.rht2ht_householder(A1, B1, Q1, Z1, r, nq)
    oracle.rht2ht_householder(A, B, Q, Z, r, nq)
    for X, Y in zip((A1, B1, Q1, Z1), (A, B, Q, Z)):
        assert np.array_equal(X, Y)
