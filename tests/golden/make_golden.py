"""Generates the committed golden fixtures (tests/golden/*.npz) from the CPU oracle.

Each fixture holds a seeded input pencil (A0, B0), the oracle's stage-1 output (A1, B1, Q1, Z1)
and its final output (H, T, Q, Z), for the parameters in CASES.  The GPU parity tests compare
against these files, so a GPU run does not depend on rebuilding the oracle, and the CPU tests
check that the oracle still reproduces them.

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from paraht_gb300.generate import identity, pencil  # noqa: E402

# (name, n, r, p, nq, dist)
CASES = [
    ("n5_r2_p2_nq2", 5, 2, 2, 2, "std"),
    ("n17_r3_p3_nq2", 17, 3, 3, 2, "std"),
    ("n33_r4_p2_nq3", 33, 4, 2, 3, "std"),
    ("n64_r8_p4_nq8_graded", 64, 8, 4, 8, "graded"),
    ("n100_r16_p8_nq8", 100, 16, 8, 8, "std"),
    ("n96_r16_p8_nq8_refcompat", 96, 16, 8, 8, "refcompat"),
]


def run_case(n, r, p, nq, dist):
    A0, B0 = pencil(n, dist, seed=1302)
    A = A0.copy(order="F")
    B = B0.copy(order="F")
    Q, Z = identity(n), identity(n)
    O.ab2rht_simple(A, B, Q, Z, r, p)
    A1, B1, Q1, Z1 = (X.copy(order="F") for X in (A, B, Q, Z))
    O.rht2ht_householder(A, B, Q, Z, r, nq)
    return dict(A0=A0, B0=B0, A1=A1, B1=B1, Q1=Q1, Z1=Z1, H=A, T=B, Q=Q, Z=Z,
                params=np.array([n, r, p, nq]), dist=np.array(dist))


def main():
    O.set_blas_threads(1)
    for name, n, r, p, nq, dist in CASES:
        d = run_case(n, r, p, nq, dist)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print("wrote", name)


if __name__ == "__main__":
    main()
