"""Seeded synthetic pencils (A, B) for tests and benchmarks.

The reference driver draws U[0,1) entries with the gfortran RNG and seed 1302, then replaces B
by the R factor of its QR factorisation (src/profilereduction.f90:38-44, :114-123).  The
gfortran stream cannot be reproduced without gfortran, so every pencil here comes from numpy's
PCG64 generator with the same seed (1302 by default); the same arrays are fed to the GPU path
and to the CPU oracle.

Distributions
-------------
``std``       A ~ N(0,1); B = R factor of QR(G), G ~ N(0,1); A <- Q^T A.
              Generated through the Bartlett decomposition: the R factor of a Gaussian matrix has
              independent N(0,1) entries above the diagonal and chi(n-i+1)-distributed diagonal
              entries, and Q^T A is again i.i.d. N(0,1) by orthogonal invariance.  This is the same
              distribution as the explicit construction at O(n^2) cost, which matters at n=16000.
``std_qr``    the explicit construction (numpy QR), for small n.
``graded``    A ~ N(0,1); B upper triangular with N(0,1) strictly upper part and diagonal
              d_i = 10^(-10 (i-1)/(n-1)); exactly round(0.02 n) diagonal entries (seeded choice)
              are set to 0, which gives infinite eigenvalues.
``refcompat`` A, B ~ U[0,1); B <- R of QR(B); A unchanged (the reference driver's recipe).
"""
from __future__ import annotations

import numpy as np

DISTRIBUTIONS = ("std", "std_qr", "graded", "refcompat")


def pencil(n: int, dist: str = "std", seed: int = 1302):
    """Returns Fortran-ordered float64 (A, B) of size n x n, B upper triangular."""
    if n < 1:
        raise ValueError("n must be >= 1")
    rng = np.random.default_rng(seed)
    if dist == "std":
        A = rng.standard_normal((n, n))
        B = np.triu(rng.standard_normal((n, n)), 1)
        dfree = n - np.arange(n)  # chi(n-i+1) for row i (0-based i -> n-i degrees of freedom)
        diag = np.sqrt(rng.chisquare(dfree))
        diag *= np.where(rng.random(n) < 0.5, -1.0, 1.0)
        B[np.arange(n), np.arange(n)] = diag
    elif dist == "std_qr":
        A = rng.standard_normal((n, n))
        G = rng.standard_normal((n, n))
        q, r = np.linalg.qr(G)
        A = q.T @ A
        B = np.triu(r)
    elif dist == "graded":
        A = rng.standard_normal((n, n))
        B = np.triu(rng.standard_normal((n, n)), 1)
        expo = -10.0 * np.arange(n) / max(n - 1, 1)
        d = 10.0 ** expo
        nz = int(round(0.02 * n))
        if nz > 0:
            d[rng.choice(n, size=nz, replace=False)] = 0.0
        B[np.arange(n), np.arange(n)] = d
    elif dist == "refcompat":
        A = rng.random((n, n))
        G = rng.random((n, n))
        B = np.triu(np.linalg.qr(G)[1])
    else:
        raise ValueError(f"unknown distribution {dist!r}; choose from {DISTRIBUTIONS}")
    return np.asfortranarray(A, dtype=np.float64), np.asfortranarray(B, dtype=np.float64)


def identity(n: int):
    return np.asfortranarray(np.eye(n))


def batch_sizes(count: int, lo: int, hi: int, law: str = "uniform", seed: int = 1302):
    """Pencil sizes of a batch: n ~ U{lo..hi} (law "uniform") or n = floor(exp(U[ln lo, ln hi]))
    (law "loguniform"), seeded."""
    rng = np.random.default_rng(seed)
    if law == "uniform":
        return [int(v) for v in rng.integers(lo, hi + 1, size=count)]
    if law == "loguniform":
        return [int(np.floor(np.exp(v))) for v in rng.uniform(np.log(lo), np.log(hi), size=count)]
    raise ValueError(f"unknown size law {law!r}")
