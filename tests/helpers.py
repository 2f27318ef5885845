"""Shared helpers for the parity tests: inputs, metrics and oracle runs."""
from __future__ import annotations

import numpy as np

from paraht_gb300.generate import identity, pencil

EPS = float(np.finfo(np.float64).eps)


def copies(*arrs):
    return [np.array(a, dtype=np.float64, order="F", copy=True) for a in arrs]


def bwd(Q, X0, Z, X):
    """||Q^T X0 Z - X||_F / ||X0||_F  (src/profilereduction.f90:165-174)."""
    nrm = np.linalg.norm(X0)
    return float(np.linalg.norm(Q.T @ X0 @ Z - X) / (nrm if nrm > 0 else 1.0))


def orth(Q):
    n = Q.shape[0]
    return float(np.abs(Q.T @ Q - np.eye(n)).max())


def rel_max_diff(X, Y):
    s = max(np.abs(Y).max(), 1e-300)
    return float(np.abs(X - Y).max() / s)


def abs_rel_max_diff(X, Y):
    """Elementwise |X| vs |Y| (HT form is unique up to row/column signs when Q e1 = e1)."""
    return rel_max_diff(np.abs(X), np.abs(Y))


def oracle_reduce(O, A0, B0, r, p, nq, stage=3):
    A, B = copies(A0, B0)
    n = A.shape[0]
    Q, Z = identity(n), identity(n)
    if stage & 1:
        O.ab2rht_simple(A, B, Q, Z, r, p)
    if stage & 2:
        O.rht2ht_householder(A, B, Q, Z, r, nq)
    return A, B, Q, Z


def make(n, dist="std", seed=1302):
    return pencil(n, dist, seed)


def eig_mismatch(l1, l2):
    """Largest distance from an eigenvalue of l1 to its greedy match in l2, relative to
    max(1, |lambda|); infinite eigenvalues must match infinite ones."""
    l1 = list(np.asarray(l1, dtype=complex))
    l2 = list(np.asarray(l2, dtype=complex))
    if len(l1) != len(l2):
        return np.inf
    worst = 0.0
    for lam in l1:
        if not np.isfinite(lam):
            idx = [i for i, m in enumerate(l2) if not np.isfinite(m)]
            if not idx:
                return np.inf
            l2.pop(idx[0])
            continue
        d = [abs(lam - m) if np.isfinite(m) else np.inf for m in l2]
        i = int(np.argmin(d))
        worst = max(worst, d[i] / max(1.0, abs(lam)))
        l2.pop(i)
    return worst
