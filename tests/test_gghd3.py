"""DGGHD3-compatible entry (paraht_gghd3): reduction of rows/columns ilo..ihi only.

Against LAPACK dgghd3 with the same compq/compz/ilo/ihi (the oracle): backward error and
orthogonality <= 10 n eps, exact structure, the same |H|, |T| up to signs (both leave
Q e_ilo = e_ilo), the 'V' and 'N' semantics, and LAPACK-style argument errors.
"""
import numpy as np
import pytest

import paraht_gb300 as ph
from helpers import EPS, abs_rel_max_diff, bwd, orth
from paraht_gb300.generate import identity, pencil

pytestmark = pytest.mark.gpu


def balanced_pencil(n, ilo, ihi, seed=11):
    """A pencil as balancing leaves it: A upper triangular in columns 1..ilo-1 and rows ihi+1..n,
    B upper triangular."""
    A, B = pencil(n, "std", seed=seed)
    A = A.copy(order="F")
    for j in range(ilo - 1):
        A[j + 1:, j] = 0.0
    for i in range(ihi, n):
        A[i, :i] = 0.0
    return np.asfortranarray(A), np.asfortranarray(np.triu(B))


@pytest.mark.parametrize("n,ilo,ihi,r,p,nq", [(90, 1, 90, 8, 4, 8), (120, 11, 100, 8, 4, 8), (150, 30, 150, 16, 4, 16),
                                              (70, 1, 41, 4, 3, 4), (40, 5, 5, 4, 2, 2)])
def test_gghd3_matches_lapack(oracle, n, ilo, ihi, r, p, nq):
    A0, B0 = balanced_pencil(n, ilo, ihi)
    A, B, Q, Z = A0.copy(order="F"), B0.copy(order="F"), identity(n), identity(n)
    ph.gghd3("I", "I", ilo, ihi, A, B, Q, Z, r, p, nq)
    tol = 10 * n * EPS
    assert bwd(Q, A0, Z, A) <= tol and bwd(Q, B0, Z, B) <= tol
    assert orth(Q) <= tol and orth(Z) <= tol
    assert np.all(np.tril(A, -2) == 0.0) and np.all(np.tril(B, -1) == 0.0)
    Ao, Bo, Qo, Zo = A0.copy(order="F"), B0.copy(order="F"), identity(n), identity(n)
    assert oracle.dgghd3_range("I", "I", ilo, ihi, Ao, Bo, Qo, Zo) == 0
    assert abs_rel_max_diff(A, Ao) < 1e-8 and abs_rel_max_diff(B, Bo) < 1e-8
    # Q and Z are the identity outside the block
    out = np.r_[0:ilo - 1, ihi:n]
    assert np.array_equal(Q[np.ix_(out, out)], np.eye(len(out)))


def test_gghd3_accumulates_and_skips():
    n, ilo, ihi = 100, 7, 93
    A0, B0 = balanced_pencil(n, ilo, ihi, seed=5)
    A1, B1, Q1, Z1 = A0.copy(order="F"), B0.copy(order="F"), identity(n), identity(n)
    ph.gghd3("I", "I", ilo, ihi, A1, B1, Q1, Z1, 8, 4, 8)
    # 'V' right-multiplies the given orthogonal matrices
    rng = np.random.default_rng(3)
    U = np.asfortranarray(np.linalg.qr(rng.standard_normal((n, n)))[0])
    W = np.asfortranarray(np.linalg.qr(rng.standard_normal((n, n)))[0])
    A2, B2, Q2, Z2 = A0.copy(order="F"), B0.copy(order="F"), U.copy(order="F"), W.copy(order="F")
    ph.gghd3("V", "V", ilo, ihi, A2, B2, Q2, Z2, 8, 4, 8)
    assert np.array_equal(A1, A2) and np.array_equal(B1, B2)
    assert np.abs(Q2 - U @ Q1).max() < 1e-12 and np.abs(Z2 - W @ Z1).max() < 1e-12
    # 'N' leaves Q / Z alone (not referenced)
    A3, B3 = A0.copy(order="F"), B0.copy(order="F")
    ph.gghd3("N", "N", ilo, ihi, A3, B3, None, None, 8, 4, 8)
    assert np.array_equal(A1, A3) and np.array_equal(B1, B3)


def test_gghd3_argument_errors():
    n = 20
    A, B = balanced_pencil(n, 1, n)
    Q, Z = identity(n), identity(n)
    for args, code in ((("X", "I", 1, n), -1), (("I", "Y", 1, n), -2), (("I", "I", 0, n), -4),
                       (("I", "I", 3, 1), -5), (("I", "I", 1, n + 1), -5)):
        with pytest.raises(ph.ParahtError) as e:
            ph.gghd3(*args, A, B, Q, Z, 4, 2, 2)
        assert e.value.status == code
    with pytest.raises(ph.ParahtError) as e:
        ph.gghd3("I", "I", 1, n, A, B, Q, Z, 4, 2, 8)
    assert e.value.status == -16


def test_ht_convenience_returns_new_arrays(oracle):
    n = 120
    A0, B0 = pencil(n, "std", seed=21)
    for precision in ("split", "fp64"):
        H, T, Q, Z = ph.ht(A0, B0, precision)
        tol = 10 * n * EPS
        assert bwd(Q, A0, Z, H) <= tol and bwd(Q, B0, Z, T) <= tol
        assert np.all(np.tril(H, -2) == 0.0) and np.all(np.tril(T, -1) == 0.0)
    assert np.array_equal(A0, pencil(n, "std", seed=21)[0])  # inputs untouched
