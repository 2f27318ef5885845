"""CPU tests of the oracle (no GPU).

The reference ships no golden vectors and cannot be compiled here (no Fortran compiler), so
the oracle is pinned by:
* the reference's own acceptance figure: backward error ~4e-15 at n=1000, r=16, p=8, nq=8
  (README.md:12-13) -- checked here at n=400 with the same parameters and bound 10*n*eps;
* essential uniqueness: ParaHT and LAPACK DGGHD3 both leave Q e1 = e1 (no left transform touches
  row 1: src/ab2rht.f90:94 starts at jb+nb >= 2, src/rht2ht.f90:1487 at jc+1 >= 2), so the
  final H, T agree with DGGHD3's up to row/column signs (implicit-Q theorem);
* the reference's independent unblocked stage 2 (src/rht2ht.f90:2053-2180) on the same stage-1
  output;
* committed fixtures (tests/golden) produced by tests/golden/make_golden.py.
"""
import numpy as np
import pytest

from helpers import EPS, abs_rel_max_diff, bwd, copies, eig_mismatch, make, oracle_reduce, orth
from paraht_gb300.generate import identity

CASES = [(5, 2, 2, 2), (17, 3, 3, 2), (33, 4, 2, 3), (100, 16, 8, 8), (150, 8, 4, 8), (200, 16, 2, 4)]


@pytest.mark.parametrize("n,r,p,nq", CASES)
def test_oracle_backward_error_and_structure(oracle, n, r, p, nq):
    A0, B0 = make(n)
    A, B, Q, Z = oracle_reduce(oracle, A0, B0, r, p, nq)
    tol = 10 * n * EPS
    assert bwd(Q, A0, Z, A) <= tol and bwd(Q, B0, Z, B) <= tol
    assert orth(Q) <= tol and orth(Z) <= tol
    assert np.abs(np.tril(A, -2)).max(initial=0) == 0.0  # reduced columns are zeroed explicitly
    assert np.abs(np.tril(B, -1)).max(initial=0) <= 100 * EPS * np.abs(B).max()
    assert np.allclose(Q[:, 0], np.eye(n)[:, 0])  # Q e1 = e1


@pytest.mark.parametrize("n,r,p,nq", CASES)
def test_oracle_matches_dgghd3(oracle, n, r, p, nq):
    A0, B0 = make(n)
    A, B, Q, Z = oracle_reduce(oracle, A0, B0, r, p, nq)
    A3, B3 = copies(A0, B0)
    Q3, Z3 = identity(n), identity(n)
    assert oracle.dgghd3(A3, B3, Q3, Z3) == 0
    assert abs_rel_max_diff(A, A3) < 1e-9
    assert abs_rel_max_diff(np.triu(B), np.triu(B3)) < 1e-9
    assert abs_rel_max_diff(Q, Q3) < 1e-8


@pytest.mark.parametrize("n,r,p,nq", CASES)
def test_oracle_blocked_matches_unblocked_stage2(oracle, n, r, p, nq):
    A0, B0 = make(n)
    A1, B1, Q1, Z1 = oracle_reduce(oracle, A0, B0, r, p, nq, stage=1)
    Ab, Bb, Qb, Zb = copies(A1, B1, Q1, Z1)
    oracle.rht2ht_householder(Ab, Bb, Qb, Zb, r, nq)
    Au, Bu, Qu, Zu = copies(A1, B1, Q1, Z1)
    oracle.rht2ht_unblocked(Au, Bu, Qu, Zu, r)
    assert abs_rel_max_diff(Ab, Au) < 1e-10
    assert abs_rel_max_diff(np.triu(Bb), np.triu(Bu)) < 1e-10


def test_oracle_readme_configuration(oracle):
    # README.md:12-13: n=1000, r=16, p=8, nq=8 gives ~4e-15 backward error; same parameters at n=400.
    n = 400
    A0, B0 = make(n, "refcompat")
    A, B, Q, Z = oracle_reduce(oracle, A0, B0, 16, 8, 8)
    ea, eb = bwd(Q, A0, Z, A), bwd(Q, B0, Z, B)
    assert ea < 1e-14 and eb < 1e-14


def test_oracle_eigenvalues_preserved(oracle):
    n = 60
    A0, B0 = make(n)
    A, B, _, _ = oracle_reduce(oracle, A0, B0, 4, 4, 4)
    ar, ai, be, info = oracle.dhgeqz_eigs(A, B)
    assert info == 0
    import scipy.linalg as sl

    w = sl.eigvals(A0, B0)
    lam = (ar + 1j * ai) / be
    assert eig_mismatch(lam, w) < 1e-7


def test_oracle_graded_singular_b(oracle):
    n = 120
    A0, B0 = make(n, "graded")
    assert np.sum(np.diag(B0) == 0.0) == round(0.02 * n)
    A, B, Q, Z = oracle_reduce(oracle, A0, B0, 8, 4, 8)
    assert bwd(Q, A0, Z, A) <= 10 * n * EPS and bwd(Q, B0, Z, B) <= 10 * n * EPS


def test_oracle_phase_times(oracle):
    n = 80
    A0, B0 = make(n)
    A, B = copies(A0, B0)
    Q, Z = identity(n), identity(n)
    t1 = oracle.ab2rht_simple(A, B, Q, Z, 8, 4, time_components=True)
    t2 = oracle.rht2ht_householder(A, B, Q, Z, 8, 4, time_components=True)
    assert all(t >= 0 for t in t1 + t2) and sum(t1) > 0 and sum(t2) > 0


GIVENS_CASES = [(5, 2, 2, 2), (17, 3, 3, 2), (33, 4, 2, 3), (100, 16, 8, 8), (150, 8, 4, 8), (200, 16, 2, 16)]


@pytest.mark.parametrize("n,r,p,nq", GIVENS_CASES)
def test_oracle_givens_stage2(oracle, n, r, p, nq):
    """The reference's Givens stage 2 (src/rht2ht.f90:696-1344), restated: backward error and
    orthogonality within 10 n eps, exact Hessenberg zeros, and the Householder stage 2's H, T up to
    row/column signs (both leave Q e1 = e1)."""
    A0, B0 = make(n)
    A1, B1, Q1, Z1 = oracle_reduce(oracle, A0, B0, r, p, nq, stage=1)
    Ag, Bg, Qg, Zg = copies(A1, B1, Q1, Z1)
    oracle.rht2ht_givens(Ag, Bg, Qg, Zg, r, nq)
    tol = 10 * n * EPS
    assert bwd(Qg, A0, Zg, Ag) <= tol and bwd(Qg, B0, Zg, Bg) <= tol
    assert orth(Qg) <= tol and orth(Zg) <= tol
    assert np.abs(np.tril(Ag, -2)).max(initial=0) == 0.0
    assert np.abs(np.tril(Bg, -1)).max(initial=0) <= 100 * EPS * np.abs(Bg).max()
    Ah, Bh, Qh, Zh = copies(A1, B1, Q1, Z1)
    oracle.rht2ht_householder(Ah, Bh, Qh, Zh, r, nq)
    assert abs_rel_max_diff(np.triu(Ag, -1), np.triu(Ah, -1)) < 1e-10
    assert abs_rel_max_diff(np.triu(Bg), np.triu(Bh)) < 1e-10


@pytest.mark.parametrize("r", [4, 8, 16])
@pytest.mark.parametrize("n", [97, 160, 203, 240])
def test_oracle_givens_domain_nq_r_plus_1(oracle, n, r):
    """The Givens stage 2 is exact up to nq = r + 1, the edge of the domain the library accepts
    for both stage-2 variants (nq <= r; the reference's own index bookkeeping goes wrong for some n
    once nq exceeds r + 1 by more)."""
    nq = r + 1
    A0, B0 = make(n)
    S1 = oracle_reduce(oracle, A0, B0, r, 4, r, stage=1)
    A, B, Q, Z = copies(*S1)
    oracle.rht2ht_givens(A, B, Q, Z, r, nq)
    tol = 10 * n * EPS
    assert bwd(Q, A0, Z, A) <= tol and bwd(Q, B0, Z, B) <= tol
