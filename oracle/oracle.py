"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module.  It restates the reference's Fortran interfaces on numpy arrays
(column-major, 1-based semantics handled inside the C code):

* ``ab2rht_simple``        -> src/ab2rht.f90:8     (stage 1)
* ``rht2ht_householder``   -> src/rht2ht.f90:1346  (stage 2, compact WY, lookahead)
* ``rht2ht_unblocked``     -> src/rht2ht.f90:2053  (stage 2, simple cross-check)
* ``rht2ht_givens``        -> src/rht2ht.f90:696   (stage 2 with Givens rotations)
* ``dgghd3``               -> src/profilereduction.f90:156 (LAPACK one-stage baseline)
* ``backward_error``       -> src/profilereduction.f90:165-174
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        d = C.POINTER(C.c_double)
        i = C.c_int
        L.oracle_ab2rht_simple.argtypes = [i, d, i, d, i, d, i, d, i, i, i, i, d]
        L.oracle_rht2ht_householder.argtypes = [i, d, i, d, i, d, i, d, i, i, i, i, d]
        L.oracle_rht2ht_unblocked.argtypes = [i, d, i, d, i, d, i, d, i, i]
        L.oracle_rht2ht_givens.argtypes = [i, d, i, d, i, d, i, d, i, i, i]
        L.oracle_dgghd3.argtypes = [i, d, i, d, i, d, i, d, i]
        L.oracle_dgghd3_range.argtypes = [C.c_char, C.c_char, i, i, i, d, i, d, i, d, i, d, i]
        L.oracle_dhgeqz_eigs.argtypes = [i, d, i, d, i, d, d, d]
        L.oracle_triangularize.argtypes = [i, d, i]
        L.oracle_backward_error.argtypes = [i, d, i, d, i, d, i, d, i]
        L.oracle_backward_error.restype = C.c_double
        L.oracle_set_blas_threads.argtypes = [i]
        L.oracle_lapack_error.restype = C.c_char_p
        err = L.oracle_lapack_error()
        if err:
            raise RuntimeError("oracle LAPACK unavailable: " + err.decode())
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.f_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _check(*arrs):
    for a in arrs:
        if a.dtype != np.float64 or not a.flags.f_contiguous:
            raise TypeError("oracle arrays must be float64, Fortran-ordered")


def set_blas_threads(t: int) -> None:
    lib().oracle_set_blas_threads(int(t))


def ab2rht_simple(A, B, Q, Z, nb, p, time_components=False):
    """In-place stage 1 on Fortran-ordered float64 arrays; returns phase times (genleft, genright, mul)."""
    _check(A, B, Q, Z)
    n = A.shape[0]
    ph = (C.c_double * 3)()
    rc = lib().oracle_ab2rht_simple(n, _ptr(A), A.shape[0], _ptr(B), B.shape[0], _ptr(Q), Q.shape[0], _ptr(Z),
                                    Z.shape[0], int(nb), int(p), int(bool(time_components)), ph)
    if rc != 0:
        raise RuntimeError(f"oracle_ab2rht_simple failed: {rc}")
    return tuple(ph)


def rht2ht_householder(A, B, Q, Z, r, nq, time_components=False):
    """In-place stage 2; returns phase times (generation, lookahead, application)."""
    _check(A, B, Q, Z)
    n = A.shape[0]
    ph = (C.c_double * 3)()
    rc = lib().oracle_rht2ht_householder(n, _ptr(A), A.shape[0], _ptr(B), B.shape[0], _ptr(Q), Q.shape[0], _ptr(Z),
                                         Z.shape[0], int(r), int(nq), int(bool(time_components)), ph)
    if rc != 0:
        raise RuntimeError(f"oracle_rht2ht_householder failed: {rc}")
    return tuple(ph)


def rht2ht_unblocked(A, B, Q, Z, r):
    _check(A, B, Q, Z)
    n = A.shape[0]
    rc = lib().oracle_rht2ht_unblocked(n, _ptr(A), n, _ptr(B), n, _ptr(Q), n, _ptr(Z), n, int(r))
    if rc != 0:
        raise RuntimeError(f"oracle_rht2ht_unblocked failed: {rc}")


def rht2ht_givens(A, B, Q, Z, r, nq):
    """In-place stage 2 with Givens rotations (src/rht2ht.f90:696-1344)."""
    _check(A, B, Q, Z)
    n = A.shape[0]
    rc = lib().oracle_rht2ht_givens(n, _ptr(A), A.shape[0], _ptr(B), B.shape[0], _ptr(Q), Q.shape[0], _ptr(Z),
                                    Z.shape[0], int(r), int(nq))
    if rc != 0:
        raise RuntimeError(f"oracle_rht2ht_givens failed: {rc}")


def dgghd3(A, B, Q, Z):
    _check(A, B, Q, Z)
    n = A.shape[0]
    return lib().oracle_dgghd3(n, _ptr(A), n, _ptr(B), n, _ptr(Q), n, _ptr(Z), n)


def dgghd3_range(compq, compz, ilo, ihi, A, B, Q, Z):
    """LAPACK dgghd3(compq, compz, n, ilo, ihi, ...) in place (1-based ilo/ihi)."""
    _check(A, B, Q, Z)
    n = A.shape[0]
    return lib().oracle_dgghd3_range(compq.encode(), compz.encode(), n, int(ilo), int(ihi), _ptr(A), n, _ptr(B), n,
                                     _ptr(Q), n, _ptr(Z), n)


def dhgeqz_eigs(H, T):
    """Generalized eigenvalues (alphar, alphai, beta) of the HT pencil (H, T) via LAPACK DHGEQZ."""
    H = np.array(H, dtype=np.float64, order="F", copy=True)
    T = np.array(T, dtype=np.float64, order="F", copy=True)
    n = H.shape[0]
    ar = np.zeros(n)
    ai = np.zeros(n)
    be = np.zeros(n)
    info = lib().oracle_dhgeqz_eigs(n, _ptr(H), n, _ptr(T), n, ar.ctypes.data_as(C.POINTER(C.c_double)),
                                    ai.ctypes.data_as(C.POINTER(C.c_double)), be.ctypes.data_as(C.POINTER(C.c_double)))
    return ar, ai, be, info


def triangularize(B):
    _check(B)
    return lib().oracle_triangularize(B.shape[0], _ptr(B), B.shape[0])


def backward_error(Q, A0, Z, H):
    _check(Q, A0, Z, H)
    n = A0.shape[0]
    return lib().oracle_backward_error(n, _ptr(Q), n, _ptr(A0), n, _ptr(Z), n, _ptr(H), n)


def reduce(A, B, Q, Z, r, p, nq, time_components=False):
    """Both stages, as profilereduction.f90:136,144 calls them."""
    t1 = ab2rht_simple(A, B, Q, Z, r, p, time_components)
    t2 = rht2ht_householder(A, B, Q, Z, r, nq, time_components)
    return t1, t2
