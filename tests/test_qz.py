"""QZ eigenvalues of Hessenberg-triangular pencils (paraht_hgeqz_eigs, paraht_hgeqz_eigs_d): the step
after the reduction, checked against LAPACK's DGGEV (scipy.linalg.eigvals) on the same pencils.

The reference's driver stops at the reduced pencil (src/profilereduction.f90:156); the eigenvalues
of (H, T) are those of the original pencil, so the reference's own check of a reduction is
available here too: the eigenvalues of the library's (H, T) against DGGEV of (A, B).
"""
import ctypes as C

import numpy as np
import pytest
import scipy.linalg as sla

from helpers import eig_mismatch, make

# Relative eigenvalue mismatch allowed against DGGEV.  T's diagonal is bounded away from zero, but
# the eigenvalues of random Hessenberg pencils still have condition numbers up to about 1e6 at
# these sizes: both sides are backward stable, and the largest difference seen is 1.35e-10 (one
# eigenvalue of a pencil of the batch test, n = 236, the same for the complex single-shift form).
TOL = 1e-9


def _pencil(n, seed, scale_t=1.0):
    rng = np.random.default_rng(seed)
    H = np.triu(rng.standard_normal((n, n)), -1)
    T = np.triu(rng.standard_normal((n, n))) * scale_t
    T[np.diag_indices(n)] = np.sign(T.diagonal() + 0.5) * (1.0 + np.abs(rng.standard_normal(n)))
    return np.asfortranarray(H), np.asfortranarray(T)


def _lam(alpha, beta):
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(beta == 0.0, np.inf, alpha / np.where(beta == 0.0, 1.0, beta))


def _pairs_exact(alpha):
    """Real eigenvalues with zero imaginary parts, complex ones as adjacent exact conjugate pairs
    (positive imaginary part first)."""
    j = 0
    while j < len(alpha):
        if alpha[j].imag == 0.0:
            j += 1
            continue
        if not (alpha[j].imag > 0.0 and j + 1 < len(alpha) and alpha[j + 1] == np.conj(alpha[j])):
            return False
        j += 2
    return True


def test_hgeqz_rejects_before_the_gpu():
    from paraht_gb300 import _lib

    L = _lib.lib()
    n = (C.c_int * 1)(4)
    ld = (C.c_int * 1)(4)
    P = C.c_void_p * 1
    info = (C.c_int * 1)()
    buf = (C.c_double * 16)()
    p = P(C.cast(buf, C.c_void_p))
    assert L.paraht_hgeqz_eigs(-1, n, p, ld, p, ld, p, p, p, info) == -2
    assert L.paraht_hgeqz_eigs(0, None, None, None, None, None, None, None, None, None) == 0
    assert L.paraht_hgeqz_eigs(1, None, p, ld, p, ld, p, p, p, info) == -3
    assert L.paraht_hgeqz_eigs(1, (C.c_int * 1)(-1), p, ld, p, ld, p, p, p, info) == -3
    assert L.paraht_hgeqz_eigs(1, n, P(None), ld, p, ld, p, p, p, info) == -4
    assert L.paraht_hgeqz_eigs(1, n, p, (C.c_int * 1)(3), p, ld, p, p, p, info) == -5
    assert L.paraht_hgeqz_eigs(1, n, p, ld, p, (C.c_int * 1)(2), p, p, p, info) == -7
    assert L.paraht_hgeqz_eigs(1, n, p, ld, p, ld, p, P(None), p, info) == -9
    assert L.paraht_hgeqz_eigs(1, n, p, ld, p, ld, p, p, p, None) == -11
    assert L.paraht_hgeqz_eigs_d(None, 1, n, p, ld, p, ld, p, p, p, info) == -1007


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 33, 64, 150, 257])
def test_hgeqz_against_dggev(n):
    import paraht_gb300 as ph

    H, T = _pencil(n, 100 + n)
    alpha, beta, info = ph.hgeqz_eigs(H, T)
    assert info == 0
    assert np.all(beta >= 0.0) and _pairs_exact(alpha)
    assert eig_mismatch(alpha / beta, sla.eigvals(H, T)) <= TOL


@pytest.mark.gpu
def test_hgeqz_complex_pairs_repeated_and_singular():
    import paraht_gb300 as ph

    # rotation blocks: eigenvalues k +- i k / 2 of a block diagonal pencil made Hessenberg by a
    # unit lower subdiagonal coupling of size 1e-3 (still complex pairs), plus a repeated
    # eigenvalue 2 (a Jordan-like 2 x 2) and a scaled T
    n = 12
    H = np.zeros((n, n))
    for k in range(0, 8, 2):
        a, b = 1.0 + k, 0.5 * (1.0 + k)
        H[k:k + 2, k:k + 2] = [[a, b], [-b, a]]
    H[8:10, 8:10] = [[2.0, 1.0], [0.0, 2.0]]
    H[10:, 10:] = [[-3.0, 0.25], [1e-3, 5.0]]
    for k in range(1, n):
        if H[k, k - 1] == 0.0:
            H[k, k - 1] = 1e-3
    T = np.diag(np.linspace(1.0, 2.0, n)) + np.triu(np.full((n, n), 0.1), 1)
    alpha, beta, info = ph.hgeqz_eigs(H, T)
    assert info == 0
    ref = sla.eigvals(H, T)
    assert eig_mismatch(alpha / beta, ref) <= 1e-7  # the near-Jordan pair is sensitive: O(sqrt(eps))
    assert _pairs_exact(alpha)
    # zeros on T's diagonal (top, inside, bottom): infinite eigenvalues, beta = 0, as many as
    # DGGEV finds, the finite ones matched
    Hs, Ts = _pencil(20, 7)
    Ts[[0, 5, 6, 19], [0, 5, 6, 19]] = 0.0
    a2, b2, info2 = ph.hgeqz_eigs(Hs, Ts)
    ref2 = sla.eigvals(Hs, Ts)
    assert info2 == 0 and int(np.sum(b2 == 0.0)) == int(np.sum(~np.isfinite(ref2))) > 0
    assert eig_mismatch(_lam(a2, b2), ref2) <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("sh,st", [(1e160, 1e160), (1e-160, 1e-160), (1e-300, 1e-300), (1e150, 1e-100),
                                   (1.0, 1e-200)])
def test_hgeqz_scaled_pencils(sh, st):
    """Pencils scaled toward the overflow and underflow thresholds (H by sh, T by st): the core
    scales both by powers of two first, so the eigenvalues (those of the unscaled pencil times
    sh / st) keep full accuracy.  Compared after dividing by the largest modulus."""
    import paraht_gb300 as ph

    H, T = _pencil(60, 77)
    alpha, beta, info = ph.hgeqz_eigs(H * sh, T * st)
    assert info == 0
    ref = sla.eigvals(H * sh, T * st)
    m = np.max(np.abs(ref))
    assert np.isfinite(m) and m > 0.0
    assert eig_mismatch((alpha / beta) / m, ref / m) <= TOL


@pytest.mark.gpu
def test_hgeqz_of_the_reduction_matches_dggev_of_the_pencil():
    """The eigenvalues of the library's reduced pencil against DGGEV of the original pencil (both
    precision paths), the whole pipeline reduction -> QZ on the GPU."""
    import paraht_gb300 as ph

    n = 300
    A, B = make(n, "std")
    A, B = np.asfortranarray(A), np.asfortranarray(np.triu(B))
    ref = sla.eigvals(A, B)
    for prec in ("fp64", "split"):
        H, T, _, _ = ph.ht(A.copy(order="F"), B.copy(order="F"), precision=prec)
        alpha, beta, info = ph.hgeqz_eigs(H, T)
        assert info == 0
        assert eig_mismatch(alpha / beta, ref) <= 1e-9, prec


@pytest.mark.gpu
def test_hgeqz_of_a_graded_reduction_is_backward_stable():
    """The library's reduction of a graded pencil (B with zero diagonal entries: infinite
    eigenvalues, finite ones up to about 1e12, too ill conditioned to compare): as many infinite
    eigenvalues as DGGEV finds in (H, T), and each eigenvalue's backward error
    sigma_min(beta H - alpha T) / (|beta| ||H|| + |alpha| ||T||) within a few eps."""
    import paraht_gb300 as ph

    A, B = make(150, "graded")
    A, B = np.asfortranarray(A), np.asfortranarray(np.triu(B))
    H, T, _, _ = ph.ht(A, B, precision="fp64")
    H, T = np.triu(H, -1), np.triu(T)
    alpha, beta, info = ph.hgeqz_eigs(H, T)
    assert info == 0 and np.any(beta == 0.0)
    assert int(np.sum(beta == 0.0)) == int(np.sum(~np.isfinite(sla.eigvals(H, T))))
    nh, nt = np.linalg.norm(H, 2), np.linalg.norm(T, 2)
    worst = max(np.linalg.svd(b * H - a * T, compute_uv=False)[-1] / (abs(b) * nh + abs(a) * nt)
                for a, b in zip(alpha, beta))
    assert worst <= 1e-14


@pytest.mark.gpu
def test_hgeqz_batched_device_entry_matches_host_entry():
    """A batch of 40 pencils of mixed sizes through the device entry (a warp per pencil below
    n = 128, a CTA per pencil from there) gives bitwise the host entry's results, pencil by pencil,
    and DGGEV's eigenvalues; two pencils carry zero diagonal entries of T."""
    torch = pytest.importorskip("torch")
    import paraht_gb300 as ph

    rng = np.random.default_rng(3)
    ns = [int(v) for v in rng.integers(1, 300, 40)]
    pens = [_pencil(n, 1000 + i) for i, n in enumerate(ns)]
    for k in (3, 17):  # infinite eigenvalues in the batch too
        pens[k][1][0, 0] = 0.0
        pens[k][1][ns[k] - 1, ns[k] - 1] = 0.0
    ctx = ph.Context()
    try:
        dH = [torch.from_numpy(np.ascontiguousarray(h.T)).cuda() for h, _ in pens]  # column-major
        dT = [torch.from_numpy(np.ascontiguousarray(t.T)).cuda() for _, t in pens]
        out = [torch.zeros(3, n, dtype=torch.float64, device="cuda") for n in ns]
        info = ctx.hgeqz_eigs_d(ns, [x.data_ptr() for x in dH], ns, [x.data_ptr() for x in dT], ns,
                                [o[0].data_ptr() for o in out], [o[1].data_ptr() for o in out],
                                [o[2].data_ptr() for o in out])
        assert info == [0] * len(ns)
        host = ph.hgeqz_eigs([h for h, _ in pens], [t for _, t in pens])
        for (h, t), o, (alpha, beta, inf) in zip(pens, out, host):
            ar, ai, be = o.cpu().numpy()
            assert inf == 0
            assert np.array_equal(ar, alpha.real) and np.array_equal(ai, alpha.imag) and np.array_equal(be, beta)
            assert eig_mismatch(_lam(ar + 1j * ai, be), sla.eigvals(h, t)) <= TOL
    finally:
        ctx.close()
