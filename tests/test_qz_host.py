"""The GPU QZ core (paraht_gb300/csrc/qz_real.cuh, real double shift) built for the host, no GPU:
against LAPACK's DGGEV (scipy.linalg.eigvals), with its lane-split loops run by 4 and 32 host
threads with a barrier for each lane synchronisation (tests/qz_host/qz_lanes.cpp), which must
give the one-lane results bitwise: every lane computes the same reflectors from the same values,
so a result that depends on the lane count means a missing synchronisation."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest
import scipy.linalg as sla

from helpers import eig_mismatch

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "paraht_gb300", "csrc")


def _cuda_include():
    for root in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        inc = os.path.join(root, "include")
        if root and os.path.exists(os.path.join(inc, "cuda_runtime.h")):
            return inc
    return None


@pytest.fixture(scope="module")
def qzlib(tmp_path_factory):
    gxx = shutil.which("g++")
    inc = _cuda_include()
    if not gxx or not inc:
        pytest.skip("g++ or the CUDA headers are missing")
    out = str(tmp_path_factory.mktemp("qz_host") / "libqz_lanes.so")
    cmd = [gxx, "-O2", "-std=c++20", "-shared", "-fPIC", "-I", CSRC, "-I", inc,
           os.path.join(HERE, "qz_host", "qz_lanes.cpp"), "-o", out, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(out)
    lib.qzr_lanes.argtypes = [C.c_int, C.c_int] + [C.c_void_p, C.c_int] * 2 + [C.c_void_p] * 3
    return lib


def _pencil(n, seed):
    rng = np.random.default_rng(seed)
    H = np.triu(rng.standard_normal((n, n)), -1)
    T = np.triu(rng.standard_normal((n, n)))
    T[np.diag_indices(n)] = np.sign(T.diagonal() + 0.5) * (1.0 + np.abs(rng.standard_normal(n)))
    return np.asfortranarray(H), np.asfortranarray(T)


def _eigs(lib, nlanes, H, T):
    n = H.shape[0]
    H, T = np.asfortranarray(H, dtype=np.float64), np.asfortranarray(T, dtype=np.float64)
    ar, ai, be = np.zeros(n), np.zeros(n), np.zeros(n)
    rc = lib.qzr_lanes(nlanes, n, H.ctypes.data, max(1, n), T.ctypes.data, max(1, n), ar.ctypes.data,
                      ai.ctypes.data, be.ctypes.data)
    return rc, ar, ai, be


def _lam(ar, ai, be):
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(be == 0.0, np.inf, (ar + 1j * ai) / np.where(be == 0.0, 1.0, be))


def _pairs_exact(ar, ai):
    """Real eigenvalues with zero imaginary parts, complex ones as adjacent exact conjugate pairs
    (positive imaginary part first)."""
    j = 0
    while j < len(ar):
        if ai[j] == 0.0:
            j += 1
            continue
        if not (ai[j] > 0.0 and j + 1 < len(ar) and ai[j + 1] == -ai[j] and ar[j + 1] == ar[j]):
            return False
        j += 2
    return True


@pytest.mark.timeout(300)
@pytest.mark.parametrize("n", [0, 1, 2, 3, 4, 9, 40, 120, 257])
def test_real_qz_core_against_dggev(qzlib, n):
    H, T = _pencil(n, 300 + n)
    rc, ar, ai, be = _eigs(qzlib, 1, H, T)
    assert rc == 0
    if n:
        assert np.all(be >= 0.0) and _pairs_exact(ar, ai)
        assert eig_mismatch(_lam(ar, ai, be), sla.eigvals(H, T)) <= 1e-10


@pytest.mark.timeout(300)
@pytest.mark.parametrize("nlanes,n", [(4, 37), (4, 70), (32, 65)])
def test_real_qz_lane_split_matches_one_lane_bitwise(qzlib, nlanes, n):
    H, T = _pencil(n, 900 + n)
    T[[0, n // 3, n // 3 + 1, n - 1], [0, n // 3, n // 3 + 1, n - 1]] = 0.0  # the zero chase too
    one = _eigs(qzlib, 1, H, T)
    many = _eigs(qzlib, nlanes, H, T)
    assert one[0] == 0 and many[0] == 0
    for a, b in zip(one[1:], many[1:]):
        assert np.array_equal(a, b)


@pytest.mark.timeout(300)
@pytest.mark.parametrize("zeros", [[0], [5], [19], [0, 1], [3, 4], [18, 19], [0, 7, 19], [2, 9, 10, 11]])
def test_real_qz_infinite_eigenvalues(qzlib, zeros):
    """Zero diagonal entries of T at the top, inside and at the bottom, alone and adjacent: as many
    infinite eigenvalues (beta = 0) as DGGEV finds, and the finite ones matched."""
    H, T = _pencil(20, 55)
    T[zeros, zeros] = 0.0
    rc, ar, ai, be = _eigs(qzlib, 4, H, T)
    assert rc == 0
    ref = sla.eigvals(H, T)
    assert int(np.sum(be == 0.0)) == int(np.sum(~np.isfinite(ref)))
    assert eig_mismatch(_lam(ar, ai, be), ref) <= 1e-10


@pytest.mark.timeout(300)
@pytest.mark.parametrize("sh,st", [(1e160, 1e160), (1e-300, 1e-300), (1e150, 1e-100)])
def test_real_qz_scaled_pencils(qzlib, sh, st):
    H, T = _pencil(40, 77)
    rc, ar, ai, be = _eigs(qzlib, 4, H * sh, T * st)
    assert rc == 0
    ref = sla.eigvals(H * sh, T * st)
    m = np.max(np.abs(ref))
    assert eig_mismatch(_lam(ar, ai, be) / m, ref / m) <= 1e-10


@pytest.mark.timeout(300)
def test_real_qz_graded_reduced_pencil_backward_stable(qzlib, oracle):
    """The oracle's reduction of a graded pencil (B with zero diagonal entries, eigenvalues up to
    about 1e12 and infinite ones): the eigenvalues are too ill conditioned to compare, so each is
    checked by its backward error sigma_min(beta H - alpha T) / (|beta| ||H|| + |alpha| ||T||),
    within a few eps like LAPACK DHGEQZ's on the same pencil."""
    from helpers import make, oracle_reduce

    A0, B0 = make(150, "graded")
    A0, B0 = np.asfortranarray(A0), np.asfortranarray(np.triu(B0))
    Ao, Bo, _, _ = oracle_reduce(oracle, A0, B0, 8, 4, 8)
    H, T = np.asfortranarray(np.triu(Ao, -1)), np.asfortranarray(np.triu(Bo))
    rc, ar, ai, be = _eigs(qzlib, 4, H, T)
    assert rc == 0 and np.any(be == 0.0)
    assert int(np.sum(be == 0.0)) == int(np.sum(~np.isfinite(sla.eigvals(H, T))))
    nh, nt = np.linalg.norm(H, 2), np.linalg.norm(T, 2)
    worst = max(np.linalg.svd(b * H - a * T, compute_uv=False)[-1] / (abs(b) * nh + abs(a) * nt)
                for a, b in zip(ar + 1j * ai, be))
    assert worst <= 1e-14


@pytest.mark.timeout(600)
def test_real_qz_randomized_backward_stability(qzlib):
    """Seeded random pencils of mixed structure (sizes 1-60; zero diagonal entries of T at random
    places; exact zeros on H's subdiagonal; H and T scaled by powers of ten between 1e-100 and
    1e100; 1 or 4 lanes): every eigenvalue's backward error
    sigma_min(beta H - alpha T) / (|beta| ||H|| + |alpha| ||T||) within a few eps, and beta >= 0,
    real eigenvalues or exact conjugate pairs."""
    rng = np.random.default_rng(2024)
    worst, where = 0.0, None
    for case in range(100):
        n = int(rng.integers(1, 61))
        H, T = _pencil(n, 5000 + case)
        if n > 1 and case % 3 == 0:
            z = rng.integers(0, n, int(rng.integers(1, 4)))
            T[z, z] = 0.0
        if n > 2 and case % 4 == 1:
            k = int(rng.integers(1, n))
            H[k, k - 1] = 0.0
        H, T = H * 10.0 ** rng.integers(-100, 101), T * 10.0 ** rng.integers(-100, 101)
        rc, ar, ai, be = _eigs(qzlib, (1, 4)[case % 2], H, T)
        assert rc == 0, case
        assert np.all(be >= 0.0) and _pairs_exact(ar, ai), case
        nh, nt = np.linalg.norm(H, 2), np.linalg.norm(T, 2)
        for a, b in zip(ar + 1j * ai, be):
            bb, aa = b * nh, a * nt  # the pair for the normalised pencil (H / nh, T / nt)
            sc = max(abs(bb), abs(aa))
            sv = np.linalg.svd((bb / sc) * (H / nh) - (aa / sc) * (T / nt), compute_uv=False)[-1]
            err = sv * sc / (abs(bb) + abs(aa))
            if err > worst:
                worst, where = err, case
    assert worst <= 1e-14, (worst, where)
    print("worst backward error %.2e (case %s)" % (worst, where))
