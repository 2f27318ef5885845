"""The GPU QZ core (paraht_gb300/csrc/qz.cuh) built for the host, no GPU: the algorithm against
LAPACK's DGGEV (scipy.linalg.eigvals), and its lane-split loops run by 4 and 32 host threads with
a barrier for each lane synchronisation (tests/qz_host/qz_lanes.cpp), which must give the
one-lane results bitwise: every lane computes the same rotations from the same values, so a
result that depends on the lane count means a missing synchronisation."""
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
    lib.qz_lanes.argtypes = [C.c_int, C.c_int] + [C.c_void_p, C.c_int] * 2 + [C.c_void_p] * 3
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
    rc = lib.qz_lanes(nlanes, n, H.ctypes.data, max(1, n), T.ctypes.data, max(1, n), ar.ctypes.data,
                      ai.ctypes.data, be.ctypes.data)
    return rc, ar, ai, be


@pytest.mark.timeout(300)
@pytest.mark.parametrize("n", [0, 1, 2, 3, 9, 40, 120])
def test_qz_core_against_dggev(qzlib, n):
    H, T = _pencil(n, 300 + n)
    rc, ar, ai, be = _eigs(qzlib, 1, H, T)
    assert rc == 0
    if n:
        assert np.all(be >= 0.0)
        assert eig_mismatch((ar + 1j * ai) / be, sla.eigvals(H, T)) <= 1e-10


@pytest.mark.timeout(300)
@pytest.mark.parametrize("nlanes,n", [(4, 37), (4, 70), (32, 24)])
def test_qz_lane_split_matches_one_lane_bitwise(qzlib, nlanes, n):
    H, T = _pencil(n, 700 + n)
    one = _eigs(qzlib, 1, H, T)
    many = _eigs(qzlib, nlanes, H, T)
    assert one[0] == 0 and many[0] == 0
    for a, b in zip(one[1:], many[1:]):
        assert np.array_equal(a, b)


@pytest.mark.timeout(300)
@pytest.mark.parametrize("sh,st", [(1e160, 1e160), (1e-300, 1e-300), (1e150, 1e-100)])
def test_qz_core_scaled_pencils(qzlib, sh, st):
    H, T = _pencil(40, 77)
    rc, ar, ai, be = _eigs(qzlib, 4, H * sh, T * st)
    assert rc == 0
    ref = sla.eigvals(H * sh, T * st)
    m = np.max(np.abs(ref))
    assert eig_mismatch(((ar + 1j * ai) / be) / m, ref / m) <= 1e-10


@pytest.mark.timeout(300)
def test_qz_core_reports_singular_t(qzlib):
    H, T = _pencil(20, 7)
    T[5, 5] = 0.0
    assert _eigs(qzlib, 4, H, T)[0] == 1
