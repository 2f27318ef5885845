"""profilereduction -- command-line driver with the reference's argv and report line.

    python -m paraht_gb300.profilereduction n algorithm [r p nq time_components] [--dist D] [--seed S]

Mirrors src/profilereduction.f90: algorithm 1 runs the two-stage reduction (on the GPU through
libparaht), algorithm 2 runs LAPACK DGGHD3('V','V',n,1,n,...) on the host (:156).  The input
pencil is generated with the library's seeded generator (default: the reference's recipe,
U[0,1) entries and B <- R of QR(B), seed 1302; the gfortran random stream itself cannot be
reproduced).  The timed region covers only the reduction (:134-160); the backward errors
||Q^T A0 Z - H||_F/||A0||_F and ||Q^T B0 Z - T||_F/||B0||_F are computed afterwards (:165-174)
and the same line as the reference is printed (:178-184).
"""
from __future__ import annotations

import argparse
import ctypes as C
import glob
import os
import sys
import time

import numpy as np


def _lapack_dgghd3():
    """DGGHD3 from the OpenBLAS bundled with scipy (profilereduction's LAPACK baseline, algorithm 2)."""
    import scipy

    base = os.path.dirname(os.path.dirname(scipy.__file__))
    libs = [p for p in glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")) if "64_" not in p]
    if not libs:
        raise RuntimeError("no LAPACK found for algorithm 2")
    L = C.CDLL(libs[0])
    f = getattr(L, "scipy_dgghd3_", None) or getattr(L, "dgghd3_")
    f.restype = None
    return f


def dgghd3(A, B, Q, Z):
    f = _lapack_dgghd3()
    n = A.shape[0]
    ci = lambda v: C.byref(C.c_int(v))  # noqa: E731
    p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    info = C.c_int(0)
    q = np.zeros(1)
    args = [C.c_char_p(b"V"), C.c_char_p(b"V"), ci(n), ci(1), ci(n), p(A), ci(n), p(B), ci(n), p(Q), ci(n), p(Z), ci(n)]
    f(*args, p(q), ci(-1), C.byref(info), C.c_size_t(1), C.c_size_t(1))
    work = np.zeros(max(1, int(q[0])))
    f(*args, p(work), ci(work.size), C.byref(info), C.c_size_t(1), C.c_size_t(1))
    return info.value


def backward_errors(Q, A0, Z, A, B0, B):
    try:
        import torch

        if torch.cuda.is_available():
            t = lambda X: torch.from_numpy(np.ascontiguousarray(X)).cuda()  # noqa: E731
            Qd, Zd = t(Q), t(Z)
            ea = torch.linalg.norm(Qd.T @ t(A0) @ Zd - t(A)) / torch.linalg.norm(t(A0))
            eb = torch.linalg.norm(Qd.T @ t(B0) @ Zd - t(B)) / torch.linalg.norm(t(B0))
            return float(ea), float(eb)
    except ImportError:
        pass
    ea = np.linalg.norm(Q.T @ A0 @ Z - A) / np.linalg.norm(A0)
    eb = np.linalg.norm(Q.T @ B0 @ Z - B) / np.linalg.norm(B0)
    return float(ea), float(eb)


def main(argv=None):
    ap = argparse.ArgumentParser(usage="profilereduction n algorithm (r p nq time_components)")
    ap.add_argument("n", type=int)
    ap.add_argument("algorithm", type=int)
    ap.add_argument("rest", type=int, nargs="*")
    ap.add_argument("--dist", default="refcompat")
    ap.add_argument("--seed", type=int, default=1302)
    a = ap.parse_args(argv)
    n, alg = a.n, a.algorithm
    if alg == 1 and len(a.rest) < 3:
        print(" if using ParaHT, you should supply the parameters r, p and nq")  # profilereduction.f90:49
        return 0
    from .generate import identity, pencil

    A0, B0 = pencil(n, a.dist, seed=a.seed)
    A, B, Q, Z = A0.copy(order="F"), B0.copy(order="F"), identity(n), identity(n)
    if alg == 1:
        import paraht_gb300 as ph

        r, p, nq = a.rest[:3]
        tc = len(a.rest) >= 4 and a.rest[3] == 1
        t0 = time.perf_counter()
        ph.ab2rht_simple(n, A, n, B, n, Q, n, Z, n, r, p, tc)
        t1 = time.perf_counter()
        ph.rht2ht_householder(n, A, n, B, n, Q, n, Z, n, r, nq, tc)
        t2 = time.perf_counter()
        rht, ht = t1 - t0, t2 - t1
        total = rht + ht
    elif alg == 2:
        t0 = time.perf_counter()
        dgghd3(A, B, Q, Z)
        total = time.perf_counter() - t0
    else:
        print("algorithm must be 1 (ParaHT) or 2 (LAPACK)")
        return 1
    ea, eb = backward_errors(Q, A0, Z, A, B0, B)
    if alg == 1:
        print("n:%6d ;runtime:%16.6f ;error:%16.6E%16.6E ;phase 1 time:%16.6f ;phase 2 time:%16.6f ;r:%4d ;p:%4d ;nq:%4d"
              % (n, total, ea, eb, rht, ht, r, p, nq))
    else:
        print("n:%6d ;runtime:%16.6f ;error:%16.6E%16.6E" % (n, total, ea, eb))
    return 0


if __name__ == "__main__":
    sys.exit(main())
