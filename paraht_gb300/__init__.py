"""paraht_gb300 -- GB300-native two-stage Hessenberg-triangular reduction of a pencil (A, B).

Python mirror of the reference's Fortran interface (same names, argument order and meaning):

* ``ab2rht_simple(n, A, lda, B, ldb, Q, ldq, Z, ldz, nb, p, time_components)``
      src/ab2rht.f90:8 -- stage 1, (A, B) -> (r-Hessenberg, triangular)
* ``rht2ht_householder(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq, time_components)``
      src/rht2ht.f90:1346 -- stage 2, r-Hessenberg -> Hessenberg
* ``rht2ht_givens(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq)``
      src/rht2ht.f90:696 -- stage 2 with Givens rotations (the reference's other stage-2 variant)

Arrays are numpy float64 in Fortran (column-major) order and are overwritten in place; Q and Z
are accumulated (right-multiplied), as in the reference.  The work runs on the GPU through
libparaht.so (C ABI in include/paraht.h); there is no CPU path.  Invalid arguments raise
``ParahtError`` carrying the LAPACK-style negative argument index instead of silently
producing garbage (the reference performs no checks).

``Context`` exposes the device-pointer entry points (arrays resident in GPU memory), per-phase
timings and the fill residue.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (PARAHT_BATCH_MAX_N, PARAHT_FLAG_BATCH_LOOP, PARAHT_FLAG_CHECK_FINITE, PARAHT_FLAG_GIVENS,
                   PARAHT_FLAG_KERNEL_TIMES, PARAHT_FLAG_NO_ZERO_FILL, PARAHT_FLAG_SEQUENTIAL, PARAHT_FLAG_SPLIT,
                   PARAHT_FLAG_TIME_CHAIN, PARAHT_FLAG_TIME_COMPONENTS, ParahtError, check, lib)

__all__ = [
    "ab2rht_simple", "rht2ht_householder", "rht2ht_givens", "reduce", "ht", "gghd3", "hgeqz_eigs", "Context",
    "BatchPlan",
    "ParahtError",
    "PARAHT_FLAG_TIME_COMPONENTS", "PARAHT_FLAG_CHECK_FINITE", "PARAHT_FLAG_SPLIT", "PARAHT_FLAG_NO_ZERO_FILL",
    "PARAHT_FLAG_SEQUENTIAL", "PARAHT_FLAG_KERNEL_TIMES", "PARAHT_FLAG_BATCH_LOOP", "PARAHT_FLAG_GIVENS",
    "PARAHT_FLAG_TIME_CHAIN",
    "PARAHT_BATCH_MAX_N",
]

PHASE_NAMES = ("s1_genleft", "s1_genright", "s1_mul", "s2_gen", "s2_lookahead", "s2_application", "copies", "total")


def _host_ptr(a):
    if a is None:
        return None
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.f_contiguous:
        raise TypeError("matrices must be Fortran-ordered float64 numpy arrays")
    if not a.flags.writeable:
        raise TypeError("matrices are overwritten in place and must be writeable")
    return a.ctypes.data


def ab2rht_simple(n, A, lda, B, ldb, Q, ldq, Z, ldz, nb, p, time_components=False):
    """Stage 1 (src/ab2rht.f90:8-13), in place on host arrays."""
    check(lib().paraht_ab2rht(int(n), _host_ptr(A), int(lda), _host_ptr(B), int(ldb), _host_ptr(Q), int(ldq),
                              _host_ptr(Z), int(ldz), int(nb), int(p), int(bool(time_components))), "ab2rht_simple")


def rht2ht_householder(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq, time_components=False):
    """Stage 2 (src/rht2ht.f90:1346-1351), in place on host arrays."""
    check(lib().paraht_rht2ht(int(n), _host_ptr(A), int(lda), _host_ptr(B), int(ldb), _host_ptr(Q), int(ldq),
                              _host_ptr(Z), int(ldz), int(r), int(nq), int(bool(time_components))),
          "rht2ht_householder")


def rht2ht_givens(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq):
    """Stage 2 with Givens rotations (src/rht2ht.f90:696-700), in place on host arrays; the same
    H, T as rht2ht_householder up to row/column signs.  Needs r <= 32 and r + nq <= 64."""
    check(lib().paraht_rht2ht_givens(int(n), _host_ptr(A), int(lda), _host_ptr(B), int(ldb), _host_ptr(Q), int(ldq),
                                     _host_ptr(Z), int(ldz), int(r), int(nq)), "rht2ht_givens")


def reduce(A, B, Q, Z, r, p, nq, flags=0):
    """Both stages in sequence (src/profilereduction.f90:136, :144) on host arrays."""
    n = A.shape[0]
    check(lib().paraht_reduce(int(n), _host_ptr(A), A.shape[0], _host_ptr(B), B.shape[0], _host_ptr(Q), Q.shape[0],
                              _host_ptr(Z), Z.shape[0], int(r), int(p), int(nq), int(flags)), "reduce")


def ht(A, B, precision="split", params=None):
    """Hessenberg-triangular form of the pencil (A, B), B upper triangular, as new arrays:
    returns (H, T, Q, Z) with H = Q^T A Z upper Hessenberg and T = Q^T B Z upper triangular.
    `precision` "split" (split-precision bulk updates) or "fp64"; `params` (r, p, nq) or None for
    the autotuner's choice for this size (paraht_gb300.tune), which also picks the stage-2 variant
    (Givens rotations or small reflectors) measured faster for the precision.  Inputs are not
    modified."""
    from . import tune

    if precision not in ("split", "fp64"):
        raise ValueError("precision must be 'split' or 'fp64'")
    H = np.array(A, dtype=np.float64, order="F", copy=True)
    T = np.array(B, dtype=np.float64, order="F", copy=True)
    n = H.shape[0]
    if H.shape != (n, n) or T.shape != (n, n):
        raise ValueError("A and B must be square and of the same size")
    if n > 1 and np.any(np.tril(T, -1) != 0.0):
        # the reduction assumes it, as the reference's ab2rht_simple does (src/profilereduction.f90:117-123
        # triangularises B before the call); a general B would give a wrong (H, T, Q, Z) silently
        raise ValueError("B must be upper triangular (triangularise it first, e.g. by a QR factorisation, "
                         "and apply the orthogonal factor's transpose to A)")
    Q = np.asfortranarray(np.eye(n))
    Z = np.asfortranarray(np.eye(n))
    if n == 0:
        return H, T, Q, Z
    r, p, nq = params if params is not None else tune.pick(n, precision)
    flags = PARAHT_FLAG_SPLIT if precision == "split" else 0
    if tune.stage2(precision, r, nq) == "givens":
        flags |= PARAHT_FLAG_GIVENS
    reduce(H, T, Q, Z, r, p, nq, flags)
    return H, T, Q, Z


def gghd3(compq, compz, ilo, ihi, A, B, Q, Z, r=16, p=4, nq=16, flags=0):
    """LAPACK DGGHD3-compatible reduction of rows/columns ilo..ihi (1-based) on host arrays, in
    place: compq/compz 'N' (Q/Z not referenced, may be None), 'I' (identity first) or 'V'
    (accumulated).  No counterpart in the reference (which ignores ilo/ihi)."""
    n = A.shape[0]
    check(lib().paraht_gghd3(compq.encode(), compz.encode(), int(n), int(ilo), int(ihi), _host_ptr(A), A.shape[0],
                             _host_ptr(B), B.shape[0], _host_ptr(Q), Q.shape[0] if Q is not None else 1,
                             _host_ptr(Z), Z.shape[0] if Z is not None else 1, int(r), int(p), int(nq), int(flags)),
          "gghd3")


def hgeqz_eigs(H, T):
    """Generalized eigenvalues of Hessenberg-triangular pencils by the real double-shift QZ
    iteration on the GPU (LAPACK DHGEQZ with JOB='E'; paraht_hgeqz_eigs), the step after the
    reduction.  H, T: one pair of float64 arrays (H upper Hessenberg, T upper triangular; entries
    below ignored) or two lists of them, reduced together.  Returns (alpha, beta, info) for one
    pair, else a list of them: alpha complex (real eigenvalues with zero imaginary part, complex
    ones as adjacent conjugate pairs), beta real >= 0, eigenvalue alpha / beta (infinite where
    beta = 0); info 2 (no convergence) leaves alpha and beta None."""
    single = not isinstance(H, (list, tuple))
    Hs = [np.asfortranarray(h, dtype=np.float64) for h in ([H] if single else H)]
    Ts = [np.asfortranarray(t, dtype=np.float64) for t in ([T] if single else T)]
    if len(Hs) != len(Ts) or any(h.ndim != 2 or h.shape[0] != h.shape[1] or h.shape != t.shape
                                 for h, t in zip(Hs, Ts)):
        raise ValueError("H and T must be square arrays of equal shapes")
    cnt = len(Hs)
    ns = [h.shape[0] for h in Hs]
    ar, ai, be = ([np.zeros(n) for n in ns] for _ in range(3))
    info = (C.c_int * cnt)()
    IA, PA = C.c_int * cnt, C.c_void_p * cnt
    lds = IA(*[max(1, n) for n in ns])
    check(lib().paraht_hgeqz_eigs(cnt, IA(*ns), PA(*[h.ctypes.data for h in Hs]), lds,
                                  PA(*[t.ctypes.data for t in Ts]), lds, PA(*[a.ctypes.data for a in ar]),
                                  PA(*[a.ctypes.data for a in ai]), PA(*[b.ctypes.data for b in be]), info),
          "hgeqz_eigs")
    out = [(ar[i] + 1j * ai[i], be[i], 0) if info[i] == 0 else (None, None, int(info[i])) for i in range(cnt)]
    return out[0] if single else out


class Context:
    """A libparaht context: one CUDA device, one stream, reusable workspace."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        check(lib().paraht_ctx_create(C.byref(self._h), int(device)), "paraht_ctx_create")

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().paraht_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int):
        check(lib().paraht_ctx_set_stream(self._h, C.c_void_p(stream_ptr or None)), "set_stream")

    # -- device pointers (ints, e.g. torch.Tensor.data_ptr()) --
    def reduce_d(self, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, p, nq, flags=0):
        check(lib().paraht_reduce_d(self._h, int(n), A, int(lda), B, int(ldb), Q, int(ldq), Z, int(ldz), int(r),
                                    int(p), int(nq), int(flags)), "reduce_d")

    def ab2rht_d(self, n, A, lda, B, ldb, Q, ldq, Z, ldz, nb, p, flags=0):
        check(lib().paraht_ab2rht_d(self._h, int(n), A, int(lda), B, int(ldb), Q, int(ldq), Z, int(ldz), int(nb),
                                    int(p), int(flags)), "ab2rht_d")

    def rht2ht_d(self, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq, flags=0):
        check(lib().paraht_rht2ht_d(self._h, int(n), A, int(lda), B, int(ldb), Q, int(ldq), Z, int(ldz), int(r),
                                    int(nq), int(flags)), "rht2ht_d")

    def kernel_stats(self):
        """Split-precision op-list kernel statistics of the last call made with
        PARAHT_FLAG_KERNEL_TIMES: per stage, summed launch seconds, launches and algorithmic
        FP64-equivalent flops."""
        out = (C.c_double * 8)()
        check(lib().paraht_ctx_kernel_stats(self._h, out, 8), "kernel_stats")
        return {"stage1": {"seconds": out[0], "launches": int(out[1]), "flops": out[2], "busy_seconds": out[6]},
                "stage2": {"seconds": out[3], "launches": int(out[4]), "flops": out[5], "busy_seconds": out[7]}}

    def rht2ht_d_noalloc(self, n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq, flags=0):
        """paraht_rht2ht_d with the scratch in a fixed device array (no allocation; calls that
        overlap in time on one device race)."""
        check(lib().paraht_rht2ht_d_noalloc(self._h, int(n), A, int(lda), B, int(ldb), Q, int(ldq), Z, int(ldz),
                                            int(r), int(nq), int(flags)), "rht2ht_d_noalloc")

    # -- host arrays on this context --
    def reduce_host(self, A, B, Q, Z, r, p, nq, flags=0):
        n = A.shape[0]
        check(lib().paraht_reduce_host(self._h, int(n), _host_ptr(A), A.shape[0], _host_ptr(B), B.shape[0],
                                       _host_ptr(Q), Q.shape[0], _host_ptr(Z), Z.shape[0], int(r), int(p), int(nq),
                                       int(flags)), "reduce_host")

    def reduce_batched_d(self, ns, As, ldas, Bs, ldbs, Qs, ldqs, Zs, ldzs, rs, ps, nqs, flags=0):
        cnt = len(ns)
        IA = C.c_int * cnt
        PA = C.c_void_p * cnt
        check(lib().paraht_reduce_batched_d(self._h, cnt, IA(*ns), PA(*As), IA(*ldas), PA(*Bs), IA(*ldbs), PA(*Qs),
                                            IA(*ldqs), PA(*Zs), IA(*ldzs), IA(*rs), IA(*ps), IA(*nqs), int(flags)),
              "reduce_batched_d")

    def batch_plan(self, ns, As, ldas, Bs, ldbs, Qs, ldqs, Zs, ldzs, rs, ps, nqs, flags=0):
        """A BatchPlan: the persistent batched launch for these pencils captured as a CUDA graph
        (paraht_batch_plan_create); replay it with .launch(stream)."""
        return BatchPlan(self, ns, As, ldas, Bs, ldbs, Qs, ldqs, Zs, ldzs, rs, ps, nqs, flags)

    def hgeqz_eigs_d(self, ns, Hs, ldhs, Ts, ldts, alphars, alphais, betas):
        """QZ eigenvalues of Hessenberg-triangular pencils in device memory (paraht_hgeqz_eigs_d);
        returns the per-pencil info list (0, or 2 for no convergence)."""
        cnt = len(ns)
        IA, PA = C.c_int * cnt, C.c_void_p * cnt
        info = IA()
        check(lib().paraht_hgeqz_eigs_d(self._h, cnt, IA(*ns), PA(*Hs), IA(*ldhs), PA(*Ts), IA(*ldts), PA(*alphars),
                                        PA(*alphais), PA(*betas), info), "hgeqz_eigs_d")
        return [int(v) for v in info]

    def selftest_wait_timeout(self, spin_limit: int = 1000) -> int:
        """Runs the chase's bounded wait on a flag nothing sets; returns the reported status
        (PARAHT_ERR_TIMEOUT, -1003, when the failure path works)."""
        return int(lib().paraht_selftest_wait_timeout(self._h, int(spin_limit)))

    def selftest_reflector(self, count: int, alpha_ptr: int, xnorm2_ptr: int, out_ptr: int) -> None:
        """Reflector scalars (tau, scal, beta per entry) of the generation chains' branch-free
        formula for device arrays alpha, xnorm2 (paraht_selftest_reflector)."""
        check(lib().paraht_selftest_reflector(self._h, int(count), alpha_ptr, xnorm2_ptr, out_ptr), "selftest_reflector")

    def phase_times(self) -> dict:
        buf = (C.c_double * 8)()
        check(lib().paraht_ctx_phase_times(self._h, buf, 8), "phase_times")
        return dict(zip(PHASE_NAMES, list(buf)))

    def launch_count(self) -> int:
        v = C.c_longlong()
        check(lib().paraht_ctx_launch_count(self._h, C.byref(v)), "launch_count")
        return int(v.value)

    def fill_residue(self):
        buf = (C.c_double * 2)()
        check(lib().paraht_ctx_fill_residue(self._h, buf, 2), "fill_residue")
        return float(buf[0]), float(buf[1])


class BatchPlan:
    """A fixed set of pencils reduced by replaying a CUDA graph (paraht_batch_plan_*)."""

    def __init__(self, ctx, ns, As, ldas, Bs, ldbs, Qs, ldqs, Zs, ldzs, rs, ps, nqs, flags=0):
        cnt = len(ns)
        IA = C.c_int * cnt
        PA = C.c_void_p * cnt
        self._h = C.c_void_p()
        self._ctx = ctx  # the plan's launches use the context's device
        check(lib().paraht_batch_plan_create(ctx.handle, cnt, IA(*ns), PA(*As), IA(*ldas), PA(*Bs), IA(*ldbs),
                                             PA(*Qs), IA(*ldqs), PA(*Zs), IA(*ldzs), IA(*rs), IA(*ps), IA(*nqs),
                                             int(flags), C.byref(self._h)), "paraht_batch_plan_create")

    def launch(self, stream_ptr: int = 0):
        check(lib().paraht_batch_plan_launch(self._h, C.c_void_p(stream_ptr or None)), "paraht_batch_plan_launch")

    def close(self):
        if self._h:
            lib().paraht_batch_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
