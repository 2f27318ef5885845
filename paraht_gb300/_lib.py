"""ctypes binding of libparaht.so (the C ABI in include/paraht.h).

There is no fallback: if the native library is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libparaht.so")

PARAHT_FLAG_TIME_COMPONENTS = 1
PARAHT_FLAG_CHECK_FINITE = 2
PARAHT_FLAG_SPLIT = 4
PARAHT_FLAG_NO_ZERO_FILL = 8
PARAHT_FLAG_SEQUENTIAL = 16
PARAHT_FLAG_KERNEL_TIMES = 32
PARAHT_FLAG_BATCH_LOOP = 64
PARAHT_FLAG_GIVENS = 128
PARAHT_FLAG_TIME_CHAIN = 256
PARAHT_BATCH_MAX_N = 1024

ERRORS = {
    -1001: "PARAHT_ERR_CUDA",
    -1002: "PARAHT_ERR_ALLOC",
    -1003: "PARAHT_ERR_TIMEOUT",
    -1004: "PARAHT_ERR_NONFINITE",
    -1005: "PARAHT_ERR_NOT_SUPPORTED",
    -1006: "PARAHT_ERR_NO_DEVICE",
    -1007: "PARAHT_ERR_BAD_CTX",
    -1008: "PARAHT_ERR_TOO_LARGE",
}

# (name, argtypes) for every exported entry point; the tests check this list against the header.
_d = C.c_void_p  # double* (host or device address)
_i = C.c_int
SIGNATURES = {
    "paraht_ctx_create": [C.POINTER(C.c_void_p), _i],
    "paraht_ctx_destroy": [C.c_void_p],
    "paraht_ctx_set_stream": [C.c_void_p, C.c_void_p],
    "paraht_ctx_phase_times": [C.c_void_p, C.POINTER(C.c_double), _i],
    "paraht_ctx_fill_residue": [C.c_void_p, C.POINTER(C.c_double), _i],
    "paraht_ctx_launch_count": [C.c_void_p, C.POINTER(C.c_longlong)],
    "paraht_ab2rht": [_i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i, _i],
    "paraht_rht2ht": [_i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i, _i],
    "paraht_reduce": [_i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i, _i, _i],
    "paraht_rht2ht_givens": [_i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i],
    "paraht_reduce_host": [C.c_void_p, _i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i, _i, _i],
    "paraht_ab2rht_d": [C.c_void_p, _i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i, _i],
    "paraht_rht2ht_d": [C.c_void_p, _i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i, _i],
    "paraht_reduce_d": [C.c_void_p, _i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i, _i, _i],
    "paraht_ctx_kernel_stats": [C.c_void_p, C.POINTER(C.c_double), _i],
    "paraht_rht2ht_d_noalloc": [C.c_void_p, _i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i, _i],
    "paraht_reduce_batched_d": [C.c_void_p, _i, C.POINTER(_i), C.POINTER(_d), C.POINTER(_i), C.POINTER(_d),
                                C.POINTER(_i), C.POINTER(_d), C.POINTER(_i), C.POINTER(_d), C.POINTER(_i),
                                C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), _i],
    "paraht_batch_plan_create": [C.c_void_p, _i, C.POINTER(_i), C.POINTER(_d), C.POINTER(_i), C.POINTER(_d),
                                 C.POINTER(_i), C.POINTER(_d), C.POINTER(_i), C.POINTER(_d), C.POINTER(_i),
                                 C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), _i, C.POINTER(C.c_void_p)],
    "paraht_batch_plan_launch": [C.c_void_p, C.c_void_p],
    "paraht_batch_plan_destroy": [C.c_void_p],
    "paraht_gghd3": [C.c_char, C.c_char, _i, _i, _i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i, _i, _i],
    "paraht_gghd3_d": [C.c_void_p, C.c_char, C.c_char, _i, _i, _i, _d, _i, _d, _i, _d, _i, _d, _i, _i, _i, _i, _i],
    "paraht_hgeqz_eigs_d": [C.c_void_p, _i, C.POINTER(_i), C.POINTER(_d), C.POINTER(_i), C.POINTER(_d),
                            C.POINTER(_i), C.POINTER(_d), C.POINTER(_d), C.POINTER(_d), C.POINTER(_i)],
    "paraht_hgeqz_eigs": [_i, C.POINTER(_i), C.POINTER(_d), C.POINTER(_i), C.POINTER(_d), C.POINTER(_i),
                          C.POINTER(_d), C.POINTER(_d), C.POINTER(_d), C.POINTER(_i)],
    "paraht_selftest_wait_timeout": [C.c_void_p, C.c_longlong],
    "paraht_selftest_reflector": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p],
    "paraht_strerror": [_i],
    "paraht_version": [],
}

_lib = None


class ParahtError(RuntimeError):
    def __init__(self, status: int, where: str = ""):
        self.status = status
        name = ERRORS.get(status, f"invalid argument {-status}" if -20 <= status < 0 else str(status))
        super().__init__(f"{where}: {name} ({status})" if where else f"{name} ({status})")


def lib():
    """Loads libparaht.so.  Raises if it has not been built (or is older than its sources)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build

    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libparaht.so missing at {LIB_PATH}; build it with paraht_gb300.build.build()")
    if not _build.up_to_date():
        raise RuntimeError(f"libparaht.so at {LIB_PATH} is stale or built for another host; rebuild it")
    L = C.CDLL(LIB_PATH)
    for name, argt in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = argt
        f.restype = C.c_char_p if name == "paraht_strerror" else C.c_int
    _lib = L
    return L


def check(status: int, where: str = "") -> None:
    if status != 0:
        raise ParahtError(status, where)
