"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``paraht_oracle.c`` + ``lapack_loader.c`` with gcc/OpenMP into
``oracle/_build/libparaht_oracle.so``.  LAPACK is resolved at run time (dlopen) from the
OpenBLAS bundled with scipy, whose path is baked in as the default and can be overridden
with the environment variable PARAHT_ORACLE_LAPACK.

The reference itself (Fortran 90 + MKL, src/*.f90) cannot be compiled here: the image has
no Fortran compiler, so there is no ``oracle/_ref`` build.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libparaht_oracle.so")
SOURCES = ["paraht_oracle.c", "lapack_loader.c"]


def find_lapack() -> str:
    env = os.environ.get("PARAHT_ORACLE_LAPACK")
    if env:
        return env
    import scipy  # noqa: F401  (only used to locate its bundled OpenBLAS)

    base = os.path.dirname(os.path.dirname(scipy.__file__))
    cands = sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")))
    cands = [c for c in cands if "openblas64" not in os.path.basename(c)]
    if not cands:
        raise RuntimeError("no LP64 OpenBLAS found next to scipy; set PARAHT_ORACLE_LAPACK")
    return cands[0]


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES] + [os.path.join(HERE, "lapack_loader.h")]
    if not force and os.path.exists(LIB):
        lib_m = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= lib_m for s in srcs) and _same_host(LIB):
            return LIB
    lapack = find_lapack()
    cmd = [
        "gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=gnu11",
        f'-DORACLE_DEFAULT_LAPACK="{lapack}"',
        "-o", LIB + ".tmp",
    ] + [os.path.join(HERE, s) for s in SOURCES] + ["-ldl", "-lm", "-lpthread"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    with open(LIB + ".host", "w") as f:
        f.write(_host_tag())
    return LIB


def _host_tag() -> str:
    import platform

    return platform.machine()


def _same_host(lib: str) -> bool:
    try:
        with open(lib + ".host") as f:
            return f.read().strip() == _host_tag()
    except OSError:
        return False


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
