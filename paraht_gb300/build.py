"""Build recipe for libparaht.so (sm_103a), the GPU product library.

Compiles every ``csrc/*.cu`` translation unit with nvcc in parallel and links them into
``paraht_gb300/_build/libparaht.so`` (C ABI: ``include/paraht.h``).  No torch, no cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libparaht.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH
# Per-file flags: the pipelined chase reads data other CTAs wrote, so its global loads bypass L1.
FILE_FLAGS = {"stage2_chase.cu": ["-Xptxas", "-dlcm=cg"], "stage2g_chase.cu": ["-Xptxas", "-dlcm=cg"]}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))) + [
        os.path.join(os.path.dirname(HERE), "include", "paraht.h")
    ]


def _stamp() -> str:
    return platform.machine()


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    try:
        with open(LIB + ".host") as f:
            if f.read().strip() != _stamp():
                return False
    except OSError:
        return False
    m = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= m for d in _deps())


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    flags = NVCC_FLAGS + list(extra_flags or [])
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc(), "-c", src, "-o", obj] + flags + FILE_FLAGS.get(os.path.basename(src), [])
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["--cudart", "shared"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(LIB + ".host", "w") as f:
        f.write(_stamp())
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, extra_flags=[a for a in sys.argv[1:] if a.startswith("-X")]))
