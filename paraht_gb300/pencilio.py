"""Pencil files: a reduced or partially reduced pencil (A, B, Q, Z) on disk.

Lets stage 2 be run, timed and tuned on its own at large n without re-running stage 1: save the
r-Hessenberg pencil after paraht_ab2rht (stage 1, src/ab2rht.f90:8-495), load it, and run
paraht_rht2ht (stage 2, src/rht2ht.f90:1346-2051) on it.  The reference keeps the stage-1 output
only in memory (src/profilereduction.f90:136-144).

Format (little-endian): the 8-byte magic ``PHTPENC1``, an 8-byte header length h, h bytes of
UTF-8 JSON ({"n": n, "stage": s, "r": r, "p": p, "matrices": ["A", "B", "Q", "Z"], ...}), then the
listed n x n matrices one after the other, each column-major float64 (n*n*8 bytes, the layout the
library works in, so a file maps straight into device buffers).
"""
from __future__ import annotations

import json
import os
import struct

import numpy as np

MAGIC = b"PHTPENC1"


def save_pencil(path: str, A, B, Q=None, Z=None, **meta) -> None:
    """Writes the pencil (Fortran-ordered float64 n x n arrays; Q, Z optional) and metadata."""
    mats = {"A": A, "B": B}
    if Q is not None:
        mats["Q"] = Q
    if Z is not None:
        mats["Z"] = Z
    n = A.shape[0]
    for k, X in mats.items():
        if X.shape != (n, n):
            raise ValueError(f"{k} must be {n} x {n}")
    head = dict(meta, n=int(n), matrices=list(mats))
    hb = json.dumps(head, sort_keys=True).encode()
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<Q", len(hb)))
        f.write(hb)
        for X in mats.values():
            np.asarray(X, dtype="<f8").ravel(order="F").tofile(f)
    os.replace(tmp, path)


def read_header(path: str) -> dict:
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError(f"{path}: not a pencil file")
        (h,) = struct.unpack("<Q", f.read(8))
        return json.loads(f.read(h).decode())


def load_pencil(path: str, mmap: bool = False):
    """Returns (header, {name: Fortran-ordered n x n float64 array}).  mmap=True maps the file
    instead of reading it (read-only views)."""
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError(f"{path}: not a pencil file")
        (h,) = struct.unpack("<Q", f.read(8))
        head = json.loads(f.read(h).decode())
        off = 16 + h
    n = int(head["n"])
    names = head["matrices"]
    size = n * n * 8
    if os.path.getsize(path) != off + size * len(names):
        raise ValueError(f"{path}: truncated or oversized ({os.path.getsize(path)} bytes)")
    out = {}
    if mmap:
        mm = np.memmap(path, dtype="<f8", mode="r", offset=off, shape=(len(names), n * n))
        for i, k in enumerate(names):
            out[k] = mm[i].reshape((n, n), order="F")
    else:
        with open(path, "rb") as f:
            f.seek(off)
            for k in names:
                out[k] = np.fromfile(f, dtype="<f8", count=n * n).reshape((n, n), order="F")
    return head, out
