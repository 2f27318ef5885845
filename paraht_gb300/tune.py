"""Autotuner for the ParaHT parameters (r, p, nq) per pencil size, on the GPU it runs on.

The reference leaves r (= nb), p and nq to the caller (src/profilereduction.f90 reads them from
the command line).  Here a table measured on GB300 maps a pencil size to the fastest parameters
for each mode:

* ``"split"`` / ``"fp64"``: one pencil through paraht_reduce_d (split-precision or FP64 bulk
  updates), time per reduction;
* ``"batch"``: pencils of that size in the persistent batched kernel (paraht_reduce_batched_d,
  one CTA per pencil, p r <= 64), throughput in pencils/s.

``pick(n, mode)`` returns the entry of the nearest measured size (log scale); sizes outside the
table take the nearest end.  ``stage2(mode, r, nq)`` names the faster stage-2 variant for a mode
("givens", rht2ht_givens, or "householder", rht2ht_householder), from the table's measured
comparison, where the Givens variant takes the parameters.  ``python -m paraht_gb300.tune``
measures a new table:

    python -m paraht_gb300.tune --mode split --sizes 1000,2000,4000 --out paraht_gb300/tune_table.json

Each candidate is timed after one untimed call of the same shape (CUDA events on the context's
stream, inputs restored between calls outside the timed region).  The split kernel's slice count
is fixed, not tuned: 8 digits of 7 bits with the 43 digit-pair products of level t + u <= 8;
dropping level 8 (36 products) measured a backward error of 1.5e-13 at n = 4000, above the split
path's 1e-13 bound.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_PATH = os.path.join(HERE, "tune_table.json")

# used when no measured table is present: the reference driver's documented example (r=16,
# p=8, nq=8) adjusted to what GB300 measurements favour (p=4 for the single pencil, p r <= 64 for
# the persistent batched kernel)
FALLBACK = {
    "split": [[1000, 16, 4, 16]],
    "fp64": [[1000, 16, 4, 16]],
    "batch": [[256, 16, 4, 16]],
}

# stage-2 variant per mode when the table has none: the measured comparison at n = 4000 (one
# pencil, r=16 p=4 nq=16): split 6.67 s with Givens rotations vs 8.01 s with small reflectors;
# FP64 9.57 s with small reflectors vs 10.78 s with Givens rotations
STAGE2_FALLBACK = {"split": "givens", "fp64": "householder", "batch": "householder"}

CANDIDATES = {
    "split": [(16, 4, 16), (16, 3, 16), (16, 5, 16), (16, 4, 8), (32, 2, 16), (8, 4, 8)],
    "fp64": [(16, 4, 16), (16, 3, 16), (16, 5, 16), (16, 4, 8), (32, 2, 16), (32, 4, 16)],
    "batch": [(16, 4, 16), (16, 2, 16), (16, 4, 8), (8, 4, 8), (8, 8, 8), (32, 2, 16), (16, 3, 8)],
}


def load_table(path: str = TABLE_PATH) -> dict:
    try:
        with open(path) as f:
            t = json.load(f)
        return {m: t.get(m, FALLBACK[m]) or FALLBACK[m] for m in FALLBACK}
    except (OSError, ValueError):
        return dict(FALLBACK)


def stage2(mode: str = "split", r: int = 16, nq: int = 16, table: dict | None = None) -> str:
    """The faster stage-2 variant for `mode`: "givens" or "householder".  The Givens variant needs
    r <= 32 and r + nq <= 64 (split-precision dense ops up to 48 wide), and the persistent batched
    kernel chases with reflectors only."""
    if mode not in FALLBACK:
        raise ValueError(f"unknown mode {mode!r}")
    t = table if table is not None else _raw_table()
    choice = (t.get("stage2") or {}).get(mode, STAGE2_FALLBACK[mode])
    if choice == "givens" and (mode == "batch" or r > 32 or r + nq > 64):
        return "householder"
    return choice


def _raw_table(path: str = TABLE_PATH) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def pick(n: int, mode: str = "split", table: dict | None = None):
    """(r, p, nq) for a pencil of size n in `mode` ("split", "fp64" or "batch")."""
    if mode not in FALLBACK:
        raise ValueError(f"unknown mode {mode!r}")
    rows = (table or load_table())[mode]
    best = min(rows, key=lambda e: abs(math.log(max(n, 1)) - math.log(e[0])))
    r, p, nq = int(best[1]), int(best[2]), int(best[3])
    r = max(1, min(r, max(1, n - 1)))  # tiny pencils: a bandwidth below n
    return r, p, min(nq, r)


def _time_single(ctx, torch, n, cand, flags, reps):
    from .generate import pencil

    r, p, nq = cand
    A0, B0 = pencil(n, "std", seed=1302)
    import numpy as np

    pris = [torch.from_numpy(np.ascontiguousarray(X.T)).cuda() for X in (A0, B0)]
    eye = torch.eye(n, dtype=torch.float64, device="cuda")
    work = [torch.empty_like(eye) for _ in range(4)]
    ts = []
    for i in range(reps + 1):
        work[0].copy_(pris[0])
        work[1].copy_(pris[1])
        work[2].copy_(eye)
        work[3].copy_(eye)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.reduce_d(n, work[0].data_ptr(), n, work[1].data_ptr(), n, work[2].data_ptr(), n, work[3].data_ptr(), n,
                     r, p, nq, flags)
        if i:
            ts.append(time.perf_counter() - t0)
    return min(ts)


def _time_batch(ctx, torch, n, cand, reps, count):
    import numpy as np

    from .generate import pencil

    r, p, nq = cand
    pencils = [pencil(n, "std", seed=1302 + i) for i in range(count)]
    pris = [[torch.from_numpy(np.ascontiguousarray(X.T)).cuda() for X in ab] for ab in pencils]
    eye = torch.eye(n, dtype=torch.float64, device="cuda")
    work = [[torch.empty_like(eye) for _ in range(4)] for _ in range(count)]
    ns = [n] * count
    ts = []
    for i in range(reps + 1):
        for w, (a, b) in zip(work, pris):
            w[0].copy_(a)
            w[1].copy_(b)
            w[2].copy_(eye)
            w[3].copy_(eye)
        torch.cuda.synchronize()
        ptr = lambda j: [w[j].data_ptr() for w in work]  # noqa: E731
        t0 = time.perf_counter()
        ctx.reduce_batched_d(ns, ptr(0), ns, ptr(1), ns, ptr(2), ns, ptr(3), ns, [r] * count, [p] * count,
                             [nq] * count)
        if i:
            ts.append(time.perf_counter() - t0)
    return count / min(ts)


def measure(mode: str, sizes, candidates=None, reps: int = 1, batch_count: int = 304):
    """Times every candidate at every size; returns (table rows, all timings)."""
    import torch

    import paraht_gb300 as ph

    ctx = ph.Context(0)
    rows, raw = [], []
    for n in sizes:
        best = None
        for cand in candidates or CANDIDATES[mode]:
            r, p, nq = cand
            if nq > r or r >= n or (mode == "batch" and p * r > 64):
                continue
            if mode == "batch":
                v = _time_batch(ctx, torch, n, cand, reps, batch_count)
                better = best is None or v > best[1]
            else:
                flags = ph.PARAHT_FLAG_SPLIT if mode == "split" else 0
                v = _time_single(ctx, torch, n, cand, flags, reps)
                better = best is None or v < best[1]
            raw.append({"n": n, "r": r, "p": p, "nq": nq, "value": v,
                        "unit": "pencils/s" if mode == "batch" else "s"})
            print(json.dumps(raw[-1]), flush=True)
            if better:
                best = (cand, v)
        if best:
            rows.append([n, *best[0]])
    ctx.close()
    return rows, raw


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--mode", choices=tuple(FALLBACK), default="split")
    ap.add_argument("--sizes", default="1000,2000,4000")
    ap.add_argument("--reps", type=int, default=1)
    ap.add_argument("--out", default=None, help="merge the result into this table file")
    args = ap.parse_args(argv)
    sizes = [int(s) for s in args.sizes.split(",") if s]
    rows, raw = measure(args.mode, sizes, reps=args.reps)
    if args.out:
        doc = {}
        if os.path.exists(args.out):
            with open(args.out) as f:
                doc = json.load(f)
        keep = [e for e in doc.get(args.mode, []) if e[0] not in sizes]
        doc[args.mode] = sorted(keep + rows)
        meas = doc.get("measurements", {})
        meas[args.mode] = [m for m in meas.get(args.mode, []) if m["n"] not in sizes] + raw
        doc["measurements"] = meas
        with open(args.out, "w") as f:
            json.dump(doc, f, indent=1)
    print(json.dumps({"mode": args.mode, "table": rows}))


if __name__ == "__main__":
    main()
