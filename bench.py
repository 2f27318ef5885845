#!/usr/bin/env python3
"""Headline benchmark: seconds for the two-stage HT reduction of one n=16000 pencil on one GB300,
split-precision bulk updates against the all-FP64 GPU path.

Metric: "HT-reduction sec at n=16000: split-prec vs FP64 GPU at bwd err<=1e-13".
A step is one full reduction (stage 1 + stage 2, Q and Z accumulated) of the synthetic pencil
"std" (A ~ N(0,1), B the R factor of a Gaussian matrix, seed 1302) with the reference's
parameter surface (r, p, nq), as src/profilereduction.f90:134-148 times it: one call of each
stage on device-resident arrays, then the backward-error report (:165-184).  Arrays are
column-major FP64 resident in HBM; the pristine input is restored (device-to-device copy) before
every step, outside the timed region.  The inputs (4 x n^2 x 8 B = 8.2 GB at n=16000) are far
larger than L2, so no extra L2 flush is needed.

One reduction at n=16000 takes minutes, so the run is bounded by a wall budget (--budget-s,
measured from process start): the warm-up runs W-1 reductions at n=2000 and one full-size
reduction; then one FP64 reduction at the FP64 path's own tuned parameters; then timed
split-precision reductions until the budget left covers only the end-to-end step, the checks
and the CPU baselines.  ``steps`` is the number of split reductions actually timed,
``steps_requested`` the --steps asked for.

* ``value``: mean device time per split step (CUDA events on the library's stream, max over ranks).
* ``fp64``: the all-FP64 path's device time for one reduction at its tuned (r, p, nq) and stage-2
  variant (small reflectors), its backward errors, and ``split_vs_fp64`` = fp64 seconds / split
  seconds.  The split path runs its faster stage-2 variant, Givens rotations (--stage2).
* ``check``: backward errors ||Q^T A0 Z - H||/||A0||, ||Q^T B0 Z - T||/||B0|| and orthogonality
  ||Q^T Q - I||_F, ||Z^T Z - I||_F of the last split step (FP64 GEMMs on the device); ``eig``: the
  generalized eigenvalues of a seeded n=600 pencil against those of its (H, T) from each arm.
* ``e2e``: one split reduction through the public host entry point paraht_reduce_host with
  pinned host buffers, host<->device copies inside the timed region.
* ``roofline``: the dominant kernel (the split-precision op-list kernel of stage 2), every launch
  timed with CUDA events on its stream during the timed steps; ``traffic`` is its DRAM bytes per
  launch from an ncu capture of the same kernel at n=6000, scaled by the flops per launch.
* ``cpu_baseline``: the CPU oracle (a restatement of the reference's OpenMP algorithm) on a
  bounded sample, scaled by (n / n_sample)^3 to the metric's unit.
* ``--impl reference``: times that CPU implementation on the host cores (the reference itself
  is Fortran and cannot be compiled on this image).

Multi-GPU: the single-pencil path does not shard (replicas only): with N ranks every rank
reduces its own pencil; value = max-over-ranks step time / N (job seconds per reduction).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

T_PROC0 = time.perf_counter()
ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "HT-reduction sec at n=16000: split-prec vs FP64 GPU at bwd err<=1e-13"
EPS = float(np.finfo(np.float64).eps)
# FP64 roof when it cannot be measured in the run: 2 FMA/clk/SM x 152 SMs x 2.07 GHz on GB300
FP64_PEAK_TFLOPS = 1.26


# DRAM bytes per FP64-equivalent flop of the split op-list kernel, measured with ncu on the Q and Z
# lists of one n=6000 sweep group (207.9456 MB over 2.1504 GFLOP)
TRAFFIC_BYTES_PER_FLOP = 207.9456e6 / 2.1504e9


def measure_fp64_peak(torch, n: int = 8192, reps: int = 3):
    """The FP64 roof used for the FP64 kernels' roofline fraction: cuBLAS DGEMM (torch.matmul on
    float64, 2 n^3 flops) on this GPU, best of `reps` after one warm-up, in TFLOP/s."""
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("paraht", "reference"), default="paraht")
    ap.add_argument("--workload", choices=("pencil", "batch4096", "batch256", "qz1216"), default="pencil",
                    help="pencil: one n x n pencil (the headline); batch4096: 4096 FP64 pencils, n ~ U{32..512}; "
                         "batch256: 256 pencils, n log-uniform in [256, 4096], 30%% graded, split precision; "
                         "qz1216: QZ eigenvalues of 1216 Hessenberg-triangular pencils, n ~ U{32..256}")
    ap.add_argument("--loop-sample", type=int, default=0,
                    help="pencils of the looped baseline (batch workloads; 0: the workload's default)")
    ap.add_argument("--n", type=int, default=16000)
    ap.add_argument("--r", type=int, default=16)
    ap.add_argument("--p", type=int, default=4)
    ap.add_argument("--nq", type=int, default=16)
    ap.add_argument("--fp64-params", default="32,4,16",
                    help="r,p,nq of the FP64 comparison step (the FP64 path's tuned parameters at n >= 4000)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison step")
    ap.add_argument("--dist", default="std")
    ap.add_argument("--precision", choices=("fp64", "split"), default="split")
    ap.add_argument("--stage2", choices=("householder", "givens"), default="givens",
                    help="stage-2 variant of the timed path: Givens rotations (rht2ht_givens, the faster split "
                         "path) or small reflectors (rht2ht_householder)")
    ap.add_argument("--fp64-stage2", choices=("householder", "givens"), default="householder",
                    help="stage-2 variant of the FP64 comparison step (small reflectors: the faster FP64 path)")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--cpu-sample-n", type=int, default=4000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-check", action="store_true", help="skip the backward-error / orthogonality check")
    ap.add_argument("--check", action="store_true", help=argparse.SUPPRESS)  # the check is on by default
    ap.add_argument("--budget-s", type=float, default=1500.0,
                    help="wall-clock budget of the whole run in seconds, from process start")
    ap.add_argument("--warmup-n", type=int, default=2000, help="size of the reduced-size warm-up steps")
    ap.add_argument("--phases", action="store_true", help="one extra serialised step for the per-phase times")
    ap.add_argument("--chain", action="store_true",
                    help="one extra overlapped step with the critical-path share of each phase (PARAHT_FLAG_TIME_CHAIN)")
    ap.add_argument("--save-stage1", default="", help="after the run, save this pencil's stage-1 output here")
    ap.add_argument("--stage2-from", default="", help="time stage 2 alone on a saved stage-1 output")
    return ap.parse_args(argv)


def elapsed() -> float:
    return time.perf_counter() - T_PROC0


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                f = [x.strip() for x in out.stdout.strip().split(",")]
                if len(f) >= 7:
                    self.samples.append(f)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def job_time(t_local: float, device) -> float:
    """The job's step time: the maximum over ranks of each rank's own step time (replicas: every
    rank reduces its own pencils, no data is exchanged; one all-reduce of a scalar)."""
    import torch
    import torch.distributed as td

    if not (td.is_available() and td.is_initialized()) or td.get_world_size() == 1:
        return t_local
    tt = torch.tensor([t_local], dtype=torch.float64, device=device)
    td.all_reduce(tt, op=td.ReduceOp.MAX)
    return float(tt.item())


def all_agree(flag: bool, device) -> bool:
    """True only if every rank passes True (replicas decide together whether to time another
    step, so that all of them reach the same barriers)."""
    import torch
    import torch.distributed as td

    if not (td.is_available() and td.is_initialized()) or td.get_world_size() == 1:
        return flag
    tt = torch.tensor([1 if flag else 0], dtype=torch.int32, device=device)
    td.all_reduce(tt, op=td.ReduceOp.MIN)
    return bool(int(tt.item()))


def replica_seed(base: int, rank: int) -> int:
    """Seed of rank `rank`'s own input (replicas reduce different pencils of one distribution)."""
    return base + rank


def flops_nominal(n: int) -> float:
    # fixed nominal count used for "effective GFLOP/s" (stage 1 at p=8 plus stage 2): 18.67 n^3
    return 18.67 * float(n) ** 3


def budget_plan(budget_s: float, now_s: float, t_step_s: float, done: int, requested: int, reserve_s: float) -> bool:
    """Whether to time another step: always the first one, then while fewer than `requested`
    are done and another step of t_step_s plus the work still to come (reserve_s) fits in the
    wall budget."""
    if done >= requested:
        return False
    if done == 0:
        return True
    return now_s + t_step_s + reserve_s <= budget_s


def cpu_oracle_seconds(n_sample: int, r: int, p: int, nq: int, dist: str):
    """Times the CPU oracle (restatement of the reference's OpenMP ParaHT) once on n_sample."""
    from oracle import oracle as O
    from paraht_gb300.generate import identity, pencil

    O.set_blas_threads(1)
    A, B = pencil(n_sample, dist, seed=1302)
    Q, Z = identity(n_sample), identity(n_sample)
    t0 = time.perf_counter()
    O.reduce(A, B, Q, Z, min(r, n_sample), p, min(nq, r))
    return time.perf_counter() - t0


def cpu_dgghd3_seconds(n_sample: int, dist: str):
    """Times LAPACK DGGHD3 (the reference driver's one-stage baseline, src/profilereduction.f90:156)
    once on n_sample with a multithreaded BLAS on all host cores."""
    from oracle import oracle as O
    from paraht_gb300.generate import identity, pencil

    O.set_blas_threads(os.cpu_count() or 1)
    A, B = pencil(n_sample, dist, seed=1302)
    Q, Z = identity(n_sample), identity(n_sample)
    t0 = time.perf_counter()
    O.dgghd3(A, B, Q, Z)
    dt = time.perf_counter() - t0
    O.set_blas_threads(1)
    return dt


def reference_line(args, ts, ns, cores):
    """The reference arm's JSON line: the CPU oracle's mean time per sample reduction at n=ns,
    extrapolated by (n/ns)^3 to the workload size."""
    scale = (args.n / ns) ** 3
    v = statistics.mean(ts) * scale
    return {
        "metric": METRIC, "value": v, "unit": "s", "impl": "reference", "n_gpus": args.gpus, "steps": len(ts),
        "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(ts) * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"HT reduction n={args.n} r={args.r} p={args.p} nq={args.nq} dist={args.dist}",
                   "n": args.n, "r": args.r, "p": args.p, "nq": args.nq},
        "sample_n": ns, "extrapolated": True, "extrapolation": f"(n/{ns})^3 = {scale:.2f}",
        "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port",
                         "sample": f"oracle (C/OpenMP restatement of ab2rht_simple+rht2ht_householder, single-threaded "
                                   f"BLAS inside tasks) at n={ns}, mean of {len(ts)} runs, scaled by (n/{ns})^3; "
                                   f"ms_per_step is the n={ns} sample's time"},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference(args, rank: int):
    """--impl reference: the CPU implementation of the path on the host cores, sample reductions
    at n = --cpu-sample-n timed until --steps are done or the wall budget runs out."""
    if rank != 0:
        return 0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    ns = min(args.cpu_sample_n, args.n)
    for _ in range(args.warmup):
        cpu_oracle_seconds(max(200, ns // 4), args.r, args.p, args.nq, args.dist)
    ts = []
    budget = min(args.budget_s, 600.0)
    while budget_plan(budget, elapsed(), ts[-1] if ts else 0.0, len(ts), max(1, args.steps), 0.0):
        ts.append(cpu_oracle_seconds(ns, args.r, args.p, args.nq, args.dist))
    print(json.dumps(reference_line(args, ts, ns, cores)), flush=True)
    return 0


BATCHES = {
    # the batch workloads: 4096 FP64 pencils n ~ U{32..512}; 256 pencils n log-uniform in [256, 4096],
    # 70% Std / 30% graded-singular B, split-precision updates
    "batch4096": dict(count=4096, lo=32, hi=512, law="uniform", graded=0.0, split=False, loop=256,
                      metric="batched HT reduction: pencils/s, 4096 pencils n~U{32..512}, FP64"),
    "batch256": dict(count=256, lo=256, hi=4096, law="loguniform", graded=0.3, split=True, loop=12,
                     metric="batched HT reduction: pencils/s, 256 pencils n log-U[256,4096], 30% graded, split"),
}


def batch_params(n: int, split: bool):
    """(r, p, nq) of a batch pencil of size n from the autotuner's table: the persistent kernel's
    entry where it takes the pencil (n <= 1024), else the single-pencil path's."""
    from paraht_gb300 import tune

    if n <= 1024:
        r, p, nq = tune.pick(n, "batch")
        if p * r <= 64:
            return r, p, nq
    return tune.pick(n, "split" if split else "fp64")


def run_batch(args, rank: int, world: int, local: int):
    """--workload batch4096 / batch256: many pencils of uneven size in one paraht_reduce_batched_d
    call; the looped single-pencil path on a sample of the same pencils and the CPU oracle on a
    smaller sample are timed beside it."""
    import numpy as _np

    from paraht_gb300.generate import batch_sizes, identity, pencil

    spec = BATCHES[args.workload]
    count, lo, hi = spec["count"], spec["lo"], spec["hi"]
    sizes = batch_sizes(count, lo, hi, spec["law"], seed=replica_seed(1302, rank))
    rng = _np.random.default_rng(replica_seed(2604, rank))
    dists = ["graded" if rng.random() < spec["graded"] else "std" for _ in sizes]
    params = [batch_params(n, spec["split"]) for n in sizes]
    flops = sum(18.67 * float(n) ** 3 for n in sizes)
    n3 = statistics.mean(float(n) ** 3 for n in sizes)
    workload = (f"{count} pencils, n {'~U{' + str(lo) + '..' + str(hi) + '}' if spec['law'] == 'uniform' else 'log-U[' + str(lo) + ',' + str(hi) + ']'}"
                f" (seeded), {int(round(100 * spec['graded']))}% graded, r/p/nq from the autotuner table, "
                f"{'split-precision single-pencil path above n=1024, one paraht_reduce_batched_d call' if spec['split'] else 'FP64, one replay of the CUDA graph of the size-bucketed persistent launches (paraht_batch_plan)'}")

    def cpu_rate(nsample):
        """Oracle on the first pencils with n <= 1500, per-pencil time scaled by the batch's mean n^3."""
        from oracle import oracle as O

        O.set_blas_threads(1)
        idx = [i for i, n in enumerate(sizes) if n <= 1500][:nsample]
        per = []
        for i in idx:
            A, B = pencil(sizes[i], dists[i], seed=7 + i)
            r, p, nq = params[i]
            t0 = time.perf_counter()
            O.reduce(A, B, identity(sizes[i]), identity(sizes[i]), min(r, sizes[i]), p, min(nq, r))
            per.append((time.perf_counter() - t0) / float(sizes[i]) ** 3)
        v = 1.0 / (statistics.mean(per) * n3)
        return v, {"value": v, "unit": "pencils/s", "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
                   "kind": "port", "sample": f"CPU oracle on {len(idx)} pencils of the batch (n <= 1500), one after the "
                                             f"other, time per pencil scaled by the batch's mean n^3"}

    if args.impl == "reference":
        if rank != 0:
            return 0
        vs = [cpu_rate(4 if spec["split"] else 16) for _ in range(max(1, args.steps))]
        v = statistics.mean(x[0] for x in vs)
        print(json.dumps({
            "metric": spec["metric"], "value": v, "unit": "pencils/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * count / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload}, "cpu_baseline": {**vs[-1][1], "value": v},
            "e2e": {"value": v, "unit": "pencils/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}), flush=True)
        return 0

    # the batched call runs up to 8 worker contexts of 4 streams each beside the persistent
    # launch: ask for 32 hardware queues instead of CUDA's default 8 (read at context creation)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    import torch

    import paraht_gb300 as ph

    torch.cuda.set_device(local)
    dist_on = world > 1
    if dist_on:
        import torch.distributed as td

        td.init_process_group("nccl", device_id=torch.device("cuda", local))
    flags = ph.PARAHT_FLAG_SPLIT if spec["split"] else 0
    host = [pencil(n, d, seed=100000 * rank + i) for i, (n, d) in enumerate(zip(sizes, dists))]
    pris = [[torch.from_numpy(np.ascontiguousarray(X.T)).cuda() for X in ab] for ab in host]
    work = [[torch.empty_like(a), torch.empty_like(a), torch.empty_like(a), torch.empty_like(a)] for a, _ in pris]
    eyes = {}
    for n in set(sizes):
        eyes[n] = torch.eye(n, dtype=torch.float64, device="cuda")
    ctx = ph.Context(local)

    def restore(idx):
        for i in idx:
            w, (a, b) = work[i], pris[i]
            w[0].copy_(a)
            w[1].copy_(b)
            w[2].copy_(eyes[sizes[i]])
            w[3].copy_(eyes[sizes[i]])
        torch.cuda.synchronize()

    # when the persistent kernel takes every pencil (FP64, n <= 1024, p r <= 64) the whole batch is
    # a plan: its size buckets' persistent launches captured once in a CUDA graph, replayed per step
    use_plan = not spec["split"] and all(
        n <= ph.PARAHT_BATCH_MAX_N and params[i][0] * params[i][1] <= 64 for i, n in enumerate(sizes))
    plan = None
    if use_plan:
        ptr0 = lambda j: [work[i][j].data_ptr() for i in range(count)]  # noqa: E731
        plan = ctx.batch_plan(sizes, ptr0(0), sizes, ptr0(1), sizes, ptr0(2), sizes, ptr0(3), sizes,
                              [q[0] for q in params], [q[1] for q in params], [q[2] for q in params])

    def call(idx, f):
        if plan is not None and f == flags and len(idx) == count:
            plan.launch(0)
            torch.cuda.synchronize()
            return
        ns = [sizes[i] for i in idx]
        ptr = lambda j: [work[i][j].data_ptr() for i in idx]  # noqa: E731
        ctx.reduce_batched_d(ns, ptr(0), ns, ptr(1), ns, ptr(2), ns, ptr(3), ns, [params[i][0] for i in idx],
                             [params[i][1] for i in idx], [params[i][2] for i in idx], f)

    def barrier():
        if dist_on:
            import torch.distributed as td

            td.barrier()

    allidx = list(range(count))
    for _ in range(args.warmup):
        restore(allidx)
        call(allidx, flags)
    ts, launches = [], 0
    sampler = ClockSampler(local)
    with sampler:
        for _ in range(args.steps):
            restore(allidx)
            barrier()
            t0 = time.perf_counter()
            call(allidx, flags)
            ts.append(time.perf_counter() - t0)
            launches += ctx.launch_count()
            barrier()
    t_step = statistics.mean(ts)
    t_step = job_time(t_step, "cuda")
    value = world * count / t_step
    # backward errors of the last timed call, on the device (FP64 matmuls), every pencil
    errs = []
    for i in allidx:
        A0, B0 = pris[i][0].T, pris[i][1].T
        H, T, Q, Z = (work[i][j].T for j in range(4))
        errs.append(max(float(torch.linalg.norm(Q.T @ A0 @ Z - H) / torch.linalg.norm(A0)),
                        float(torch.linalg.norm(Q.T @ B0 @ Z - T) / torch.linalg.norm(B0))))
    errs_sorted = sorted(errs)
    # looped baseline: the same call with PARAHT_FLAG_BATCH_LOOP on a sample of the batch
    sample = allidx[: min(count, args.loop_sample if args.loop_sample > 0 else spec["loop"])]
    restore(sample)
    t0 = time.perf_counter()
    call(sample, flags | ph.PARAHT_FLAG_BATCH_LOOP)
    t_loop = time.perf_counter() - t0
    loop_v = 1.0 / (t_loop / sum(float(sizes[i]) ** 3 for i in sample) * n3)  # per-pencil time scaled by n^3
    # end to end: pinned host pencils -> device, batched call, results back (all four matrices)
    hostp = [[torch.from_numpy(np.ascontiguousarray(X.T)).pin_memory() for X in ab] for ab in host]
    outp = [[torch.empty(w[0].shape, dtype=torch.float64).pin_memory() for _ in range(4)] for w in work]
    h2d = d2h = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in allidx:
        w = work[i]
        w[0].copy_(hostp[i][0], non_blocking=True)
        w[1].copy_(hostp[i][1], non_blocking=True)
        w[2].copy_(eyes[sizes[i]])
        w[3].copy_(eyes[sizes[i]])
        h2d += 2 * w[0].numel() * 8
    torch.cuda.synchronize()
    call(allidx, flags)
    for i in allidx:
        for j in range(4):
            outp[i][j].copy_(work[i][j], non_blocking=True)
            d2h += work[i][j].numel() * 8
    torch.cuda.synchronize()
    e2e_v = world * count / (time.perf_counter() - t0)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_rate(4 if spec["split"] else 8)[1]
    if rank == 0:
        fp64_peak = measure_fp64_peak(torch)
        achieved = flops / t_step / 1e12 * world
        print(json.dumps({
            "metric": spec["metric"], "value": value, "unit": "pencils/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload, "pencils": count, "n_lo": lo, "n_hi": hi, "size_law": spec["law"],
                       "graph": plan is not None,
                       "graded_fraction": spec["graded"], "split": spec["split"],
                       "l2": "inputs >> L2; pristine inputs restored between steps outside the timed region"},
            "e2e": {"value": e2e_v, "unit": "pencils/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "looped_baseline": {"value": loop_v, "unit": "pencils/s", "sample": len(sample),
                                "note": "paraht_reduce_d per pencil, time per pencil scaled to the batch's mean n^3",
                                "speedup": value / world / loop_v},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp64_peak, "traffic": None,
                         "kernel": "k_batch_reduce and the single-pencil kernels (nominal 18.67 n^3 flops per pencil)",
                         "peak_source": "cuBLAS DGEMM 8192^3 measured in this run, of measured"},
            "bwd_err": {"max": errs_sorted[-1], "p99": errs_sorted[min(len(errs) - 1, int(0.99 * len(errs)))]},
            "cpu_baseline": cpu,
            "clocks": sampler.summary(),
        }), flush=True)
    if plan is not None:
        plan.close()
    ctx.close()
    if dist_on:
        import torch.distributed as td

        td.destroy_process_group()
    return 0




def device_check(torch, work, dev0):
    """Backward errors ||Q^T X0 Z - X||_F / ||X0||_F (src/profilereduction.f90:165-174) and
    orthogonality ||Q^T Q - I||_F, ||Z^T Z - I||_F of a reduced pencil, FP64 GEMMs on the device.
    The arrays are column-major data held as row-major tensors of the transposes."""
    H, T, Q, Z = (w.T for w in work)
    Af, Bf = dev0[0].T, dev0[1].T
    n = H.shape[0]
    out = {}
    out["bwd_err_A"] = float(torch.linalg.norm(Q.T @ Af @ Z - H) / torch.linalg.norm(Af))
    out["bwd_err_B"] = float(torch.linalg.norm(Q.T @ Bf @ Z - T) / torch.linalg.norm(Bf))
    eye = torch.eye(n, dtype=torch.float64, device=H.device)
    out["orth_Q_fro"] = float(torch.linalg.norm(Q.T @ Q - eye))
    out["orth_Z_fro"] = float(torch.linalg.norm(Z.T @ Z - eye))
    out["below_structure_nonzeros"] = int(torch.count_nonzero(torch.tril(H, -2)) + torch.count_nonzero(torch.tril(T, -1)))
    return out


def eig_mismatch(l1, l2) -> float:
    """Largest distance from an eigenvalue of l1 to its greedy nearest match in l2 (each used
    once), relative to max(1, |lambda|); infinite eigenvalues must match infinite ones."""
    a = np.asarray(l1, dtype=complex)
    b = np.asarray(l2, dtype=complex)
    if a.shape != b.shape:
        return float("inf")
    free = np.ones(b.shape[0], dtype=bool)
    worst = 0.0
    for lam in a:
        if not np.isfinite(lam):
            idx = np.flatnonzero(free & ~np.isfinite(b))
            if idx.size == 0:
                return float("inf")
            free[idx[0]] = False
            continue
        d = np.where(free & np.isfinite(b), np.abs(b - lam), np.inf)
        i = int(np.argmin(d))
        if not np.isfinite(d[i]):
            return float("inf")
        free[i] = False
        worst = max(worst, float(d[i]) / max(1.0, abs(lam)))
    return worst


def eig_check(ctx, arms, n_e: int = 600, seed: int = 7) -> dict:
    """Generalized eigenvalues of a seeded n_e pencil (LAPACK DGGEV through scipy) against those of
    its Hessenberg-triangular forms from each arm, reduced through the host entry point:
    arms = [(name, (r, p, nq), flags)].  The largest relative distance per arm."""
    import scipy.linalg as sla

    from paraht_gb300.generate import identity, pencil

    A0, B0 = pencil(n_e, "std", seed=seed)
    ref = sla.eigvals(A0, B0)
    out = {"n": n_e, "method": "scipy.linalg.eigvals (LAPACK DGGEV) of (A0, B0) vs of (H, T), greedy matching, "
                               "relative to max(1, |lambda|)"}
    for name, (r, p, nq), fl in arms:
        H, T = np.asfortranarray(A0.copy()), np.asfortranarray(B0.copy())
        Q, Z = identity(n_e), identity(n_e)
        ctx.reduce_host(H, T, Q, Z, r, p, nq, fl)
        out[name] = float(eig_mismatch(ref, sla.eigvals(H, T)))
    return out


def run_pencil(args, rank: int, world: int, local: int):
    import torch

    import paraht_gb300 as ph
    from paraht_gb300.generate import pencil

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    dist_on = world > 1
    if dist_on:
        import torch.distributed as td

        td.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist_on:
            import torch.distributed as td

            td.barrier()

    n, r, p, nq = args.n, args.r, args.p, args.nq
    split = args.precision == "split"
    variant = ph.PARAHT_FLAG_GIVENS if args.stage2 == "givens" else 0
    fvariant = ph.PARAHT_FLAG_GIVENS if args.fp64_stage2 == "givens" else 0
    flags = (ph.PARAHT_FLAG_SPLIT if split else 0) | variant
    fr, fp, fnq = (int(x) for x in args.fp64_params.split(","))
    do_fp64 = split and not args.no_fp64
    do_check = not args.no_check
    stage2_only = bool(args.stage2_from)
    if stage2_only:  # a saved stage-1 output (paraht_gb300.pencilio): time stage 2 alone
        args.e2e_steps, do_check, do_fp64 = 0, False, False
        from paraht_gb300 import pencilio

        head, mats = pencilio.load_pencil(args.stage2_from)
        n, r = int(head["n"]), int(head.get("r", r))
        A0, B0 = mats["A"], mats["B"]
        Q0, Z0 = mats.get("Q"), mats.get("Z")
    else:
        A0, B0 = pencil(n, args.dist, seed=replica_seed(1302, rank))
        Q0 = Z0 = None
    # pristine inputs on the device (column-major: a row-major tensor of the transpose)
    dev0 = [torch.from_numpy(np.ascontiguousarray(X.T)).cuda() for X in (A0, B0)]
    eye = torch.eye(n, dtype=torch.float64, device="cuda")
    qz0 = [torch.from_numpy(np.ascontiguousarray(X.T)).cuda() if X is not None else eye for X in (Q0, Z0)]
    work = [torch.empty_like(eye) for _ in range(4)]
    ctx = ph.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)

    def restore(w=work, src=None):
        a, b, q, z = src if src is not None else (dev0[0], dev0[1], qz0[0], qz0[1])
        with torch.cuda.stream(stream):
            w[0].copy_(a)
            w[1].copy_(b)
            w[2].copy_(q)
            w[3].copy_(z)
        stream.synchronize()

    def launch(w, m, prm, f):
        rr, pp, qq = prm
        ptrs = (m, w[0].data_ptr(), m, w[1].data_ptr(), m, w[2].data_ptr(), m, w[3].data_ptr(), m)
        if stage2_only:
            ctx.rht2ht_d(*ptrs, rr, qq, f)
        else:
            ctx.reduce_d(*ptrs, rr, pp, qq, f)

    def timed(prm, f):
        """One reduction of the full pencil on `work`; device seconds (CUDA events on the stream)."""
        restore()
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        launch(work, n, prm, f)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3

    # ---- warm-up: W-1 reductions at a reduced size (each parameter set used later), then one at
    # full size (module loading, workspace sizing, operand slots) ----
    nw = min(n, args.warmup_n)
    small0 = pencil(nw, args.dist, seed=7)
    sdev = [torch.from_numpy(np.ascontiguousarray(X.T)).cuda() for X in small0]
    seye = torch.eye(nw, dtype=torch.float64, device="cuda")
    swork = [torch.empty_like(seye) for _ in range(4)]
    warm_sets = [((r, p, nq), flags)] + ([((fr, fp, fnq), fvariant)] if do_fp64 else [])
    for i in range(max(0, args.warmup - 1)):
        prm, f = warm_sets[i % len(warm_sets)]
        restore(swork, (sdev[0], sdev[1], seye, seye))
        launch(swork, nw, prm, f)
    if do_fp64 and args.warmup < 3:  # the FP64 parameter set gets at least one small warm-up
        restore(swork, (sdev[0], sdev[1], seye, seye))
        launch(swork, nw, (fr, fp, fnq), fvariant)
    del swork, sdev, seye
    t0w = time.perf_counter()
    if args.warmup > 0:
        restore()
        launch(work, n, (r, p, nq), flags)
    torch.cuda.synchronize()
    t_warm_full = time.perf_counter() - t0w

    try:
        fp64_peak = measure_fp64_peak(torch)
    except RuntimeError:
        fp64_peak = FP64_PEAK_TFLOPS
    ms, launches = [], 0
    kst = {k: {"seconds": 0.0, "launches": 0, "flops": 0.0, "busy_seconds": 0.0} for k in ("stage1", "stage2")}
    fp64 = None
    check = None
    t_check = 0.0
    sampler = ClockSampler(local)
    with sampler:
        # ---- one FP64 reduction at the FP64 path's own parameters ----
        if do_fp64:
            t_f = timed((fr, fp, fnq), fvariant | ph.PARAHT_FLAG_KERNEL_TIMES)
            t_f = job_time(t_f, "cuda")
            fst = ctx.kernel_stats()["stage2"]
            fp64 = {"seconds": t_f, "r": fr, "p": fp, "nq": fnq, "stage2": args.fp64_stage2, "launches": ctx.launch_count(),
                    "effective_gflops": flops_nominal(n) / t_f / 1e9,
                    "op_list_kernel": {"kernel": ("k_apply_left/k_apply_right<GeoS2G> (FP64 dense op lists)"
                                                  if args.fp64_stage2 == "givens" else
                                                  "k_apply_left/k_apply_right<GeoS2> (FP64 compact-WY op lists)"),
                                       "achieved_tflops": fst["flops"] / fst["seconds"] / 1e12 if fst["seconds"] > 0 else None,
                                       "peak_tflops": fp64_peak,
                                       "peak_source": "cuBLAS DGEMM 8192^3 measured in this run, of measured",
                                       "frac": (fst["flops"] / fst["seconds"] / 1e12 / fp64_peak
                                                if fst["seconds"] > 0 else None),
                                       "launches": fst["launches"], "seconds": fst["seconds"],
                                       "busy_seconds": fst["busy_seconds"],
                                       "achieved_busy_tflops": (fst["flops"] / fst["busy_seconds"] / 1e12
                                                                if fst["busy_seconds"] > 0 else None)}}
            if do_check:
                tc = time.perf_counter()
                fp64["check"] = device_check(torch, work, dev0)
                t_check = time.perf_counter() - tc
        # ---- timed split (or --precision) reductions within the budget ----
        t_est = t_warm_full
        cpu_est = 0.0 if (args.no_cpu_baseline or rank != 0 or stage2_only) else 90.0 * (min(args.cpu_sample_n, n) / 4000.0) ** 3 + 10.0
        e2e_est = (t_est * 1.05 + 5.0) * max(0, args.e2e_steps)
        reserve = e2e_est + (t_check if do_check else 0.0) + cpu_est + 20.0
        while all_agree(budget_plan(args.budget_s, elapsed(), t_est, len(ms), max(1, args.steps), reserve), "cuda"):
            ms.append(timed((r, p, nq), flags | ph.PARAHT_FLAG_KERNEL_TIMES))
            t_est = max(t_est, ms[-1] * 1.02)
            launches += ctx.launch_count()
            st = ctx.kernel_stats()
            for k in kst:
                for f in kst[k]:
                    kst[k][f] += st[k][f]
            barrier()
    steps_done = len(ms)
    t_step = job_time(statistics.mean(ms), "cuda")
    value = t_step / world

    # backward errors and orthogonality of the last timed step (outside the timed region)
    if do_check:
        check = device_check(torch, work, dev0)
        check["bound_split"] = 1e-13
        check["bound_10n_eps"] = 10 * n * EPS
        if rank == 0 and not stage2_only:  # eigenvalues of a small pencil through both arms (a few seconds)
            arms = [(args.precision, (r, p, nq), flags & ~ph.PARAHT_FLAG_KERNEL_TIMES)]
            if do_fp64:
                arms.append(("fp64", (fr, fp, fnq), fvariant))
            try:
                check["eig"] = eig_check(ctx, arms)
            except Exception as exc:  # the line keeps its timing even if this check cannot run
                check["eig"] = {"error": f"{type(exc).__name__}: {exc}"[:200]}

    # end to end through the host entry point, copies inside the timed region
    hbuf = [torch.empty((n, n), dtype=torch.float64).pin_memory() for _ in range(4)] if args.e2e_steps > 0 else []

    def host_step():
        hbuf[0].copy_(torch.from_numpy(np.asfortranarray(A0).T))
        hbuf[1].copy_(torch.from_numpy(np.asfortranarray(B0).T))
        hbuf[2].copy_(torch.eye(n, dtype=torch.float64))
        hbuf[3].copy_(torch.eye(n, dtype=torch.float64))
        nA, nB, nQ, nZ = (x.numpy().T for x in hbuf)  # Fortran-ordered views of pinned memory
        barrier()
        t0 = time.perf_counter()
        ctx.reduce_host(nA, nB, nQ, nZ, r, p, nq, flags)
        return time.perf_counter() - t0

    e2e_v = None
    if args.e2e_steps > 0:
        e2e_v = job_time(statistics.mean([host_step() for _ in range(args.e2e_steps)]), "cuda") / world

    phases = None
    if args.phases:  # time_components serialises the streams: one extra, slower step
        restore()
        launch(work, n, (r, p, nq), flags | ph.PARAHT_FLAG_TIME_COMPONENTS)
        phases = {k: round(v, 4) for k, v in ctx.phase_times().items()}
    chain = None
    if args.chain:  # the phase marks on each stage's critical-path stream, side streams overlapped
        restore()
        launch(work, n, (r, p, nq), flags | ph.PARAHT_FLAG_TIME_CHAIN)
        chain = {k: round(v, 4) for k, v in ctx.phase_times().items()}

    # roofline of the dominant kernel: the compact-WY op-list kernel of stage 2 (bulk and
    # lookahead updates), timed launch by launch with CUDA events on its streams during the timed
    # steps; its algorithmic work is 4 len k FP64-equivalent flops per strip row per op
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except (OSError, ValueError):
        pass
    s2 = kst["stage2"]
    fp64eq = s2["flops"] / s2["seconds"] / 1e12 if s2["seconds"] > 0 else None
    # the lists run on four streams at once: flops over the time at least one of them ran
    fp64eq_busy = s2["flops"] / s2["busy_seconds"] / 1e12 if s2["busy_seconds"] > 0 else None
    if split:
        # each FP64-equivalent flop is 43 FP16 digit-pair flops on the tensor cores (pairs t+u <= 8)
        measured = "bf16_tflops" in peaks
        peak = float(peaks["bf16_tflops"]) if measured else 1900.0
        achieved = 43.0 * fp64eq if fp64eq else None
        # DRAM bytes per launch: the ncu capture of the Q and Z lists at n=6000 (207.9 MB of DRAM
        # reads + writes per 2.1504 GFLOP FP64-equivalent) scaled to this run's mean launch; a list's
        # bytes and flops both grow as the rows x columns of its span (ops 32 wide, 2048 flops per
        # strip row per op in either stage-2 variant)
        per_launch_flops = s2["flops"] / s2["launches"] if s2["launches"] else 0.0
        traffic = TRAFFIC_BYTES_PER_FLOP * per_launch_flops if per_launch_flops else None
        roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak if achieved else None, "traffic": traffic,
                    "traffic_unit": "bytes per launch",
                    "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the Q and Z lists at "
                                       "n=6000 (0.0967 B per FP64-equivalent flop), scaled by this run's mean "
                                       "flops per launch; writes still dirty in L2 at kernel end are not counted "
                                       "(0.125 B/flop with them, the algorithmic figure)"),
                    "algorithmic_bytes": 0.125 * per_launch_flops if per_launch_flops else None,
                    "kernel": ("k_ws_apply<GeoS2G> (split-precision op lists of the Givens stage 2: dense "
                               "(r+nq)^2 blocks, FP16 digit MMAs)" if args.stage2 == "givens" else
                               "k_ws_apply<GeoS2> (split-precision compact-WY op lists, FP16 digit MMAs)"),
                    "work": ("2 len^2 FP64-equivalent flops per strip row per dense op" if args.stage2 == "givens" else
                             "4 len k FP64-equivalent flops per strip row per op") + ", x43 FP16 digit-pair products",
                    "peak_source": ("MEASURED_PEAKS.json bf16_tflops (FP16 and BF16 mma run at the same rate), of measured"
                                    if measured else "1.9 PFLOP/s BF16 burst, of fallback (no MEASURED_PEAKS.json)"),
                    "fp64_equivalent_tflops": fp64eq,
                    "aggregate": {"note": "achieved/frac divide by the mean launch duration (the contract's "
                                          "definition); launches on the four bulk streams overlap, so this "
                                          "divides the same flops by the time at least one launch ran",
                                  "busy_s_per_step": s2["busy_seconds"] / max(1, steps_done),
                                  "achieved": 43.0 * fp64eq_busy if fp64eq_busy else None,
                                  "frac": 43.0 * fp64eq_busy / peak if fp64eq_busy else None,
                                  "fp64_equivalent_tflops": fp64eq_busy},
                    "launches_per_step": s2["launches"] / max(1, steps_done),
                    "avg_launch_ms": 1e3 * s2["seconds"] / max(1, s2["launches"])}
    else:
        roofline = {"bound": "fp64", "achieved": fp64eq, "peak": fp64_peak, "unit": "TFLOP/s",
                    "frac": fp64eq / fp64_peak if fp64eq else None, "traffic": None,
                    "kernel": ("k_apply_left/k_apply_right<GeoS2G> (FP64 dense op lists of the Givens stage 2)"
                               if args.stage2 == "givens" else
                               "k_apply_left/k_apply_right<GeoS2> (FP64 compact-WY op lists)"),
                    "work": "4 len k flops per strip row per op",
                    "peak_source": "cuBLAS DGEMM 8192^3 measured in this run, of measured",
                    "aggregate": {"busy_s_per_step": s2["busy_seconds"] / max(1, steps_done),
                                  "achieved": fp64eq_busy,
                                  "frac": fp64eq_busy / fp64_peak if fp64eq_busy else None},
                    "launches_per_step": s2["launches"] / max(1, steps_done),
                    "avg_launch_ms": 1e3 * s2["seconds"] / max(1, s2["launches"])}

    if args.save_stage1 and rank == 0 and not stage2_only:
        from paraht_gb300 import pencilio

        restore()
        ctx.ab2rht_d(n, work[0].data_ptr(), n, work[1].data_ptr(), n, work[2].data_ptr(), n, work[3].data_ptr(), n,
                     r, p, flags & ph.PARAHT_FLAG_SPLIT)
        torch.cuda.synchronize()
        H1, T1, Q1, Z1 = (np.asfortranarray(w.cpu().numpy().T) for w in work)
        pencilio.save_pencil(args.save_stage1, H1, T1, Q1, Z1, stage=1, r=r, p=p, dist=args.dist,
                             precision=args.precision)

    cpu = cpu_dgghd3 = None
    if rank == 0 and not args.no_cpu_baseline and not stage2_only:
        ns = min(args.cpu_sample_n, n)
        ts = cpu_oracle_seconds(ns, r, p, nq, args.dist)
        cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
        cpu = {"value": ts * (n / ns) ** 3, "unit": "s", "cores": cores, "kind": "port", "sample_n": ns,
               "extrapolated": ns != n,
               "sample": f"CPU oracle (OpenMP restatement of the reference) at n={ns}: {ts:.2f} s, scaled by (n/{ns})^3"}
        nd = ns if elapsed() + 60.0 < args.budget_s + 200.0 else min(ns, 2000)
        td3 = cpu_dgghd3_seconds(nd, args.dist)
        cpu_dgghd3 = {"value": td3 * (n / nd) ** 3, "unit": "s", "cores": os.cpu_count() or 1, "sample_n": nd,
                      "extrapolated": nd != n,
                      "sample": f"LAPACK DGGHD3 (scipy's OpenBLAS, all cores) at n={nd}: {td3:.2f} s, scaled by (n/{nd})^3"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "s", "n_gpus": world, "steps": steps_done,
            "steps_requested": args.steps, "warmup": args.warmup,
            "warmup_detail": (f"{max(0, args.warmup - 1)} reductions at n={nw}, then 1 at n={n}"
                              if args.warmup > 0 else "none"),
            "ms_per_step": t_step * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": (f"stage 2 alone on the saved stage-1 output {args.stage2_from}, n={n}, "
                                    if stage2_only else "") +
                                   f"HT reduction of one pencil n={n} (A N(0,1), B triangular Gaussian R), "
                                   f"r={r} p={p} nq={nq}, {args.precision}, stage 2 {args.stage2}",
                       "n": n, "r": r, "p": p, "nq": nq, "precision": args.precision, "dist": args.dist,
                       "stage2": args.stage2,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs 8.2 GB >> L2; pristine input restored between steps outside the timed region",
                       "budget_s": args.budget_s},
            "e2e": ({"value": e2e_v, "unit": "s", "h2d_bytes_per_step": 4 * n * n * 8, "d2h_bytes_per_step": 4 * n * n * 8}
                    if e2e_v is not None else None),
            "gpu_launches": launches // max(1, steps_done),
            "effective_gflops": flops_nominal(n) / t_step / 1e9,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "cpu_dgghd3": cpu_dgghd3,
            "clocks": sampler.summary(),
            "wall_s": elapsed(),
        }
        if fp64 is not None:
            line["fp64"] = fp64
            line["split_vs_fp64"] = fp64["seconds"] / t_step
        if check:
            line["check"] = check
        if phases:
            line["phases_s"] = phases
        if chain:
            line["critical_path_s"] = chain
        print(json.dumps(line), flush=True)
    if dist_on:
        import torch.distributed as td

        td.destroy_process_group()
    ctx.close()
    return 0


def qz_pencil(n: int, seed: int):
    """A random Hessenberg-triangular pencil: H with N(0,1) entries on and above the subdiagonal,
    T upper triangular N(0,1) with diagonal entries of modulus 1 + |N(0,1)|."""
    rng = np.random.default_rng(seed)
    H = np.triu(rng.standard_normal((n, n)), -1)
    T = np.triu(rng.standard_normal((n, n)))
    T[np.diag_indices(n)] = np.sign(T.diagonal() + 0.5) * (1.0 + np.abs(rng.standard_normal(n)))
    return np.asfortranarray(H), np.asfortranarray(T)


def _qz_cpu_chunk(job):
    """Process-pool worker: LAPACK DHGEQZ (the oracle's, one BLAS thread) on the pencils (n, seed)
    of job, each generated as qz_pencil does; returns the seconds spent inside DHGEQZ."""
    from oracle import oracle as O

    O.set_blas_threads(1)
    spent = 0.0
    for n, seed in job:
        H, T = qz_pencil(n, seed)
        t0 = time.perf_counter()
        O.dhgeqz_eigs(H, T)
        spent += time.perf_counter() - t0
    return spent


def qz_cpu_rate(sizes, seeds, workers: int):
    """Pencils/s of LAPACK DHGEQZ over all the given pencils on `workers` processes (spawned, one
    BLAS thread each), the pencils dealt largest first to the least-loaded worker by n^3; the
    rate is the pencil count over the busiest worker's time inside DHGEQZ (pool start-up and
    pencil generation excluded)."""
    import concurrent.futures as cf
    import multiprocessing as mp

    jobs = [[] for _ in range(workers)]
    load = [0.0] * workers
    for i in sorted(range(len(sizes)), key=lambda i: -sizes[i]):
        w = min(range(workers), key=load.__getitem__)
        jobs[w].append((sizes[i], seeds[i]))
        load[w] += float(sizes[i]) ** 3
    with cf.ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
        spent = list(ex.map(_qz_cpu_chunk, jobs))
    return len(sizes) / max(spent)


def run_qz(args, rank: int, world: int, local: int):
    """--workload qz1216: generalized eigenvalues of 1216 Hessenberg-triangular pencils (152 SMs x 8,
    n ~ U{32..256}) in one paraht_hgeqz_eigs_d call, the QZ step after the reduction; LAPACK DHGEQZ
    (the oracle's) on the same pencils, one process per host core, is the CPU baseline."""
    from paraht_gb300.generate import batch_sizes

    count, lo, hi = 1216, 32, 256
    sizes = batch_sizes(count, lo, hi, "uniform", seed=replica_seed(4242, rank))
    n3 = statistics.mean(float(n) ** 3 for n in sizes)
    metric = "QZ eigenvalues: pencils/s, 1216 Hessenberg-triangular pencils n~U{32..256}"
    workload = (f"{count} random Hessenberg-triangular pencils, n ~U{{{lo}..{hi}}} (seeded), eigenvalues only, "
                "one paraht_hgeqz_eigs_d call (real double-shift QZ, a warp per pencil below n=128, a 2-warp CTA from there)")

    def cpu_rate(nsample):
        """DHGEQZ on all host cores over the whole batch, and on one core over its first nsample
        pencils (time per pencil scaled by the batch's mean n^3)."""
        from oracle import oracle as O

        O.set_blas_threads(1)
        per = []
        for i in range(nsample):
            H, T = qz_pencil(sizes[i], 9000 + i)
            t0 = time.perf_counter()
            O.dhgeqz_eigs(H, T)
            per.append((time.perf_counter() - t0) / float(sizes[i]) ** 3)
        one = 1.0 / (statistics.mean(per) * n3)
        cores = os.cpu_count() or 1
        v = qz_cpu_rate(sizes, [9000 + i for i in range(count)], cores)
        return v, {"value": v, "unit": "pencils/s", "cores": cores, "kind": "port", "one_core": one,
                   "sample": f"LAPACK DHGEQZ (eigenvalues only) on all {count} pencils, one process per core "
                             f"({cores}, one BLAS thread each, largest pencils first); one_core: the first "
                             f"{nsample} pencils on one core, time per pencil scaled by the batch's mean n^3"}

    if args.impl == "reference":
        if rank != 0:
            return 0
        vs = [cpu_rate(64) for _ in range(max(1, args.steps))]
        v = statistics.mean(x[0] for x in vs)
        print(json.dumps({
            "metric": metric, "value": v, "unit": "pencils/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * count / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload}, "cpu_baseline": {**vs[-1][1], "value": v},
            "e2e": {"value": v, "unit": "pencils/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}), flush=True)
        return 0

    import torch

    import paraht_gb300 as ph

    torch.cuda.set_device(local)
    dist_on = world > 1
    if dist_on:
        import torch.distributed as td

        td.init_process_group("nccl", device_id=torch.device("cuda", local))
    host = [qz_pencil(n, 9000 + i) for i, n in enumerate(sizes)]
    dH = [torch.from_numpy(np.ascontiguousarray(h.T)).cuda() for h, _ in host]
    dT = [torch.from_numpy(np.ascontiguousarray(t.T)).cuda() for _, t in host]
    out = [torch.zeros(3, n, dtype=torch.float64, device="cuda") for n in sizes]
    ctx = ph.Context(local)
    ptrs = ([x.data_ptr() for x in dH], [x.data_ptr() for x in dT], [o[0].data_ptr() for o in out],
            [o[1].data_ptr() for o in out], [o[2].data_ptr() for o in out])

    def call():
        return ctx.hgeqz_eigs_d(sizes, ptrs[0], sizes, ptrs[1], sizes, ptrs[2], ptrs[3], ptrs[4])

    def barrier():
        if dist_on:
            import torch.distributed as td

            td.barrier()

    for _ in range(args.warmup):
        call()
    ts, launches, infos = [], 0, []
    sampler = ClockSampler(local)
    with sampler:
        for _ in range(args.steps):
            barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            infos = call()  # synchronous: returns after the kernel and the status copy
            ts.append(time.perf_counter() - t0)
            launches += ctx.launch_count()
            barrier()
    t_step = job_time(statistics.mean(ts), "cuda")
    value = world * count / t_step
    # end to end through the host entry: pencils from host memory, eigenvalues back
    t0 = time.perf_counter()
    res = ph.hgeqz_eigs([h for h, _ in host], [t for _, t in host])
    e2e_v = world * count / (time.perf_counter() - t0)
    h2d = sum(2 * 8 * n * n for n in sizes)
    d2h = sum(3 * 8 * n for n in sizes)
    check = None
    cpu = None
    if rank == 0:
        from oracle import oracle as O

        def lam(alpha, beta):  # alpha / beta, infinite where beta = 0
            with np.errstate(divide="ignore", invalid="ignore"):
                return np.where(beta == 0.0, np.inf, alpha / np.where(beta == 0.0, 1.0, beta))

        worst, compared = 0.0, 0
        for i in range(32):
            a, b, inf = res[i]
            if inf:  # not converged: counted in info_nonzero below
                continue
            ar, ai, be, _ = O.dhgeqz_eigs(*host[i])
            worst = max(worst, eig_mismatch(lam(a, b), lam(ar + 1j * ai, be)))
            compared += 1
        check = {"pencils": compared, "eig_mismatch_vs_dhgeqz": worst, "info_nonzero": sum(1 for v in infos if v)}
        if not args.no_cpu_baseline:
            cpu = cpu_rate(64)[1]
        print(json.dumps({
            "metric": metric, "value": value, "unit": "pencils/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": workload, "pencils": count, "n_lo": lo, "n_hi": hi,
                       "l2": "working set about 0.5 GB of copies, above L2"},
            "e2e": {"value": e2e_v, "unit": "pencils/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": {"bound": "fp64", "achieved": None, "peak": None, "unit": None, "frac": None,
                         "traffic": None, "kernel": "k_qz_eigs: a warp or a 2-warp CTA per pencil; each pencil a serial "
                                                      "chain of dependent 3 x 3 reflectors, bound by its latency "
                                                      "and the FP64 issue rate; flops not counted"},
            "check": check, "cpu_baseline": cpu, "clocks": sampler.summary(),
        }), flush=True)
    if dist_on:
        import torch.distributed as td

        td.destroy_process_group()
    ctx.close()
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "qz1216":
        return run_qz(args, rank, world, local)
    if args.workload != "pencil":
        return run_batch(args, rank, world, local)
    if args.impl == "reference":
        return run_reference(args, rank)
    return run_pencil(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
