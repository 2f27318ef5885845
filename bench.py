#!/usr/bin/env python3
"""Headline benchmark: seconds for the two-stage HT reduction of one n=16000 pencil on one GB300.

Metric: "HT-reduction sec at n=16000: split-prec vs FP64 GPU at bwd err<=1e-13".
A step is one full reduction (stage 1 + stage 2, Q and Z accumulated) of the synthetic pencil
"std" (A ~ N(0,1), B the R factor of a Gaussian matrix, seed 1302) with the reference's
parameter surface (r, p, nq).  Arrays are column-major FP64 resident in HBM; the pristine input
is restored (device-to-device copy) before every step, outside the timed region.  The inputs
(4 x n^2 x 8 B = 8.2 GB at n=16000) are far larger than L2, so no extra L2 flush is needed.

* ``value``: mean device time per step (CUDA events on the library's stream, max over ranks).
* ``e2e``:   the same reduction through the public host entry point paraht_reduce_host with
             pinned host buffers, host<->device copies inside the timed region.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "HT-reduction sec at n=16000: split-prec vs FP64 GPU at bwd err<=1e-13"
EPS = float(np.finfo(np.float64).eps)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("paraht", "reference"), default="paraht")
    ap.add_argument("--workload", choices=("pencil", "batch4096", "batch256"), default="pencil",
                    help="pencil: one n x n pencil (the headline); batch4096: 4096 FP64 pencils, n ~ U{32..512}; "
                         "batch256: 256 pencils, n log-uniform in [256, 4096], 30%% graded, split precision")
    ap.add_argument("--loop-sample", type=int, default=0,
                    help="pencils of the looped baseline (batch workloads; 0: the workload's default)")
    ap.add_argument("--n", type=int, default=16000)
    ap.add_argument("--r", type=int, default=16)
    ap.add_argument("--p", type=int, default=4)
    ap.add_argument("--nq", type=int, default=16)
    ap.add_argument("--dist", default="std")
    ap.add_argument("--precision", choices=("fp64", "split"), default="split")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--cpu-sample-n", type=int, default=2500)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--check", action="store_true", help="also compute the backward error of the last step")
    ap.add_argument("--phases", action="store_true", help="one extra serialised step for the per-phase times")
    ap.add_argument("--save-stage1", default="", help="after the run, save this pencil's stage-1 output here")
    ap.add_argument("--stage2-from", default="", help="time stage 2 alone on a saved stage-1 output")
    return ap.parse_args()


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


def replica_seed(base: int, rank: int) -> int:
    """Seed of rank `rank`'s own input (replicas reduce different pencils of one distribution)."""
    return base + rank


def flops_nominal(n: int) -> float:
    # fixed nominal count used for "effective GFLOP/s" (stage 1 at p=8 plus stage 2): 18.67 n^3
    return 18.67 * float(n) ** 3


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


def run_reference(args, rank: int):
    """--impl reference: the CPU implementation of the path on the host cores."""
    if rank != 0:
        return 0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    ns = args.cpu_sample_n
    for _ in range(args.warmup):
        cpu_oracle_seconds(max(200, ns // 4), args.r, args.p, args.nq, args.dist)
    ts = [cpu_oracle_seconds(ns, args.r, args.p, args.nq, args.dist) for _ in range(max(1, args.steps))]
    scale = (args.n / ns) ** 3
    v = statistics.mean(ts) * scale
    line = {
        "metric": METRIC, "value": v, "unit": "s", "impl": "reference", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(ts) * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"HT reduction n={args.n} r={args.r} p={args.p} nq={args.nq} dist={args.dist}",
                   "n": args.n, "r": args.r, "p": args.p, "nq": args.nq},
        "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port",
                         "sample": f"oracle (C/OpenMP restatement of ab2rht_simple+rht2ht_householder, single-threaded "
                                   f"BLAS inside tasks) at n={ns}, mean of {len(ts)} runs, scaled by (n/{ns})^3"},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
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
                f"{'split-precision single-pencil path above n=1024' if spec['split'] else 'FP64'}, one paraht_reduce_batched_d call")

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

    # the batched call runs up to 8 worker contexts of 3 streams each beside the persistent
    # launch: ask for more hardware queues than CUDA's default 8 (read at context creation)
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

    def call(idx, f):
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
        achieved = flops / t_step / 1e12 * world
        print(json.dumps({
            "metric": spec["metric"], "value": value, "unit": "pencils/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload, "pencils": count, "n_lo": lo, "n_hi": hi, "size_law": spec["law"],
                       "graded_fraction": spec["graded"], "split": spec["split"],
                       "l2": "inputs >> L2; pristine inputs restored between steps outside the timed region"},
            "e2e": {"value": e2e_v, "unit": "pencils/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "looped_baseline": {"value": loop_v, "unit": "pencils/s", "sample": len(sample),
                                "note": "paraht_reduce_d per pencil, time per pencil scaled to the batch's mean n^3",
                                "speedup": value / world / loop_v},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": 1.19, "unit": "TFLOP/s",
                         "frac": achieved / 1.19, "traffic": None,
                         "kernel": "k_batch_reduce and the single-pencil kernels (nominal 18.67 n^3 flops per pencil)",
                         "peak_source": "FP64 FMA throughput measured on this pool's GB300 (fp64 probe)"},
            "bwd_err": {"max": errs_sorted[-1], "p99": errs_sorted[min(len(errs) - 1, int(0.99 * len(errs)))]},
            "cpu_baseline": cpu,
            "clocks": sampler.summary(),
        }), flush=True)
    ctx.close()
    if dist_on:
        import torch.distributed as td

        td.destroy_process_group()
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload != "pencil":
        return run_batch(args, rank, world, local)
    if args.impl == "reference":
        return run_reference(args, rank)

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
    flags = ph.PARAHT_FLAG_SPLIT if args.precision == "split" else 0
    stage2_only = bool(args.stage2_from)
    if stage2_only:  # a saved stage-1 output (paraht_gb300.pencilio): time stage 2 alone
        args.e2e_steps, args.check = 0, False
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

    def restore():
        with torch.cuda.stream(stream):
            work[0].copy_(dev0[0])
            work[1].copy_(dev0[1])
            work[2].copy_(qz0[0])
            work[3].copy_(qz0[1])
        stream.synchronize()

    def step(f=flags):
        ptrs = (n, work[0].data_ptr(), n, work[1].data_ptr(), n, work[2].data_ptr(), n, work[3].data_ptr(), n)
        if stage2_only:
            ctx.rht2ht_d(*ptrs, r, nq, f)
        else:
            ctx.reduce_d(*ptrs, r, p, nq, f)

    # host-pointer entry point (the reference-facing call): pinned host buffers, copies inside
    hostA = torch.from_numpy(np.asfortranarray(A0).T.copy()).pin_memory()
    hostB = torch.from_numpy(np.asfortranarray(B0).T.copy()).pin_memory()
    hostQ = torch.empty((n, n), dtype=torch.float64).pin_memory()
    hostZ = torch.empty((n, n), dtype=torch.float64).pin_memory()

    def host_step():
        hostA.copy_(torch.from_numpy(np.asfortranarray(A0).T))
        hostB.copy_(torch.from_numpy(np.asfortranarray(B0).T))
        hostQ.copy_(torch.eye(n, dtype=torch.float64))
        hostZ.copy_(torch.eye(n, dtype=torch.float64))
        nA, nB, nQ, nZ = (x.numpy().T for x in (hostA, hostB, hostQ, hostZ))  # Fortran-ordered views
        barrier()
        t0 = time.perf_counter()
        ctx.reduce_host(nA, nB, nQ, nZ, r, p, nq, flags)
        return time.perf_counter() - t0

    # warm-up: the last one goes through the host entry point (sizes its staging buffers)
    for i in range(args.warmup):
        if i == args.warmup - 1 and args.e2e_steps > 0:
            host_step()
        else:
            restore()
            step()
    torch.cuda.synchronize()
    ms = []
    launches = 0
    kst = {"stage1": {"seconds": 0.0, "launches": 0, "flops": 0.0}, "stage2": {"seconds": 0.0, "launches": 0, "flops": 0.0}}
    sampler = ClockSampler(local)
    with sampler:
        for _ in range(args.steps):
            restore()
            barrier()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(flags | ph.PARAHT_FLAG_KERNEL_TIMES)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            launches += ctx.launch_count()
            st = ctx.kernel_stats()
            for k in kst:
                for f in kst[k]:
                    kst[k][f] += st[k][f]
            barrier()
    t_step = statistics.mean(ms) / 1e3
    t_step = job_time(t_step, "cuda")
    value = t_step / world

    # backward error of the last timed step (outside the timed region)
    check = None
    if args.check:
        H, T, Q, Z = work[0].T, work[1].T, work[2].T, work[3].T
        Af, Bf = dev0[0].T, dev0[1].T  # column-major data stored as row-major transposes
        ea = float(torch.linalg.norm(Q.T @ Af @ Z - H) / torch.linalg.norm(Af))
        eb = float(torch.linalg.norm(Q.T @ Bf @ Z - T) / torch.linalg.norm(Bf))
        check = {"bwd_err_A": ea, "bwd_err_B": eb, "bound_10n_eps": 10 * n * EPS}

    # end to end through the host entry point, copies inside the timed region
    e2e_v = statistics.mean([host_step() for _ in range(args.e2e_steps)]) / world if args.e2e_steps > 0 else None

    phases = None
    if args.phases:  # time_components serialises the streams: one extra, slower step
        restore()
        step(flags | ph.PARAHT_FLAG_TIME_COMPONENTS)
        phases = {k: round(v, 4) for k, v in ctx.phase_times().items()}

    # roofline of the dominant kernel: the compact-WY op-list kernel of stage 2 (bulk and
    # lookahead updates), timed launch by launch with CUDA events on its streams during the timed
    # steps; its algorithmic work is 4 len k FP64-equivalent flops per strip row per op
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    s2 = kst["stage2"]
    if args.precision == "split":
        # each FP64-equivalent flop is 43 FP16 digit-pair flops on the tensor cores (pairs t+u <= 8)
        measured = "bf16_tflops" in peaks
        peak = float(peaks["bf16_tflops"]) if measured else 1900.0
        achieved = 43.0 * s2["flops"] / s2["seconds"] / 1e12 if s2["seconds"] > 0 else None
        roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak if achieved else None, "traffic": None,
                    "kernel": "k_ws_apply<GeoS2> (split-precision compact-WY op lists, FP16 digit MMAs)",
                    "peak_source": ("MEASURED_PEAKS.json bf16_tflops (FP16 and BF16 mma run at the same rate), of measured"
                                    if measured else "1.9 PFLOP/s BF16 burst, of fallback (no MEASURED_PEAKS.json)"),
                    "fp64_equivalent_tflops": s2["flops"] / s2["seconds"] / 1e12 if s2["seconds"] > 0 else None,
                    "launches_per_step": s2["launches"] / max(1, args.steps),
                    "avg_launch_ms": 1e3 * s2["seconds"] / max(1, s2["launches"])}
    else:
        fp64_peak = 1.19  # TFLOP/s, FP64 FMA throughput measured on this machine's GB300
        roofline = {"bound": "fp64", "achieved": None, "peak": fp64_peak, "unit": "TFLOP/s", "frac": None,
                    "traffic": None, "kernel": "k_apply_left/k_apply_right (FP64 compact-WY op lists)",
                    "peak_source": "FP64 FMA throughput measured on this pool's GB300 (fp64 probe)"}

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
        ns = args.cpu_sample_n
        ts = cpu_oracle_seconds(ns, r, p, nq, args.dist)
        cpu = {"value": ts * (n / ns) ** 3, "unit": "s", "cores": int(os.environ.get("OMP_NUM_THREADS",
                                                                                        os.cpu_count() or 1)),
               "kind": "port",
               "sample": f"CPU oracle (OpenMP restatement of the reference) at n={ns}: {ts:.2f} s, scaled by (n/{ns})^3"}
        td3 = cpu_dgghd3_seconds(ns, args.dist)
        cpu_dgghd3 = {"value": td3 * (n / ns) ** 3, "unit": "s", "cores": os.cpu_count() or 1,
                      "sample": f"LAPACK DGGHD3 (scipy's OpenBLAS, all cores) at n={ns}: {td3:.2f} s, scaled by (n/{ns})^3"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": (f"stage 2 alone on the saved stage-1 output {args.stage2_from}, n={n}, "
                                    if stage2_only else "") +
                                   f"HT reduction of one pencil n={n} (A N(0,1), B triangular Gaussian R), "
                                   f"r={r} p={p} nq={nq}, {args.precision}",
                       "n": n, "r": r, "p": p, "nq": nq, "precision": args.precision, "dist": args.dist,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs 8.2 GB >> L2; pristine input restored between steps outside the timed region"},
            "e2e": ({"value": e2e_v, "unit": "s", "h2d_bytes_per_step": 4 * n * n * 8, "d2h_bytes_per_step": 4 * n * n * 8}
                    if e2e_v is not None else None),
            "gpu_launches": launches,
            "effective_gflops": flops_nominal(n) / t_step / 1e9,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "cpu_dgghd3": cpu_dgghd3,
            "clocks": sampler.summary(),
        }
        if check:
            line["check"] = check
        if phases:
            line["phases_s"] = phases
        print(json.dumps(line), flush=True)
    if dist_on:
        import torch.distributed as td

        td.destroy_process_group()
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
