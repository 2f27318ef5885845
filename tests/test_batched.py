"""Batched reduction (paraht_reduce_batched_d): many pencils of uneven size in one call.

* pencils the persistent kernel takes (p r <= 64, n <= PARAHT_BATCH_MAX_N) must come out
  bitwise equal to paraht_reduce_d on the same pencil (same device bodies, same per-entry
  operation order, FP64 also when PARAHT_FLAG_SPLIT is set);
* pencils it does not take go through paraht_reduce_d inside the same call;
* PARAHT_FLAG_BATCH_LOOP (the looped baseline) gives the same bits;
* against the oracle: backward error <= 10 n eps and the same |H|, |T| (essential uniqueness).
"""
import numpy as np
import pytest

import paraht_gb300 as ph
from helpers import EPS, abs_rel_max_diff, bwd, make, oracle_reduce, orth
from paraht_gb300.generate import identity

pytestmark = pytest.mark.gpu

# n, r, p, nq, dist: persistent-kernel pencils of several shapes, edge sizes, graded pencils,
# and three the kernel does not take (p r = 128), which run concurrently on worker contexts
CASES = [
    (1, 2, 2, 2, "std"),
    (3, 2, 2, 2, "std"),
    (17, 3, 3, 2, "std"),
    (40, 4, 4, 4, "std"),
    (97, 8, 4, 8, "std"),
    (130, 16, 4, 16, "std"),
    (200, 16, 2, 8, "graded"),
    (257, 16, 4, 16, "std"),
    (64, 32, 2, 16, "std"),
    (150, 32, 4, 16, "std"),
    (120, 32, 4, 8, "std"),
    (90, 16, 8, 16, "graded"),
]


def _dev(torch, X):
    return torch.from_numpy(np.ascontiguousarray(X.T)).cuda()


def _inputs():
    out = []
    for i, (n, r, p, nq, dist) in enumerate(CASES):
        A0, B0 = make(max(n, 2), dist, seed=1302 + i)
        out.append((A0[:n, :n].copy(order="F"), np.triu(B0[:n, :n]).copy(order="F")))
    return out


def _run_batched(torch, ctx, inputs, flags):
    dev = [[_dev(torch, X) for X in (A0, B0, identity(A0.shape[0]), identity(A0.shape[0]))] for A0, B0 in inputs]
    ns = [c[0] for c in CASES]
    ld = [max(1, n) for n in ns]
    ptr = lambda j: [d[j].data_ptr() for d in dev]  # noqa: E731
    ctx.reduce_batched_d(ns, ptr(0), ld, ptr(1), ld, ptr(2), ld, ptr(3), ld, [c[1] for c in CASES],
                         [c[2] for c in CASES], [c[3] for c in CASES], flags)
    torch.cuda.synchronize()
    return [[D.cpu().numpy().T for D in d] for d in dev]


def _run_single(torch, ctx, A0, B0, r, p, nq, flags):
    n = A0.shape[0]
    dev = [_dev(torch, X) for X in (A0, B0, identity(n), identity(n))]
    ctx.reduce_d(n, dev[0].data_ptr(), max(1, n), dev[1].data_ptr(), max(1, n), dev[2].data_ptr(), max(1, n),
                 dev[3].data_ptr(), max(1, n), r, p, nq, flags)
    torch.cuda.synchronize()
    return [D.cpu().numpy().T for D in dev]


@pytest.mark.parametrize("flags", [0, ph.PARAHT_FLAG_BATCH_LOOP])
def test_batched_bitwise_equals_single(ctx, flags):
    torch = pytest.importorskip("torch")
    inputs = _inputs()
    got = _run_batched(torch, ctx, inputs, flags)
    for (n, r, p, nq, dist), (A0, B0), out in zip(CASES, inputs, got):
        ref = _run_single(torch, ctx, A0, B0, r, p, nq, 0)
        for X, Y in zip(out, ref):
            assert np.array_equal(X, Y), (n, r, p, nq, dist)


def test_batched_split_flag_small_pencils_fp64(ctx):
    """With PARAHT_FLAG_SPLIT the persistent kernel still computes in FP64 (same bits as the
    plain single-pencil path); the pencil it does not take uses the split single path."""
    torch = pytest.importorskip("torch")
    inputs = _inputs()
    got = _run_batched(torch, ctx, inputs, ph.PARAHT_FLAG_SPLIT)
    for (n, r, p, nq, dist), (A0, B0), out in zip(CASES, inputs, got):
        taken = n <= ph.PARAHT_BATCH_MAX_N and p * r <= 64
        ref = _run_single(torch, ctx, A0, B0, r, p, nq, 0 if taken else ph.PARAHT_FLAG_SPLIT)
        for X, Y in zip(out, ref):
            assert np.array_equal(X, Y), (n, r, p, nq, dist)


def test_batched_against_oracle(ctx, oracle):
    torch = pytest.importorskip("torch")
    inputs = _inputs()
    got = _run_batched(torch, ctx, inputs, 0)
    for (n, r, p, nq, dist), (A0, B0), (H, T, Q, Z) in zip(CASES, inputs, got):
        if n < 3:
            continue
        tol = 10 * n * EPS
        assert bwd(Q, A0, Z, H) <= tol and bwd(Q, B0, Z, T) <= tol, (n, r, p, nq)
        assert orth(Q) <= tol and orth(Z) <= tol
        assert np.all(np.tril(H, -2) == 0.0) and np.all(np.tril(T, -1) == 0.0)
        if dist == "std":
            Ho, To, _, _ = oracle_reduce(oracle, A0, B0, r, p, nq)
            assert abs_rel_max_diff(H, Ho) < 1e-8 and abs_rel_max_diff(T, To) < 1e-8, (n, r, p, nq)


def test_batched_rejects_bad_arguments(ctx):
    with pytest.raises(ph.ParahtError) as e:
        ctx.reduce_batched_d([10], [0], [10], [0], [10], [0], [10], [0], [10], [4], [2], [2])
    assert e.value.status == -3
    ctx.reduce_batched_d([], [], [], [], [], [], [], [], [], [], [], [])  # empty batch is a no-op


@pytest.mark.parametrize("order", ["given", "reversed"])
def test_batch_plan_graph_replays_bitwise(ctx, order):
    """paraht_batch_plan_*: the persistent launches captured as a CUDA graph (one bucket per
    (r, p, nq)) and replayed twice on new values in the same arrays give paraht_reduce_d's bits.
    Both bucket orders: a bucket with smaller tiles created after a larger one must not lower the
    shared-memory limit the larger one's captured launch needs."""
    torch = pytest.importorskip("torch")
    cases = [c for c in CASES if c[1] * c[2] <= 64]  # the pencils the persistent kernel takes
    if order == "reversed":
        cases = cases[::-1]
    ns = [c[0] for c in cases]
    ld = [max(1, n) for n in ns]
    rs, ps, nqs = [c[1] for c in cases], [c[2] for c in cases], [c[3] for c in cases]
    assert len(set(zip(rs, ps, nqs))) >= 3  # several buckets
    dev = [[torch.zeros((max(n, 1), max(n, 1)), dtype=torch.float64, device="cuda") for _ in range(4)] for n in ns]
    ptr = lambda j: [d[j].data_ptr() for d in dev]  # noqa: E731
    plan = ctx.batch_plan(ns, ptr(0), ld, ptr(1), ld, ptr(2), ld, ptr(3), ld, rs, ps, nqs)
    stream = torch.cuda.Stream()
    for rep in range(2):  # two replays on different inputs
        ref = []
        for k, (n, r, p, nq, dist) in enumerate(cases):
            A0, B0 = make(max(n, 2), dist, seed=7000 + 13 * rep + k)
            A0, B0 = A0[:n, :n].copy(order="F"), np.triu(B0[:n, :n]).copy(order="F")
            for j, X in enumerate((A0, B0, identity(n), identity(n))):
                dev[k][j].copy_(_dev(torch, X))
            ref.append(_run_single(torch, ctx, A0, B0, r, p, nq, 0))
        torch.cuda.synchronize()
        plan.launch(stream.cuda_stream)
        stream.synchronize()
        for k in range(len(cases)):
            for X, D in zip(ref[k], dev[k]):
                assert np.array_equal(X, D.cpu().numpy().T)
    plan.close()


def test_batch_plan_rejects_what_the_persistent_kernel_cannot_take(ctx):
    torch = pytest.importorskip("torch")
    X = torch.zeros((64, 64), dtype=torch.float64, device="cuda")
    p = X.data_ptr()
    for n, r, pp, nq, flags in ((64, 16, 8, 16, 0),            # p r = 128
                                (2000, 16, 4, 16, 0),          # n > PARAHT_BATCH_MAX_N
                                (64, 16, 4, 16, ph.PARAHT_FLAG_SPLIT)):
        with pytest.raises(ph.ParahtError) as e:
            ctx.batch_plan([n], [p], [n], [p], [n], [p], [n], [p], [n], [r], [pp], [nq], flags)
        assert e.value.status == -1005
