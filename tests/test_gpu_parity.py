"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle.

Tolerances (FP64 path):
* stage-level outputs (same input fed to both): elementwise relative difference <= 1e-9, since
  both follow the same sequence of Householder transformations and differ only by rounding;
* final pencil: backward errors and orthogonality <= 10*n*eps (the acceptance bound), |H|, |T|
  elementwise within 1e-8 of the oracle's (essential uniqueness: Q e1 = e1 on both sides);
* structure: exact zeros below the Hessenberg / triangular structure.
"""
import numpy as np
import pytest

import paraht_gb300 as ph
from helpers import EPS, abs_rel_max_diff, bwd, copies, eig_mismatch, make, oracle_reduce, orth, rel_max_diff
from paraht_gb300.generate import identity

pytestmark = pytest.mark.gpu

STAGE_CASES = [
    # n, r, p, nq
    (5, 2, 2, 2),
    (17, 3, 3, 2),
    (33, 4, 2, 3),
    (64, 8, 4, 4),
    (100, 16, 8, 8),
    (130, 8, 2, 8),
    (257, 16, 8, 8),
    (300, 16, 4, 16),
    (333, 32, 4, 8),
    (200, 32, 8, 8),    # L = 256: the general stage-1 generation kernels (beyond the fast ones' L <= 128)
    (300, 64, 4, 16),   # r = 64: the widest band, L = 256
]


@pytest.mark.parametrize("n,r,p,nq", STAGE_CASES)
def test_stage1_matches_oracle(oracle, n, r, p, nq):
    A0, B0 = make(n)
    Ao, Bo, Qo, Zo = oracle_reduce(oracle, A0, B0, r, p, nq, stage=1)
    A, B = copies(A0, B0)
    Q, Z = identity(n), identity(n)
    ph.ab2rht_simple(n, A, n, B, n, Q, n, Z, n, r, p, False)
    assert np.all(np.tril(A, -r - 1) == 0.0)
    assert np.all(np.tril(B, -1) == 0.0)
    # the oracle keeps roundoff below the structure; the GPU path zeroes it
    for X, Xo in ((A, np.triu(Ao, -r)), (B, np.triu(Bo)), (Q, Qo), (Z, Zo)):
        assert rel_max_diff(X, Xo) < 1e-9
    assert bwd(Q, A0, Z, A) <= 10 * n * EPS
    assert bwd(Q, B0, Z, B) <= 10 * n * EPS


@pytest.mark.parametrize("n,r,p,nq", STAGE_CASES)
def test_stage2_matches_oracle(oracle, n, r, p, nq):
    A0, B0 = make(n)
    A1, B1, Q1, Z1 = oracle_reduce(oracle, A0, B0, r, p, nq, stage=1)
    Ao, Bo, Qo, Zo = copies(A1, B1, Q1, Z1)
    oracle.rht2ht_householder(Ao, Bo, Qo, Zo, r, nq)
    A, B, Q, Z = copies(A1, B1, Q1, Z1)
    ph.rht2ht_householder(n, A, n, B, n, Q, n, Z, n, r, nq, False)
    assert np.all(np.tril(A, -2) == 0.0)
    assert np.all(np.tril(B, -1) == 0.0)
    assert rel_max_diff(A, np.triu(Ao, -1)) < 1e-9
    assert rel_max_diff(B, np.triu(Bo)) < 1e-9
    assert rel_max_diff(Q, Qo) < 1e-9
    assert rel_max_diff(Z, Zo) < 1e-9


@pytest.mark.parametrize("n,r,p,nq,dist", [
    (200, 16, 8, 8, "std"),
    (256, 8, 2, 4, "std_qr"),
    (180, 16, 4, 16, "graded"),
    (150, 4, 8, 3, "refcompat"),
])
def test_reduce_end_to_end(oracle, ctx, n, r, p, nq, dist):
    A0, B0 = make(n, dist)
    A, B = copies(A0, B0)
    Q, Z = identity(n), identity(n)
    ctx.reduce_host(A, B, Q, Z, r, p, nq, flags=ph.PARAHT_FLAG_TIME_COMPONENTS)
    tol = 10 * n * EPS
    assert bwd(Q, A0, Z, A) <= tol
    assert bwd(Q, B0, Z, B) <= tol
    assert orth(Q) <= tol and orth(Z) <= tol
    assert np.all(np.tril(A, -2) == 0.0) and np.all(np.tril(B, -1) == 0.0)
    Ao, Bo, Qo, Zo = oracle_reduce(oracle, A0, B0, r, p, nq)
    if dist != "graded":  # graded has a singular T: the HT form is no longer essentially unique
        assert abs_rel_max_diff(A, Ao) < 1e-8
        assert abs_rel_max_diff(B, Bo) < 1e-8
    t = ctx.phase_times()
    assert t["total"] > 0 and t["s1_genleft"] > 0 and t["s2_gen"] > 0


@pytest.mark.parametrize("flags", [0, ph.PARAHT_FLAG_SPLIT, ph.PARAHT_FLAG_SPLIT | ph.PARAHT_FLAG_GIVENS])
def test_time_chain_keeps_results_and_adds_up(ctx, flags):
    """PARAHT_FLAG_TIME_CHAIN times the phases on each stage's critical-path stream with the side
    streams still overlapped: bitwise the untimed results, and the six phases add up to the
    device time between the stages' first and last marks (within the total)."""
    n, r, p, nq = 600, 16, 4, 16
    A0, B0 = make(n)
    out = []
    for f in (flags, flags | ph.PARAHT_FLAG_TIME_CHAIN):
        A, B = copies(A0, B0)
        Q, Z = identity(n), identity(n)
        ctx.reduce_host(A, B, Q, Z, r, p, nq, flags=f)
        out.append((A, B, Q, Z))
    for X, Y in zip(*out):
        assert np.array_equal(X, Y)
    t = ctx.phase_times()
    parts = sum(t[k] for k in ("s1_genleft", "s1_genright", "s1_mul", "s2_gen", "s2_lookahead", "s2_application"))
    assert t["s1_genright"] > 0 and t["s2_gen"] > 0
    assert 0.5 * t["total"] < parts <= 1.01 * t["total"]


def test_reflector_scalars_newton(ctx):
    """The generation chains' branch-free reflector scalars (hardware rsqrt/rcp approximations
    refined by Newton-Raphson steps) against the exact values in extended precision: tau = 1 +
    |alpha|/nrm, scal = sign(alpha)/(|alpha| + nrm), beta = -sign(alpha) nrm, nrm = sqrt(alpha^2 +
    xnorm2), each within 4 ulps; tau = 0, scal = 1, beta = alpha when xnorm2 = 0."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    m = 100000
    alpha = rng.standard_normal(m) * 10.0 ** rng.uniform(-100, 100, m)
    xn2 = (rng.standard_normal(m) * 10.0 ** rng.uniform(-100, 100, m)) ** 2
    alpha[:50] = 0.0
    xn2[50:100] = 0.0
    xn2[100:150] = alpha[100:150] ** 2 * 1e-30  # tail far below alpha
    alpha[150:200] = alpha[150:200] * 1e-30     # alpha far below the tail
    da, dx = torch.from_numpy(alpha).cuda(), torch.from_numpy(xn2).cuda()
    out = torch.empty(3 * m, dtype=torch.float64, device="cuda")
    ctx.selftest_reflector(m, da.data_ptr(), dx.data_ptr(), out.data_ptr())
    tau, scal, beta = out.cpu().numpy().reshape(m, 3).T
    z = xn2 == 0.0
    assert np.all(tau[z] == 0.0) and np.all(scal[z] == 1.0) and np.array_equal(beta[z], alpha[z])
    a, x = alpha[~z].astype(np.longdouble), xn2[~z].astype(np.longdouble)
    nrm = np.sqrt(a * a + x)
    sg = np.where(np.signbit(alpha[~z]), -1.0, 1.0).astype(np.longdouble)
    ref = (1 + np.abs(a) / nrm, sg / (np.abs(a) + nrm), -sg * nrm)
    for got, want in zip((tau[~z], scal[~z], beta[~z]), ref):
        rel = np.abs((got.astype(np.longdouble) - want) / want)
        assert float(rel.max()) <= 4 * EPS


@pytest.mark.parametrize("n", [1, 2, 3, 4, 6, 9])
def test_tiny_sizes(oracle, n):
    r, p, nq = 2, 2, 2
    A0, B0 = make(n)
    A, B = copies(A0, B0)
    Q, Z = identity(n), identity(n)
    ph.reduce(A, B, Q, Z, r, p, nq)
    Ao, Bo, Qo, Zo = oracle_reduce(oracle, A0, B0, r, p, nq)
    assert rel_max_diff(np.abs(A), np.abs(np.triu(Ao, -1))) < 1e-10
    assert rel_max_diff(np.abs(B), np.abs(np.triu(Bo))) < 1e-10
    assert bwd(Q, A0, Z, A) <= 10 * max(n, 2) * EPS


def test_eigenvalues_match(oracle, ctx):
    n, r, p, nq = 120, 8, 4, 8
    A0, B0 = make(n)
    A, B = copies(A0, B0)
    Q, Z = identity(n), identity(n)
    ctx.reduce_host(A, B, Q, Z, r, p, nq)
    Ao, Bo, _, _ = oracle_reduce(oracle, A0, B0, r, p, nq)
    ar, ai, be, info = oracle.dhgeqz_eigs(A, B)
    aro, aio, beo, info2 = oracle.dhgeqz_eigs(Ao, Bo)
    assert info == 0 and info2 == 0
    assert eig_mismatch((ar + 1j * ai) / be, (aro + 1j * aio) / beo) < 1e-8


def test_nonfinite_input_rejected(ctx):
    n = 20
    A0, B0 = make(n)
    A, B = copies(A0, B0)
    A[3, 4] = np.nan
    with pytest.raises(ph.ParahtError) as e:
        ctx.reduce_host(A, B, identity(n), identity(n), 4, 2, 2, flags=ph.PARAHT_FLAG_CHECK_FINITE)
    assert e.value.status == -1004


def test_device_pointer_entry_matches_host(ctx):
    torch = pytest.importorskip("torch")
    n, r, p, nq = 160, 8, 4, 8
    A0, B0 = make(n)
    A, B = copies(A0, B0)
    Q, Z = identity(n), identity(n)
    ctx.reduce_host(A, B, Q, Z, r, p, nq)
    dev = [torch.from_numpy(np.ascontiguousarray(X.T)).cuda() for X in (A0, B0, identity(n), identity(n))]
    ctx.reduce_d(n, dev[0].data_ptr(), n, dev[1].data_ptr(), n, dev[2].data_ptr(), n, dev[3].data_ptr(), n, r, p, nq)
    torch.cuda.synchronize()
    for X, D in zip((A, B, Q, Z), dev):
        assert np.array_equal(X, D.cpu().numpy().T)


@pytest.mark.parametrize("n,r,nq", [(150, 8, 8), (233, 16, 16), (97, 4, 3)])
def test_pipelined_chase_bitwise_equals_sequential(ctx, oracle, n, r, nq):
    """The pipelined stage-2 schedule (one CTA per sweep, two-step lag, side stream for bulk
    updates) must perform exactly the reference-order arithmetic: bitwise equal outputs."""
    A0, B0 = make(n)
    A1, B1, Q1, Z1 = oracle_reduce(oracle, A0, B0, r, 2, nq, stage=1)
    outs = []
    for flags in (0, ph.PARAHT_FLAG_SEQUENTIAL):
        A, B, Q, Z = copies(A1, B1, Q1, Z1)
        ph_rht2ht_host(ctx, A, B, Q, Z, r, nq, flags)
        outs.append((A, B, Q, Z))
    for X, Y in zip(*outs):
        assert np.array_equal(X, Y)


def ph_rht2ht_host(ctx, A, B, Q, Z, r, nq, flags):
    import torch

    n = A.shape[0]
    dev = [torch.from_numpy(np.ascontiguousarray(X.T)).cuda() for X in (A, B, Q, Z)]
    ctx.rht2ht_d(n, dev[0].data_ptr(), n, dev[1].data_ptr(), n, dev[2].data_ptr(), n, dev[3].data_ptr(), n, r, nq,
                 flags)
    torch.cuda.synchronize()
    for X, D in zip((A, B, Q, Z), dev):
        X[:] = D.cpu().numpy().T


@pytest.mark.parametrize("n,r,p,nq,dist", [
    (100, 16, 2, 8, "std"),
    (257, 16, 4, 16, "std"),
    (300, 16, 3, 8, "graded"),
    (200, 8, 4, 8, "refcompat"),
])
def test_split_precision_reduce(oracle, ctx, n, r, p, nq, dist):
    """Split-precision (emulated FP64 on BF16 tensor cores) bulk updates: backward error and
    orthogonality <= 1e-13 (the split path's acceptance bound), exact structure, and the same
    HT pencil as the oracle up to signs."""
    A0, B0 = make(n, dist)
    A, B = copies(A0, B0)
    Q, Z = identity(n), identity(n)
    ctx.reduce_host(A, B, Q, Z, r, p, nq, flags=ph.PARAHT_FLAG_SPLIT)
    assert bwd(Q, A0, Z, A) <= 1e-13 and bwd(Q, B0, Z, B) <= 1e-13
    assert orth(Q) <= 1e-13 and orth(Z) <= 1e-13
    assert np.all(np.tril(A, -2) == 0.0) and np.all(np.tril(B, -1) == 0.0)
    if dist != "graded":
        Ao, Bo, _, _ = oracle_reduce(oracle, A0, B0, r, p, nq)
        assert abs_rel_max_diff(A, Ao) < 1e-8
        assert abs_rel_max_diff(B, Bo) < 1e-8
    assert ctx.launch_count() > 0


def _dev_run(torch, fn, mats, *args):
    n = mats[0].shape[0]
    dev = [torch.from_numpy(np.ascontiguousarray(X.T)).cuda() for X in mats]
    fn(n, dev[0].data_ptr(), n, dev[1].data_ptr(), n, dev[2].data_ptr(), n, dev[3].data_ptr(), n, *args)
    torch.cuda.synchronize()
    return [D.cpu().numpy().T for D in dev]


@pytest.mark.parametrize("n,r,p,nq", [
    (200, 8, 4, 8),    # stage 1 and 2 spans 32 / 16, k = 8: one-product form
    (300, 16, 3, 8),   # stage-1 span 48 (two products), stage-2 span 24, k = 8
    (300, 16, 4, 16),  # spans 64 / 32, k = 16
    (257, 16, 2, 4),   # stage-1 span 32, stage-2 span 20, k = 4
])
def test_split_stages_match_fp64(ctx, n, r, p, nq):
    """Each stage in split precision against the FP64 kernels on the same input: the split
    kernels (one-, two- and three-product forms, staircase masks) perform the same transformations
    to about FP64 accuracy."""
    torch = pytest.importorskip("torch")
    A0, B0 = make(n)
    I = identity(n)
    s1f = _dev_run(torch, ctx.ab2rht_d, [A0, B0, I, I], r, p, 0)
    s1s = _dev_run(torch, ctx.ab2rht_d, [A0, B0, I, I], r, p, ph.PARAHT_FLAG_SPLIT)
    for X, Y in zip(s1f, s1s):
        assert rel_max_diff(Y, X) < 1e-10
    s2f = _dev_run(torch, ctx.rht2ht_d, s1f, r, nq, 0)
    s2s = _dev_run(torch, ctx.rht2ht_d, s1f, r, nq, ph.PARAHT_FLAG_SPLIT)
    for X, Y in zip(s2f, s2s):
        assert rel_max_diff(Y, X) < 1e-10
