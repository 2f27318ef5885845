"""GPU parity of the Givens stage 2 (PARAHT_FLAG_GIVENS, paraht_rht2ht_givens) against the oracle's
restatement of src/rht2ht.f90:696-1344.

The GPU path applies the same rotations but accumulates each block's rotations on the fly and
applies the delayed left rotations as one product with U(ib), and forms a column's rotations from
a suffix sum of squares instead of a chain of DLARTG calls: the same transformations with other
rounding.  Tolerances: stage-level outputs (same input to both) elementwise within 1e-9 of the
oracle's; backward error and orthogonality within 10 n eps (1e-13 for the split path); exact zeros
below the structure; the Householder stage 2's H, T up to row/column signs within 1e-8.
"""
import numpy as np
import pytest

import paraht_gb300 as ph
from helpers import EPS, abs_rel_max_diff, bwd, copies, make, oracle_reduce, orth, rel_max_diff

pytestmark = pytest.mark.gpu

CASES = [
    # n, r, p, nq
    (5, 2, 2, 2),
    (17, 3, 3, 2),
    (33, 4, 2, 3),
    (64, 8, 4, 4),
    (100, 16, 8, 8),
    (257, 16, 4, 16),
    (300, 32, 4, 16),
    (333, 32, 2, 32),
]


@pytest.mark.parametrize("n,r,p,nq", CASES)
def test_givens_stage2_matches_oracle(oracle, n, r, p, nq):
    A0, B0 = make(n)
    A1, B1, Q1, Z1 = oracle_reduce(oracle, A0, B0, r, p, nq, stage=1)
    Ao, Bo, Qo, Zo = copies(A1, B1, Q1, Z1)
    oracle.rht2ht_givens(Ao, Bo, Qo, Zo, r, nq)
    A, B, Q, Z = copies(A1, B1, Q1, Z1)
    ph.rht2ht_givens(n, A, n, B, n, Q, n, Z, n, r, nq)
    assert np.all(np.tril(A, -2) == 0.0) and np.all(np.tril(B, -1) == 0.0)
    assert rel_max_diff(A, np.triu(Ao, -1)) < 1e-9
    assert rel_max_diff(B, np.triu(Bo)) < 1e-9
    assert rel_max_diff(Q, Qo) < 1e-9
    assert rel_max_diff(Z, Zo) < 1e-9
    tol = 10 * max(n, 2) * EPS
    assert bwd(Q, A0, Z, A) <= tol and bwd(Q, B0, Z, B) <= tol


def _dev_rht2ht(torch, ctx, mats, r, nq, flags):
    n = mats[0].shape[0]
    dev = [torch.from_numpy(np.ascontiguousarray(X.T)).cuda() for X in mats]
    ctx.rht2ht_d(n, dev[0].data_ptr(), n, dev[1].data_ptr(), n, dev[2].data_ptr(), n, dev[3].data_ptr(), n, r, nq,
                 flags)
    torch.cuda.synchronize()
    return [D.cpu().numpy().T for D in dev]


@pytest.mark.parametrize("n,r,nq", [(150, 8, 8), (233, 16, 16), (97, 4, 3)])
def test_givens_pipelined_bitwise_equals_sequential(ctx, oracle, n, r, nq):
    """The pipelined chase (one CTA per sweep, two-step lag, four bulk streams) performs exactly the
    arithmetic of the one-CTA, one-stream schedule."""
    torch = pytest.importorskip("torch")
    A0, B0 = make(n)
    S1 = oracle_reduce(oracle, A0, B0, r, 2, nq, stage=1)
    f0 = ph.PARAHT_FLAG_GIVENS
    outs = [_dev_rht2ht(torch, ctx, copies(*S1), r, nq, f) for f in (f0, f0 | ph.PARAHT_FLAG_SEQUENTIAL)]
    for X, Y in zip(*outs):
        assert np.array_equal(X, Y)


@pytest.mark.parametrize("n,r,p,nq,dist", [(400, 16, 4, 16, "std"), (300, 16, 3, 8, "graded"), (257, 8, 4, 8, "refcompat"),
                                           (420, 32, 4, 16, "std"), (380, 24, 3, 24, "graded")])
def test_givens_reduce_end_to_end(oracle, ctx, n, r, p, nq, dist):
    A0, B0 = make(n, dist)
    for flags, tol in ((ph.PARAHT_FLAG_GIVENS, 10 * n * EPS), (ph.PARAHT_FLAG_GIVENS | ph.PARAHT_FLAG_SPLIT, 1e-13)):
        A, B = copies(A0, B0)
        Q, Z = np.asfortranarray(np.eye(n)), np.asfortranarray(np.eye(n))
        ctx.reduce_host(A, B, Q, Z, r, p, nq, flags=flags)
        assert bwd(Q, A0, Z, A) <= tol and bwd(Q, B0, Z, B) <= tol
        assert orth(Q) <= tol and orth(Z) <= tol
        assert np.all(np.tril(A, -2) == 0.0) and np.all(np.tril(B, -1) == 0.0)
        if dist != "graded":  # graded B is singular: the HT form is not essentially unique
            Ah, Bh, _, _ = oracle_reduce(oracle, A0, B0, r, p, nq)
            assert abs_rel_max_diff(A, Ah) < 1e-8 and abs_rel_max_diff(B, np.triu(Bh)) < 1e-8


@pytest.mark.parametrize("n,r,nq", [
    (300, 16, 16),  # dense ops 32 wide: the one-product form
    (301, 24, 8),   # 32 wide, ragged last block
    (300, 32, 16),  # 48 wide: the wide dense form
    (317, 24, 24),  # 48 wide, ragged
    (290, 20, 20),  # 40 wide: three k-steps, the last one partly empty
])
def test_givens_split_matches_fp64(ctx, oracle, n, r, nq):
    """The split-precision dense ops (one-product forms) against the FP64 dense ops, same input."""
    torch = pytest.importorskip("torch")
    A0, B0 = make(n)
    S1 = oracle_reduce(oracle, A0, B0, r, 4, nq, stage=1)
    f = _dev_rht2ht(torch, ctx, copies(*S1), r, nq, ph.PARAHT_FLAG_GIVENS)
    s = _dev_rht2ht(torch, ctx, copies(*S1), r, nq, ph.PARAHT_FLAG_GIVENS | ph.PARAHT_FLAG_SPLIT)
    for X, Y in zip(f, s):
        assert rel_max_diff(Y, X) < 1e-10


def test_givens_unsupported_parameters(ctx):
    n = 80
    A0, B0 = make(n)
    A, B = copies(A0, B0)
    I = np.asfortranarray(np.eye(n))
    with pytest.raises(ph.ParahtError) as e:  # r > 32
        ph.rht2ht_givens(n, A, n, B, n, I.copy(order="F"), n, I.copy(order="F"), n, 40, 8)
    assert e.value.status == -1005
    with pytest.raises(ph.ParahtError) as e:  # the batched entry chases with reflectors only
        ctx.reduce_batched_d([4], [1], [4], [1], [4], [1], [4], [1], [4], [2], [2], [2], ph.PARAHT_FLAG_GIVENS)
    assert e.value.status == -1005
