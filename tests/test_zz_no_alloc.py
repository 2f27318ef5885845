"""paraht_rht2ht_d_noalloc: stage 2 with its scratch in a fixed device array.

Some callers cannot let a library allocate device memory during a call: an application whose own
pool owns all device memory, or one that keeps work in flight that a cudaMalloc would
synchronise with.  The no-allocation entry point serves them.  It must give exactly the results
of paraht_rht2ht_d (same kernels, same arithmetic, only the scratch address differs) on calls in a
row (the fixed scratch keeps the previous call's contents, including calls of the allocating
entry in between), reject inputs whose scratch would not fit, and refuse the flags that would
allocate or create events.  The file name makes pytest collect it after the other tests.
"""
import numpy as np
import pytest

import paraht_gb300 as ph
from helpers import copies, make, oracle_reduce

pytestmark = pytest.mark.gpu

ERR_TOO_LARGE = -1008
ERR_NOT_SUPPORTED = -1005


def _dev(torch, X):
    return torch.from_numpy(np.ascontiguousarray(X.T)).cuda()


def _run(torch, fn, A, B, Q, Z, r, nq, flags=0):
    n = A.shape[0]
    dev = [_dev(torch, X) for X in (A, B, Q, Z)]
    fn(n, dev[0].data_ptr(), max(1, n), dev[1].data_ptr(), max(1, n), dev[2].data_ptr(), max(1, n),
       dev[3].data_ptr(), max(1, n), r, nq, flags)
    torch.cuda.synchronize()
    return [D.cpu().numpy().T for D in dev]


def _stage1(oracle, n, r, nq, shift=0):
    A0, B0 = make(n + shift)
    A0, B0 = np.asfortranarray(A0[:n, :n]), np.asfortranarray(np.triu(B0[:n, :n]))
    return oracle_reduce(oracle, A0, B0, r, 2, nq, stage=1)


@pytest.mark.parametrize("flags", [0, ph.PARAHT_FLAG_SEQUENTIAL])
@pytest.mark.parametrize("n,r,nq", [(150, 8, 8), (301, 16, 16)])
def test_noalloc_matches_rht2ht_d_twice(oracle, n, r, nq, flags):
    torch = pytest.importorskip("torch")
    ctx = ph.Context(0)
    for shift in (0, 1):  # two calls in a row on different inputs
        S1 = _stage1(oracle, n, r, nq, shift)
        ref = _run(torch, ctx.rht2ht_d, *copies(*S1), r, nq, flags)
        got = _run(torch, ctx.rht2ht_d_noalloc, *copies(*S1), r, nq, flags)
        for X, Y in zip(ref, got):
            assert np.array_equal(X, Y)
    ctx.close()


@pytest.mark.parametrize("n", [0, 1, 2, 3])
def test_noalloc_tiny_sizes(oracle, n):
    """n < 3: stage 2 has nothing to do (src/rht2ht.f90:1417); n = 3: one column."""
    torch = pytest.importorskip("torch")
    ctx = ph.Context(0)
    if n == 0:
        dev = torch.zeros((1, 1), dtype=torch.float64, device="cuda")
        ctx.rht2ht_d_noalloc(0, dev.data_ptr(), 1, dev.data_ptr(), 1, dev.data_ptr(), 1, dev.data_ptr(), 1, 2, 2)
        ctx.close()
        return
    S1 = _stage1(oracle, n, 2, 2)
    ref = _run(torch, ctx.rht2ht_d, *copies(*S1), 2, 2)
    got = _run(torch, ctx.rht2ht_d_noalloc, *copies(*S1), 2, 2)
    for X, Y in zip(ref, got):
        assert np.array_equal(X, Y)
    ctx.close()


def test_noalloc_after_allocating_entry_on_one_context(oracle):
    """noalloc, then rht2ht_d, then noalloc on the same context: the fixed scratch still holds the
    first call's progress words and reflectors, which must not leak into the third call."""
    torch = pytest.importorskip("torch")
    ctx = ph.Context(0)
    n, r, nq = 233, 16, 16
    S1a = _stage1(oracle, n, r, nq, 0)
    S1b = _stage1(oracle, n, r, nq, 2)
    first = _run(torch, ctx.rht2ht_d_noalloc, *copies(*S1a), r, nq)
    mid = _run(torch, ctx.rht2ht_d, *copies(*S1b), r, nq)
    last = _run(torch, ctx.rht2ht_d_noalloc, *copies(*S1b), r, nq)
    again = _run(torch, ctx.rht2ht_d, *copies(*S1a), r, nq)
    for X, Y in zip(mid, last):
        assert np.array_equal(X, Y)
    for X, Y in zip(first, again):
        assert np.array_equal(X, Y)
    ctx.close()


def test_noalloc_size_limit_boundary(oracle):
    """The scratch of (n, r = 16, nq = 16) fits up to n = 5313 exactly: 5313 runs (and matches the
    allocating entry), 5314 is refused before any device access."""
    torch = pytest.importorskip("torch")
    ctx = ph.Context(0)
    r = nq = 16
    with pytest.raises(ph.ParahtError) as e:  # pointers never dereferenced: refused up front
        ctx.rht2ht_d_noalloc(5314, 256, 5314, 256, 5314, 256, 5314, 256, 5314, r, nq)
    assert e.value.status == ERR_TOO_LARGE
    n = 5313
    rng = np.random.default_rng(5313)
    A = np.asfortranarray(np.triu(rng.standard_normal((n, n)), -r))  # r-Hessenberg
    B = np.asfortranarray(np.triu(rng.standard_normal((n, n))) + 4.0 * np.eye(n))
    I = np.asfortranarray(np.eye(n))
    got = _run(torch, ctx.rht2ht_d_noalloc, *copies(A, B, I, I), r, nq)
    ref = _run(torch, ctx.rht2ht_d, *copies(A, B, I, I), r, nq)
    for X, Y in zip(ref, got):
        assert np.array_equal(X, Y)
    ctx.close()


def test_noalloc_rejects_oversize_and_unsupported_flags():
    torch = pytest.importorskip("torch")
    ctx = ph.Context(0)
    n = 6000  # stage-2 scratch for r = nq = 16 exceeds the fixed array (8 MiB)
    dev = [torch.zeros((64, 64), dtype=torch.float64, device="cuda") for _ in range(4)]
    with pytest.raises(ph.ParahtError) as e:
        ctx.rht2ht_d_noalloc(n, dev[0].data_ptr(), n, dev[1].data_ptr(), n, dev[2].data_ptr(), n,
                             dev[3].data_ptr(), n, 16, 16)
    assert e.value.status == ERR_TOO_LARGE
    m = 64
    for f in (ph.PARAHT_FLAG_SPLIT, ph.PARAHT_FLAG_TIME_COMPONENTS, ph.PARAHT_FLAG_TIME_CHAIN, ph.PARAHT_FLAG_KERNEL_TIMES,
              ph.PARAHT_FLAG_BATCH_LOOP, 1 << 20):
        with pytest.raises(ph.ParahtError) as e:
            ctx.rht2ht_d_noalloc(m, dev[0].data_ptr(), m, dev[1].data_ptr(), m, dev[2].data_ptr(), m,
                                 dev[3].data_ptr(), m, 8, 8, f)
        assert e.value.status == ERR_NOT_SUPPORTED, f
    ctx.close()
