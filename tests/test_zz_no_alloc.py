"""paraht_rht2ht_d_noalloc: stage 2 with its scratch in a fixed device array.

It must give exactly the results of paraht_rht2ht_d (same kernels, same arithmetic, only the
scratch address differs), on two calls in a row (the fixed scratch is reused), and reject inputs
whose scratch would not fit.  The file name makes pytest collect it after the other tests.
"""
import numpy as np
import pytest

import paraht_gb300 as ph
from helpers import copies, make, oracle_reduce

pytestmark = pytest.mark.gpu


def _dev(torch, X):
    return torch.from_numpy(np.ascontiguousarray(X.T)).cuda()


def _run(torch, fn, A, B, Q, Z, r, nq):
    n = A.shape[0]
    dev = [_dev(torch, X) for X in (A, B, Q, Z)]
    fn(n, dev[0].data_ptr(), n, dev[1].data_ptr(), n, dev[2].data_ptr(), n, dev[3].data_ptr(), n, r, nq)
    torch.cuda.synchronize()
    return [D.cpu().numpy().T for D in dev]


@pytest.mark.parametrize("n,r,nq", [(150, 8, 8), (301, 16, 16)])
def test_noalloc_matches_rht2ht_d_twice(oracle, n, r, nq):
    torch = pytest.importorskip("torch")
    ctx = ph.Context(0)
    for seed_shift in (0, 1):  # two calls in a row on different inputs
        A0, B0 = make(n + seed_shift)
        A0, B0 = A0[:n, :n].copy(), np.triu(B0[:n, :n]).copy()
        A1, B1, Q1, Z1 = oracle_reduce(oracle, A0, B0, r, 2, nq, stage=1)
        ref = _run(torch, ctx.rht2ht_d, *copies(A1, B1, Q1, Z1), r, nq)
        got = _run(torch, ctx.rht2ht_d_noalloc, *copies(A1, B1, Q1, Z1), r, nq)
        for X, Y in zip(ref, got):
            assert np.array_equal(X, Y)


def test_noalloc_rejects_oversize_and_unsupported_flags():
    torch = pytest.importorskip("torch")
    ctx = ph.Context(0)
    n = 6000  # stage-2 scratch for r = nq = 16 exceeds the fixed array (8 MiB)
    dev = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for _ in range(4)]
    with pytest.raises(ph.ParahtError) as e:
        ctx.rht2ht_d_noalloc(n, dev[0].data_ptr(), n, dev[1].data_ptr(), n, dev[2].data_ptr(), n,
                             dev[3].data_ptr(), n, 16, 16)
    assert e.value.status == -1008
    m = 64
    with pytest.raises(ph.ParahtError) as e:
        ctx.rht2ht_d_noalloc(m, dev[0].data_ptr(), n, dev[1].data_ptr(), n, dev[2].data_ptr(), n,
                             dev[3].data_ptr(), n, 8, 8, ph.PARAHT_FLAG_SPLIT)
    assert e.value.status == -1005
