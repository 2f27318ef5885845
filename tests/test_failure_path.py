"""Failure detection without a GPU fault: the pipelined chase's bounded wait, run on a progress
word that nothing sets, must give up after its poll limit, report PARAHT_ERR_TIMEOUT through the
status word, and leave the context usable for the next reduction."""
import numpy as np
import pytest

import paraht_gb300 as ph
from helpers import EPS, bwd, copies, make
from paraht_gb300.generate import identity

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(ctx):
    assert ctx.selftest_wait_timeout(2000) == -1003
    n, r, p, nq = 90, 8, 4, 8
    A0, B0 = make(n)
    A, B = copies(A0, B0)
    Q, Z = identity(n), identity(n)
    ctx.reduce_host(A, B, Q, Z, r, p, nq)
    assert bwd(Q, A0, Z, A) <= 10 * n * EPS and bwd(Q, B0, Z, B) <= 10 * n * EPS


def test_selftest_rejects_unbounded_limits(ctx):
    assert ctx.selftest_wait_timeout(0) == -2
    assert ctx.selftest_wait_timeout(1 << 21) == -2
