"""Multi-process (N > 1) logic of bench.py on CPU: world_size-2 gloo ranks on 127.0.0.1.

The reduction does not shard, so N ranks are replicas: each reduces its own pencils (distinct
seeds, no data exchange) and the job time is the maximum over ranks, obtained with one
all-reduce of a scalar.  No GPU is involved.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as td

    import bench

    td.init_process_group("gloo", rank=rank, world_size=world)
    t_local = [0.25, 0.75][rank]
    t = bench.job_time(t_local, "cpu")
    q.put((rank, t, bench.replica_seed(1302, rank)))
    td.destroy_process_group()


def test_two_gloo_ranks_take_the_max_and_distinct_seeds():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [t for _, t, _ in out] == [0.75, 0.75]
    assert out[0][2] != out[1][2]


def test_single_process_job_time_is_local():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.job_time(1.5, "cpu") == 1.5
