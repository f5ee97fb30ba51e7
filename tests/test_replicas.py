"""Multi-GPU form (independent replicas, one process per GPU): the host-side
aggregation over ranks, run as two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    from vkhashdag_gb300.replicas import replica_totals
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = replica_totals(10.0 + 5.0 * rank, 100.0 * (rank + 1))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_time_and_all_work():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    assert out[0] == out[1] == (15.0, 300.0)


def test_single_process_totals_are_local():
    from vkhashdag_gb300.replicas import replica_totals
    assert replica_totals(3.5, 7) == (3.5, 7.0)


def test_replicas_edit_different_seeded_batches():
    from vkhashdag_gb300 import workloads as W
    from vkhashdag_gb300.replicas import replica_seed
    a = W.mixed_batch(1024, 64, seed=replica_seed(0, 0))
    b = W.mixed_batch(1024, 64, seed=replica_seed(1, 0))
    c = W.mixed_batch(1024, 64, seed=replica_seed(0, 0))
    assert not np.array_equal(a, b) and np.array_equal(a, c)
