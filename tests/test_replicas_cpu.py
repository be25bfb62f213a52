"""The multi-GPU path of bench.py is replicas only: each rank evaluates its own
copy and the job rate is world * steps / (slowest rank's time).  These CPU
tests run the rank aggregation and the reference arm's rank handling as two
gloo processes (127.0.0.1), as torchrun would launch them."""
import os
import socket
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = 100.0 + 50.0 * rank          # rank 1 is the slower replica
        ms, value = bench.aggregate_replicas(local, 4, world)
        q.put((rank, ms, value))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for rank, ms, value in got:
        assert ms == 150.0                               # max over ranks
        assert value == pytest.approx(world * 4 / 0.150)  # whole-job rate


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_replicas(200.0, 10, 1) == (200.0, 10 / 0.2)


def test_reference_arm_other_ranks_exit_quietly(capsys):
    sys.path.insert(0, ROOT)
    import argparse

    import bench
    args = argparse.Namespace(n=1024, steps=1, warmup=0)
    bench.reference_arm(args, rank=1, world=2)
    assert capsys.readouterr().out == ""
