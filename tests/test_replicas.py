"""The multi-GPU path (replicas, weak scaling) on CPU: two gloo ranks
combine their cells and times as bench.py does (sum of cells over the
slowest rank's time), each rank with its own workload seed; and the
reference arm under torchrun prints on rank 0 only."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from saber_gb300.replicas import rank_seed, whole_job


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = [1_000_000, 3_000_000][rank]
        ms = [12.5, 10.0][rank]
        out[rank] = whole_job(units, ms, world) + (rank_seed(7, rank),)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_combine_as_weak_scaling():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        units, ms, seed = out[r]
        assert units == 4_000_000 and ms == 12.5
    assert out[0][2] != out[1][2]


def test_single_rank_is_local():
    assert whole_job(5, 2.0, 1) == (5.0, 2.0)
    assert rank_seed(0, 0) == 0 and rank_seed(0, 3) == 3000


def test_reference_arm_other_ranks_print_nothing(capsys, monkeypatch):
    import sys
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference"])
    bench.run_reference(bench.parse(), rank=1, world=2)
    assert capsys.readouterr().out == ""
