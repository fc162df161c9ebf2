"""The multi-GPU path of the benchmark is independent replicas: no collective on
the data path, only a barrier and the max over ranks of the timed region.
Checked here with two gloo ranks on the CPU (bench.slowest_rank /
replica_throughput)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        t = bench.slowest_rank([1.0 + rank, 10.0 - rank], world)
        out[rank] = (t, bench.replica_throughput(world, 30, t[0]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for rank in (0, 1):
        t, v = res[rank]
        assert t == [2.0, 10.0]  # max over ranks of each entry
        assert v == pytest.approx(2 * 30 / 2.0)


def test_single_rank_is_identity():
    assert bench.slowest_rank([1.5, 2.5], 1) == [1.5, 2.5]
    assert bench.replica_throughput(1, 10, 2.0) == 5.0


def test_bench_reads_the_committed_profile_traffic():
    """The bench's roofline `traffic` comes from the committed data file of one
    ncu capture of the pair kernel; it must parse to a per-launch byte count no
    smaller than the compulsory bytes of the workload (N x 40 B)."""
    t = bench.profile_traffic()
    assert t is not None and t >= bench.N_PARTICLES * 40
