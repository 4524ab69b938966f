"""The timing steps of bench.py's multi-rank path on CPU ranks (gloo, world size 2, 127.0.0.1): the barrier around the
timed region and the maximum of the ranks' times; the reference arm runs on rank 0 alone. (The partitioned data path
itself, trace exchange included, is covered by tests/test_partition.py on gloo ranks and tests/test_gpu_partition.py
on the GPU.)"""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        bench.ranks_barrier(torch, world)
        out[rank] = bench.ranks_max(torch, world, 1.5 + rank, "cpu")
        bench.ranks_barrier(torch, world)
    finally:
        dist.destroy_process_group()


def test_two_replicas_agree_on_the_slowest_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
        assert dict(out) == {0: 2.5, 1: 2.5}


def test_single_rank_needs_no_process_group():
    import torch
    sys.path.insert(0, REPO)
    import bench
    bench.ranks_barrier(torch, 1)
    assert bench.ranks_max(torch, 1, 3.25, "cpu") == 3.25


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, REPO)
    import argparse
    import bench
    args = argparse.Namespace(workload="hex3d", steps=1, warmup=0)
    assert bench.run_reference(args, rank=1, world=2) is None
