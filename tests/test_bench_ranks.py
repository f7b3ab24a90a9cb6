"""bench.py's multi-process path on CPU: two gloo ranks agree on the slowest rank's time
(the replicas' job time), as the N-GPU launch under torchrun does over NCCL."""

import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(10.0 + 5.0 * rank, torch.device("cpu"), world)
    finally:
        torch.distributed.destroy_process_group()


def test_slowest_rank_time_over_gloo():
    world = 2
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    assert dict(out) == {0: 15.0, 1: 15.0}


def test_single_rank_is_its_own_time():
    import bench
    assert bench.max_over_ranks(3.5, torch.device("cpu"), 1) == 3.5
