"""The multi-rank (replica) bookkeeping of the benchmark on two gloo ranks on the CPU: the
slowest rank's time defines the whole-job throughput on every rank, and a single process
works without a process group."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from opencl_fdtd_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    replicas.barrier()
    elapsed = [120.0, 150.0][rank]
    out[rank] = replicas.job_throughput(1_000_000, 100, elapsed, world)
    out[2 + rank] = replicas.max_over_ranks(float(rank + 1))
    replicas.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_slowest_rank():
    port = _free_port()
    out = mp.get_context("spawn").Manager().list([0.0] * 4)
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    want = 2 * 1_000_000 * 100 / 0.150 / 1e6
    assert out[0] == pytest.approx(want) and out[1] == pytest.approx(want)
    assert out[2] == 2.0 and out[3] == 2.0


def test_single_process_without_group():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.job_throughput(10, 2, 1000.0, 1) == pytest.approx(2e-5)
