"""The multi-GPU path is replicas only: each rank solves its own system and the
job throughput is the atoms summed over ranks over the slowest rank's time.
This runs the aggregation of bench.py on two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    atoms = 1000 * (rank + 1)        # 1000 and 2000 atoms
    ms = 10.0 * (rank + 1)           # the second rank is slower: 20 ms for the whole run
    v, mx = bench.replica_throughput(atoms, 5, ms, dist, torch.device("cpu"))
    out[rank] = (v, mx)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    for r in (0, 1):
        v, mx = out[r]
        assert mx == 20.0
        assert abs(v - 3000 * 5 / 0.020) < 1e-6


def test_replica_throughput_single_process():
    import bench
    v, mx = bench.replica_throughput(1000, 4, 8.0)
    assert mx == 8.0 and abs(v - 1000 * 4 / 0.008) < 1e-9
