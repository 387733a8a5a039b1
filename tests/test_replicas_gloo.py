"""The multi-process path of bench.py on the CPU (gloo, two ranks): every rank
runs a replica of the workload, and the whole-job throughput is the units of
all ranks over the slowest rank's time (max over ranks)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    t_local = 0.010 * (rank + 1)  # rank 1 is the slow one
    rate, t = bench.replicas_throughput(t_local, 1000, world, device="cpu")
    out[rank] = (rate, t)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    for r in range(world):
        rate, t = res[r]
        assert t == pytest.approx(0.020)
        assert rate == pytest.approx(world * 1000 / 0.020)
