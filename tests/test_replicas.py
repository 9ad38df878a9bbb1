"""The multi-GPU form of bench.py is N independent replicas (the step does
not decompose across GPUs): each rank times its own replica, the job's time
is the slowest rank's, and the rate counts every rank's cells.  These run
the same reduction over two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, ws, port, secs, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        dist.barrier()
        slowest = bench.reduce_max(secs[rank], torch)
        out[rank] = (slowest, bench.job_rate(ws, 1000, slowest))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    ws, port = 2, free_port()
    secs = [0.25, 0.5]
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(worker, args=(ws, port, secs, out), nprocs=ws, join=True)
        res = dict(out)
    assert res[0] == res[1] == (0.5, 2 * 1000 / 0.5)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert not dist.is_initialized()
    assert bench.reduce_max(0.125, torch) == 0.125
    assert bench.job_rate(1, 8, 0.5) == 16.0
