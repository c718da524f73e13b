"""The multi-GPU form is replicas only: every rank steps its own case and the
ranks meet only in the timing reduction.  Two gloo ranks on CPU check that
reduction (units summed, time = the slowest rank's)."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units = 1000.0 * (rank + 1)          # uneven replicas
    seconds = 2.0 + rank                 # rank 1 is the slowest
    value, t = bench.replica_throughput(units, seconds, dist, "cpu")
    out[rank] = (value, t)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for r in range(2):
        value, t = out[r]
        assert t == 3.0
        assert value == pytest.approx(3000.0 / 3.0)


def test_replica_throughput_single_process():
    sys.path.insert(0, REPO)
    import bench
    assert bench.replica_throughput(500.0, 2.0) == (250.0, 2.0)
