"""Multi-GPU runs are independent replicas (one scene per rank, no data-path collective); the only
cross-rank step is the bench's aggregation: all ranks' pixels over the slowest rank's time.  Checked with
two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    rate, ms = bench.replica_throughput(pixels=(rank + 1) * 1_000_000, ms=10.0 * (rank + 1))
    out[rank] = (rate, ms)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    import torch.multiprocessing as mp
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for rank in range(2):
        rate, ms = out[rank]
        assert ms == pytest.approx(20.0)
        assert rate == pytest.approx(3_000_000 / 0.020 / 1e6)


def test_replica_throughput_single_process():
    import bench
    rate, ms = bench.replica_throughput(pixels=2_000_000, ms=4.0)
    assert ms == 4.0 and rate == pytest.approx(500.0)
