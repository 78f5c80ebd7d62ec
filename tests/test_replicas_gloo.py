"""The multi-GPU bench path is replicas only: each rank runs its own circuit and the
job throughput is all ranks' work over the slowest rank's time.  Checked here with two
gloo ranks on CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    dist.init_process_group("gloo", rank=rank, world_size=2)
    import bench

    elapsed = [100.0, 250.0][rank]
    ms, value = bench.replicas_throughput(elapsed, 890 * 5, "cpu")
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_throughput_two_ranks():
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(port, out), nprocs=2, join=True)
    for rank in (0, 1):
        ms, value = out[rank]
        assert ms == 250.0
        assert value == pytest.approx(2 * 890 * 5 / 0.25)


def test_single_process_is_identity():
    import bench

    ms, value = bench.replicas_throughput(200.0, 1000, "cpu")
    assert ms == 200.0 and value == pytest.approx(5000.0)
