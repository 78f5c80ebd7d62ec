"""Global-qubit sharding with the engine's kernels as each rank's local executor: two
processes share this GPU, each owning one half of an n-qubit state in device memory,
and trade half-pieces through host memory over gloo (host-level exchanges between
kernel launches; no kernel waits on another process).  Compared with the whole state
run on the GPU in one process."""
import os
import socket

import numpy as np
import pytest

from tests.circuits_random import random_circuit

pytestmark = pytest.mark.gpu

FAMILIES = ["one", "one_p", "two_c", "two_p", "swap", "fsim", "toffoli", "u2q", "u3q", "cu1q", "zc", "fanout"]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, port, n, seed, dtype, out):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        from qibojit_gb300 import MetaBackend
        from qibojit_gb300.sharded import ShardedState, gb300_local_executor

        backend = MetaBackend.load("gb300")
        backend.set_dtype(dtype)
        st = ShardedState.zero_state(n, gb300_local_executor(backend), dtype=dtype, device="cuda")
        st.run(random_circuit(n, 60, seed, families=FAMILIES))
        torch.cuda.synchronize()
        out[rank] = (st.gather().numpy(), st.swaps)
    finally:
        dist.destroy_process_group()


def test_two_ranks_on_one_gpu_match_the_whole_state(dtype):
    import torch.multiprocessing as mp

    from qibojit_gb300 import MetaBackend

    n, seed = 12, 21
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(port, n, seed, dtype, out), nprocs=2, join=True)
    backend = MetaBackend.load("gb300")
    backend.set_dtype(dtype)
    want = backend.to_numpy(backend.execute_circuit(random_circuit(n, 60, seed, families=FAMILIES), fuse=False))
    tol = 1e-12 if dtype == "complex128" else 1e-5
    for rank in (0, 1):
        full, swaps = out[rank]
        assert swaps > 0
        np.testing.assert_allclose(full, want, rtol=0, atol=tol)
