"""Global-qubit sharding of one state over 2 and 4 ranks (gloo, CPU): the exchange
logic of ``qibojit_gb300.sharded`` with the oracle as every rank's local executor,
against the oracle run on the whole state in one process.  On GPUs the same code runs
the engine's kernels on each rank's piece and exchanges half-pieces over NCCL."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from tests.circuits_random import random_circuit

FAMILIES = ["one", "one_p", "two_c", "two_p", "swap", "fsim", "toffoli", "ccz", "u2q", "u3q", "cu1q", "cu2q",
            "zc", "fanout", "deutsch", "gfsim"]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _oracle_apply(state, n, gate):
    """One gate on the C oracle: its target matrix with its controls through the
    oracle's multi-target kernel."""
    from oracle import pyoracle as O
    from qibojit_gb300.fusion import _target_matrix

    ob = O.OracleBackend(nthreads=1)
    t, c = list(gate.target_qubits), list(gate.control_qubits)
    return ob._multi_qubit_base(state, n, t, _target_matrix(gate), ob.qubits_tensor(n, t, c))


def _oracle_full(circ, state):
    from qibojit_gb300.fusion import _expand

    s = state.copy()
    for g in _expand(circ.queue):
        s = _oracle_apply(s, circ.nqubits, g)
    return s


def _local_executor(piece, nlocal, gate):
    arr = piece.numpy()
    out = _oracle_apply(arr, nlocal, gate)
    if out is not arr:
        arr[...] = out
    return piece


def _worker(rank, world, port, n, seed, init, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from qibojit_gb300.sharded import ShardedState

        circ = random_circuit(n, 70, seed, families=FAMILIES)
        if init == "zero":
            st = ShardedState.zero_state(n, _local_executor)
        else:
            rng = np.random.default_rng(seed + 1)
            x = rng.standard_normal(2**n) + 1j * rng.standard_normal(2**n)
            st = ShardedState.from_full(torch.from_numpy(x / np.linalg.norm(x)), _local_executor)
        st.run(circ)
        full = st.gather().numpy()
        out[rank] = (full, st.swaps, list(st.phys))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,n,seed,init", [(2, 8, 1, "zero"), (2, 9, 2, "random"), (4, 8, 3, "random"),
                                               (4, 10, 4, "zero")])
def test_sharded_circuit_matches_single_state(world, n, seed, init):
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(world, port, n, seed, init, out), nprocs=world, join=True)
    circ = random_circuit(n, 70, seed, families=FAMILIES)
    if init == "zero":
        x = np.zeros(2**n, dtype=np.complex128)
        x[0] = 1
    else:
        rng = np.random.default_rng(seed + 1)
        x = rng.standard_normal(2**n) + 1j * rng.standard_normal(2**n)
        x /= np.linalg.norm(x)
    want = _oracle_full(circ, x)
    for rank in range(world):
        full, swaps, phys = out[rank]
        np.testing.assert_allclose(full, want, rtol=0, atol=1e-12)
        assert swaps > 0  # the circuit touched global qubits
        assert sorted(phys) == list(range(n))


def _worker_errors(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from qibojit_gb300.sharded import ShardedState

        errs = []
        for n in (2, 3):  # 4 ranks hold 2 global qubits: n = 2 and 3 leave fewer than 2 local ones
            try:
                ShardedState.zero_state(n, _local_executor)
            except ValueError as e:
                errs.append(str(e))
        out[rank] = errs
    finally:
        dist.destroy_process_group()


def test_sharded_state_rejects_bad_layouts():
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_worker_errors, args=(4, port, out), nprocs=4, join=True)
    assert all(len(out[r]) == 2 for r in range(4))
