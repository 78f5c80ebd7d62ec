"""Pipelined host-to-host execution (``execute_circuit_stream``): each host state comes
back equal to ``execute_circuit`` of the same state, whatever the overlap of uploads,
passes and read-backs on the three streams."""
import numpy as np
import pytest
import torch

from qibojit_gb300 import MetaBackend, circuits
from tests.circuits_random import random_circuit

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    return MetaBackend.load("gb300")


def _random_states(n, k, dtype, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(k):
        v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        v /= np.linalg.norm(v)
        out.append(torch.from_numpy(v.astype(dtype)).pin_memory())
    return out


@pytest.mark.parametrize("dt", ["complex64", "complex128"])
@pytest.mark.parametrize("n,k", [(10, 1), (12, 2), (14, 5)])
def test_stream_matches_execute_circuit(backend, n, k, dt):
    circ = random_circuit(n, 150, 40 + n)
    ins = _random_states(n, k, dt, n * 7 + k)
    outs = [torch.empty_like(x).pin_memory() for x in ins]
    backend.execute_circuit_stream(circ, ins, outs)
    tol = 1e-5 if dt == "complex64" else 1e-12
    for x, y in zip(ins, outs):
        ref = backend.execute_circuit(circ, x.clone()).cpu().numpy()
        np.testing.assert_allclose(y.numpy(), ref, atol=tol)


def test_stream_specialises_over_the_batch(backend):
    circ = circuits.brickwork(13, 4, 5)
    ins = _random_states(13, 4, "complex64", 3)
    outs = [torch.empty_like(x).pin_memory() for x in ins]
    backend.execute_circuit_stream(circ, ins, outs)
    progs = list(backend._programs.values())
    assert len(progs) == 1 and progs[0].specialized and progs[0].runs == 4
    for x, y in zip(ins, outs):
        ref = backend.execute_circuit(circ, x.clone()).cpu().numpy()
        np.testing.assert_allclose(y.numpy(), ref, atol=1e-5)


def test_stream_repeated_buffers(backend):
    """The same input and output tensor for every step, as a benchmark loop uses them."""
    n = 16
    circ = circuits.brickwork(n, 6, 9)
    host_in = backend.host_buffer(n, "complex64")
    host_in.zero_()
    host_in[0] = 1
    host_out = backend.host_buffer(n, "complex64")
    backend.execute_circuit_stream(circ, [host_in] * 6, [host_out] * 6)
    ref = backend.execute_circuit(circ, host_in.clone()).cpu().numpy()
    np.testing.assert_allclose(host_out.numpy(), ref, atol=1e-5)
    assert host_in[0].item() == 1 and abs(host_in[1:]).sum().item() == 0


def test_stream_small_and_empty(backend):
    circ = random_circuit(5, 30, 2)
    ins = _random_states(5, 3, "complex128", 11)
    outs = [torch.empty_like(x) for x in ins]
    backend.execute_circuit_stream(circ, ins, outs)
    for x, y in zip(ins, outs):
        ref = backend.execute_circuit(circ, x.clone()).cpu().numpy()
        np.testing.assert_allclose(y.numpy(), ref, atol=1e-12)
    assert backend.execute_circuit_stream(circ, [], []) == []


def test_stream_rejects_bad_buffers(backend):
    circ = random_circuit(10, 20, 3)
    good = _random_states(10, 1, "complex64", 1)
    with pytest.raises(ValueError):
        backend.execute_circuit_stream(circ, good, [])
    with pytest.raises(ValueError):
        backend.execute_circuit_stream(circ, good, [torch.empty(1 << 9, dtype=torch.complex64)])
    with pytest.raises(ValueError):
        backend.execute_circuit_stream(circ, good, [torch.empty(1 << 10, dtype=torch.complex128)])
    with pytest.raises(ValueError):
        backend.execute_circuit_stream(circ, good, [torch.empty(1 << 10, dtype=torch.complex64, device="cuda")])
