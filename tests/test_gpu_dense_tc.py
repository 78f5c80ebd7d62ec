"""Dense k-target gates (k = 4..6) on the tensor cores (complex64, tcgen05 with TF32
operands split in two and FP32 accumulation) against the oracle, the CUDA-core
kernel and unitarity, over the placements the reference's tests use for its
multi-qubit kernels (targets low, high, interleaved and unsorted, with and without
controls) and partial tiles."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.dense import random_state, random_unitary

pytestmark = pytest.mark.gpu

# complex64 parity bar of the engine, relative to the rounding scale of a gate row
TOL = 1e-5


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    b = MetaBackend.load("gb300")
    yield b
    b.ctx.set_dense_mode("auto")


def _apply(backend, mode, state, n, targets, controls, gate):
    backend.ctx.set_dense_mode(mode)
    q = O.OracleBackend.qubits_tensor(n, targets, controls)
    s = backend.cast(state, dtype="complex64", copy=True)
    out = backend.to_numpy(backend._multi_qubit_base(s, n, list(targets), gate.astype(np.complex64), q))
    backend.synchronize()
    return out


CASES = [
    (10, [0, 1, 2, 3], []), (12, [8, 9, 10, 11], []), (12, [11, 3, 7, 0], []), (14, [2, 9, 5, 13, 0], []),
    (14, [13, 12, 11, 10, 9], []), (16, [0, 4, 8, 12, 15, 1], []), (16, [10, 11, 12, 13, 14, 15], []),
    (15, [3, 1, 4, 0, 5, 2], []), (13, [6, 2, 9, 11], [0, 12]), (16, [1, 3, 5, 7, 9], [15]),
    (17, [16, 8, 4, 2, 1, 0], [10, 12]), (11, [5, 4, 3, 2, 1, 0], []), (9, [8, 7, 6, 5], [0]),
    (20, [19, 0, 10, 5, 15, 7], []), (18, [2, 3, 4, 5], [0, 1, 17]),
    # 16 groups: half of the first warp holds groups, the other half none
    (9, [0, 1, 2, 3], [4]), (10, [0, 1, 2, 3, 4], [6]),
]


@pytest.mark.parametrize("n,targets,controls", CASES)
def test_tensor_core_gate_vs_oracle(backend, n, targets, controls):
    k = len(targets)
    gate = random_unitary(2**k, 100 + n + k)
    state = random_state(n, 200 + n, "complex64")
    got = _apply(backend, "tensor", state, n, targets, controls, gate)
    want = O.OracleBackend()._multi_qubit_base(state.astype(np.complex128), n, list(targets), gate,
                                                O.OracleBackend.qubits_tensor(n, targets, controls))
    np.testing.assert_allclose(got, want, rtol=0, atol=TOL)
    simt = _apply(backend, "simt", state, n, targets, controls, gate)
    np.testing.assert_allclose(got, simt, rtol=0, atol=TOL)


@pytest.mark.parametrize("k", [4, 5, 6])
def test_tensor_core_gate_unnormalised_operand(backend, k):
    """A non-unitary operand with entries of both signs (every product of the split
    contributes), against the oracle relative to the row scale sum_j |g_ij| |x_j|."""
    n = 14
    rng = np.random.default_rng(k)
    gate = (rng.standard_normal((2**k, 2**k)) + 1j * rng.standard_normal((2**k, 2**k))) * 0.3
    targets = [int(t) for t in rng.permutation(n)[:k]]
    state = random_state(n, 300 + k, "complex64")
    got = _apply(backend, "tensor", state, n, targets, [], gate)
    ob = O.OracleBackend()
    q = O.OracleBackend.qubits_tensor(n, targets)
    want = ob._multi_qubit_base(state.astype(np.complex128), n, targets, gate, q)
    scale = ob._multi_qubit_base(np.abs(state).astype(np.complex128), n, targets, np.abs(gate).astype(np.complex128),
                                 q)
    assert np.all(np.abs(got - want) <= TOL * np.maximum(1.0, np.abs(scale)))


@pytest.mark.parametrize("k", [4, 5, 6])
def test_tensor_core_gate_inverse_restores_state(backend, k):
    n = 22
    rng = np.random.default_rng(40 + k)
    targets = [int(t) for t in rng.permutation(n)[:k]]
    gate = random_unitary(2**k, 50 + k)
    state = random_state(n, 60 + k, "complex64")
    backend.ctx.set_dense_mode("tensor")
    s = backend.cast(state, dtype="complex64", copy=True)
    q = O.OracleBackend.qubits_tensor(n, targets)
    s = backend._multi_qubit_base(s, n, targets, gate.astype(np.complex64), q)
    s = backend._multi_qubit_base(s, n, targets, gate.conj().T.astype(np.complex64), q)
    got = backend.to_numpy(s)
    backend.synchronize()
    np.testing.assert_allclose(got, state, rtol=0, atol=TOL)
    assert abs(backend.norm2(s, n) - 1) < 1e-5


def test_auto_mode_uses_tensor_cores_and_rejects_what_it_cannot_take(backend):
    n = 16
    gate = random_unitary(8, 3)
    backend.ctx.set_dense_mode("tensor")
    s = backend.cast(random_state(n, 1, "complex64"), dtype="complex64", copy=True)
    with pytest.raises(NotImplementedError):  # 3 targets: CUDA-core kernel only
        backend._multi_qubit_base(s, n, [0, 1, 2], gate.astype(np.complex64), None)
    s128 = backend.cast(random_state(n, 1), dtype="complex128", copy=True)
    with pytest.raises(NotImplementedError):
        backend._multi_qubit_base(s128, n, [0, 1, 2, 3], random_unitary(16, 4), None)
    backend.ctx.set_dense_mode("auto")


def test_repeated_calls_and_sync_status(backend):
    """Many back-to-back launches on one stream (operand buffer reused between them),
    then sv_sync reports no time-out."""
    n, k = 20, 6
    targets = [19, 3, 11, 0, 7, 15]
    state = random_state(n, 5, "complex64")
    gates = [random_unitary(2**k, 70 + j) for j in range(6)]
    backend.ctx.set_dense_mode("tensor")
    s = backend.cast(state, dtype="complex64", copy=True)
    q = O.OracleBackend.qubits_tensor(n, targets)
    for g in gates:
        s = backend._multi_qubit_base(s, n, targets, g.astype(np.complex64), q)
    backend.ctx.sync()
    got = backend.to_numpy(s)
    want = state.astype(np.complex128)
    ob = O.OracleBackend()
    for g in gates:
        want = ob._multi_qubit_base(want, n, targets, g, q)
    np.testing.assert_allclose(got, want, rtol=0, atol=3 * TOL)


@pytest.mark.parametrize("targets", [[11, 10, 9, 8, 7], [3, 7, 1, 9, 0, 11]])
def test_tensor_core_gate_on_an_8_byte_aligned_state(backend, targets):
    """A state that starts 8 bytes past a 16-byte boundary (a view into a larger
    buffer) takes the scalar loads and stores."""
    import torch

    n, k = 12, len(targets)
    gate = random_unitary(2**k, 9 + k)
    state = random_state(n, 31, "complex64")
    buf = torch.zeros(2**n + 1, dtype=torch.complex64, device="cuda")
    buf[1:] = torch.from_numpy(state).to("cuda")
    view = buf[1:]
    assert view.data_ptr() % 16 == 8
    backend.ctx.set_dense_mode("tensor")
    q = O.OracleBackend.qubits_tensor(n, targets)
    backend._multi_qubit_base(view, n, targets, gate.astype(np.complex64), q)
    got = backend.to_numpy(view)
    backend.synchronize()
    want = O.OracleBackend()._multi_qubit_base(state.astype(np.complex128), n, targets, gate, q)
    np.testing.assert_allclose(got, want, rtol=0, atol=TOL)
    assert backend.to_numpy(buf[:1])[0] == 0
