"""Density matrices: rho -> U rho U^dagger through the same kernels on the 2n-qubit
vector (the reference's two-call scheme, cpu.py:452-517), checked against dense numpy
with the placement tables of tests/test_gates.py (density_matrix=True cases)."""
import numpy as np
import pytest

from tests.conftest import ATOL
from tests.dense import apply_dense, random_complex, random_unitary

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    return MetaBackend.load("gb300")


def random_density_matrix(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((2**n, 2**n)) + 1j * rng.standard_normal((2**n, 2**n))
    rho = a @ a.conj().T
    return rho / np.trace(rho)


def full_unitary(matrix, targets, controls, n):
    cols = [apply_dense(np.eye(2**n)[:, k], matrix, targets, controls, n) for k in range(2**n)]
    return np.stack(cols, axis=1)


def _check(backend, gate, matrix, targets, controls, n, dtype):
    rho = random_density_matrix(n, 3).astype(dtype)
    backend.set_dtype(dtype)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(rho, copy=True), n))
    u = full_unitary(matrix, targets, controls, n)
    np.testing.assert_allclose(got, u @ rho @ u.conj().T, atol=ATOL[dtype])


@pytest.mark.parametrize(("nqubits", "targets", "controls"),
                         [(5, [3, 4], []), (4, [2, 0], []), (2, [0, 1], []), (3, [0, 1], [2]), (4, [1, 3], [0]),
                          (5, [3, 1], [0, 2])])
def test_apply_two_qubit_gate_density_matrix(backend, nqubits, targets, controls, dtype):
    from qibojit_gb300 import gates

    matrix = random_unitary(4, 6).astype(dtype)
    gate = gates.Unitary(matrix, *targets).controlled_by(*controls)
    _check(backend, gate, matrix, targets, controls, nqubits, dtype)


@pytest.mark.parametrize(("nqubits", "targets", "controls"),
                         [(3, [0, 1, 2], []), (4, [2, 1, 3], []), (4, [2, 1, 3], [0]), (5, [0, 2, 3], [1])])
def test_apply_multiqubit_gate_density_matrix(backend, nqubits, targets, controls, dtype):
    from qibojit_gb300 import gates

    matrix = random_complex((8, 8), 7, dtype)
    gate = gates.Unitary(matrix, *targets).controlled_by(*controls)
    _check(backend, gate, matrix, targets, controls, nqubits, dtype)


@pytest.mark.parametrize("gatename", ["H", "X", "Y", "Z", "S", "T"])
def test_gates_on_circuit_density_matrix(backend, gatename):
    from qibojit_gb300 import gates

    backend.set_dtype("complex128")
    rho = random_density_matrix(1, 4)
    c = gates.Circuit(1)
    c.add(getattr(gates, gatename)(0))
    got = backend.to_numpy(backend.execute_circuit(c, rho))
    u = c.queue[0].base_matrix()
    np.testing.assert_allclose(got, u @ rho @ u.conj().T, atol=1e-12)


@pytest.mark.parametrize("gatename,params", [("CRX", {"theta": 0.1}), ("CU1", {"theta": 0.1}),
                                             ("CU3", {"theta": 0.1, "phi": 0.2, "lam": 0.3}),
                                             ("fSim", {"theta": 0.1, "phi": 0.2}), ("CY", {}), ("CZ", {})])
def test_parametrized_gates_on_circuit_density_matrix(backend, gatename, params):
    from qibojit_gb300 import gates

    backend.set_dtype("complex128")
    rho = random_density_matrix(2, 5)
    c = gates.Circuit(2)
    c.add(getattr(gates, gatename)(0, 1, **params))
    got = backend.to_numpy(backend.execute_circuit(c, rho))
    u = c.queue[0].matrix()
    np.testing.assert_allclose(got, u @ rho @ u.conj().T, atol=1e-12)


def test_zero_state_density_matrix(backend, dtype):
    s = backend.to_numpy(backend.zero_state(4, density_matrix=True, dtype=dtype))
    want = np.zeros((16, 16), dtype=dtype)
    want[0, 0] = 1
    np.testing.assert_array_equal(s, want)
