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


# --------------------------------------------------------------------- probabilities
@pytest.mark.parametrize("n,qubits", [(3, [0]), (3, [2, 0]), (4, [0, 1, 2, 3]), (4, [3, 1, 0, 2]), (6, [5]),
                                      (6, [4, 1, 2]), (11, [0]), (11, [10, 3]), (11, [1, 2, 3, 4, 5, 6, 7, 8])])
def test_density_probabilities_vs_oracle(backend, n, qubits, dtype):
    from oracle import pyoracle as O

    rho = random_density_matrix(n, 21 + n).astype(dtype)
    got = backend.to_numpy(backend.calculate_probabilities(backend.cast(rho, dtype=dtype, copy=True), qubits, n,
                                                           density_matrix=True))
    want = O.density_probabilities(rho, qubits, n)
    assert got.dtype == (np.float64 if dtype == "complex128" else np.float32)
    np.testing.assert_allclose(got, want, atol=1e-13 if dtype == "complex128" else 1e-6)


# -------------------------------------------------------------------------- collapse
@pytest.mark.parametrize("n,qubits,shot", [(3, [1], 0), (4, [0, 3], 2), (5, [4, 0, 2], 5), (9, [8, 1], 3)])
@pytest.mark.parametrize("normalize", [True, False])
def test_density_collapse_vs_oracle(backend, n, qubits, shot, normalize, dtype):
    from oracle import pyoracle as O

    rho = random_density_matrix(n, 31 + n).astype(dtype)
    got = backend.to_numpy(backend.collapse_state(backend.cast(rho, dtype=dtype, copy=True), qubits, shot, n,
                                                  normalize=normalize, density_matrix=True))
    want = O.collapse_density_matrix(rho.astype(np.complex128), qubits, shot, n, normalize)
    assert got.dtype == np.dtype(dtype)
    np.testing.assert_allclose(got, want, atol=1e-13 if dtype == "complex128" else 1e-6)
    if normalize:
        assert abs(np.trace(got) - 1) < (1e-12 if dtype == "complex128" else 1e-5)


def test_density_collapse_rejects_bad_shot(backend):
    rho = backend.zero_state(3, density_matrix=True)
    with pytest.raises(ValueError):
        backend.collapse_state(rho, [0, 1], 4, 3, density_matrix=True)


# -------------------------------------------------------------------------- channels
def _oracle_branch(ob, cm, n, gate):
    from oracle import pyoracle as O

    name = type(gate).__name__
    t, c = list(gate.target_qubits), list(gate.control_qubits)
    if name == "Y":
        return lambda r: O.apply_gate_density_matrix(ob, r, n, t, c, "apply_y", cm.Y)
    if name == "X":
        return lambda r: O.apply_gate_density_matrix(ob, r, n, t, c, "apply_x", cm.X)
    if name == "Z":
        return lambda r: O.apply_gate_density_matrix(ob, r, n, t, c, "apply_z", cm.Z)
    m = np.asarray(gate.parameters[0], dtype=np.complex128)
    if len(t) == 1:
        return lambda r: O.apply_gate_density_matrix(ob, r, n, t, c, "apply_gate", m)
    if len(t) == 2:
        return lambda r: O.apply_gate_density_matrix(ob, r, n, t, c, "apply_two_qubit_gate", m)
    return lambda r: O.apply_gate_density_matrix(ob, r, n, t, c, "multi", m)


def _channels(n):
    from qibojit_gb300 import gates

    return [gates.PauliNoiseChannel(1, px=0.1, py=0.05, pz=0.2),
            gates.PauliNoiseChannel(n - 1, py=0.3),
            gates.UnitaryChannel([0.25, 0.1], [((0, 2), random_unitary(4, 41)), ((1,), random_unitary(2, 42))]),
            gates.UnitaryChannel([0.4], [((2, 0, 1), random_unitary(8, 43))])]


@pytest.mark.parametrize("which", range(4))
def test_channel_density_matrix_vs_oracle(backend, which, dtype):
    from oracle import pyoracle as O
    from qibojit_gb300.matrices import CustomMatrices

    n = 4
    ch = _channels(n)[which]
    rho = random_density_matrix(n, 51 + which)
    ob, cm = O.OracleBackend(), CustomMatrices("complex128")
    want = O.apply_channel_density_matrix(rho, ch.coefficients, [_oracle_branch(ob, cm, n, g) for g in ch.gates])
    backend.set_dtype(dtype)
    state = backend.cast(rho.astype(dtype), copy=True)
    got = backend.to_numpy(backend.apply_channel(ch, state, n))
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])
    np.testing.assert_array_equal(backend.to_numpy(state), rho.astype(dtype))  # input kept
    backend.set_dtype("complex128")


def test_channel_on_state_vector_draws_one_branch(backend):
    from qibojit_gb300 import gates

    n = 3
    psi = np.zeros(8, dtype=np.complex128)
    psi[0] = 1
    got = backend.to_numpy(backend.apply_channel(gates.PauliNoiseChannel(0, px=1.0), backend.cast(psi, copy=True), n))
    np.testing.assert_allclose(got, np.eye(8)[4], atol=0)
    ch = gates.PauliNoiseChannel(2, px=0.3, pz=0.3)
    for seed in range(6):
        np.random.seed(seed)
        index = np.random.choice(3, p=[0.3, 0.3, 0.4])
        np.random.seed(seed)
        out = backend.to_numpy(backend.apply_channel(ch, backend.cast(psi + 0, copy=True), n))
        want = np.eye(8)[1] if index == 0 else np.eye(8)[0]
        np.testing.assert_allclose(out, want, atol=0)


# ------------------------------------------------------------------ fused circuits
@pytest.mark.parametrize("n,ngates,seed", [(4, 40, 1), (5, 80, 2), (7, 120, 3)])
def test_fused_density_circuit_matches_gate_by_gate(backend, n, ngates, seed, dtype):
    from tests.circuits_random import random_circuit

    backend.set_dtype(dtype)
    circ = random_circuit(n, ngates, seed)
    rho = random_density_matrix(n, 61 + seed).astype(dtype)
    want = backend.to_numpy(backend.execute_circuit(circ, rho.copy(), fuse=False))
    for _ in range(4):  # the cached program specialises its passes after two runs
        got = backend.to_numpy(backend.execute_circuit(circ, rho.copy()))
        np.testing.assert_allclose(got, want, atol=10 * ATOL[dtype])
    prog = next(iter(backend._programs.values()))
    # complex128 programs stay interpreted in double-word arithmetic (faster than compiled)
    assert prog.nqubits == 2 * n and prog.specialized == (dtype == "complex64")
    backend.set_dtype("complex128")


def test_density_circuit_with_channels_vs_oracle(backend):
    from oracle import pyoracle as O
    from qibojit_gb300 import gates
    from qibojit_gb300.matrices import CustomMatrices

    n = 4
    circ = gates.Circuit(n)
    u = random_unitary(4, 71)
    chans = _channels(n)
    circ.add([gates.H(0), gates.CNOT(0, 1), chans[0], gates.Unitary(u, 2, 3), chans[2], gates.RY(3, 0.4), chans[1]])
    rho = random_density_matrix(n, 72)
    got = backend.to_numpy(backend.execute_circuit(circ, rho.copy()))
    ob, cm = O.OracleBackend(), CustomMatrices("complex128")
    ref = rho.copy()
    for g in circ.queue:
        if hasattr(g, "coefficients"):
            ref = O.apply_channel_density_matrix(ref, g.coefficients, [_oracle_branch(ob, cm, n, x) for x in g.gates])
            continue
        name = type(g).__name__
        t, c = list(g.target_qubits), list(g.control_qubits)
        if name == "H":
            O.apply_gate_density_matrix(ob, ref, n, t, c, "apply_gate", cm.H)
        elif name == "CNOT":
            O.apply_gate_density_matrix(ob, ref, n, t, c, "apply_x", cm.CNOT)
        elif name == "RY":
            O.apply_gate_density_matrix(ob, ref, n, t, c, "apply_gate", cm.RY(*g.parameters))
        else:
            O.apply_gate_density_matrix(ob, ref, n, t, c, "apply_two_qubit_gate", u)
    np.testing.assert_allclose(got, ref, atol=1e-12)
    assert abs(np.trace(got) - 1) < 1e-12


# ------------------------------------------------------------------- inverse gates
@pytest.mark.parametrize("gatename,qubits,params", [("CNOT", (0, 2), {}), ("CU3", (3, 1), {"theta": 0.3, "phi": 1.1,
                                                                                          "lam": -0.4}),
                                                    ("TOFFOLI", (0, 3, 1), {}), ("fSim", (2, 0), {"theta": 0.7,
                                                                                                "phi": 0.2}),
                                                    ("CRY", (1, 2), {"theta": 2.1}), ("CU1", (3, 0), {"theta": 0.9})])
def test_inverse_gate_restores_density_matrix(backend, gatename, qubits, params, dtype):
    """apply_gate then apply_gate(..., inverse=True) on a density matrix gives rho
    back: controls kept, the target block inverted, and for complex64 the complex128
    inverse operand cast down (U^-1 rho U after U rho U^dagger)."""
    from qibojit_gb300 import gates

    from tests.conftest import PARITY_ATOL

    n = 4
    rho = random_density_matrix(n, 41).astype(dtype)
    backend.set_dtype(dtype)
    gate = getattr(gates, gatename)(*qubits, **params)
    state = backend.cast(rho, copy=True)
    state = backend.apply_gate(gate, state, n)
    moved = backend.to_numpy(state).copy()
    state = backend.apply_gate(gate, state, n, inverse=True)
    got = backend.to_numpy(state)
    assert np.abs(moved - rho).max() > 1e-3  # the gate did act
    tol = 10 * PARITY_ATOL[dtype]
    np.testing.assert_allclose(got, rho, rtol=0, atol=tol)
