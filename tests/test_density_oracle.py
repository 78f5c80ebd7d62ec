"""The oracle's density-matrix restatements on CPU: the reference's two-call gate
scheme and channel sum (cpu.py:400-517) against U rho U^dagger and Kraus sums built
from dense matrices, and the probability / collapse definitions against explicit
loops over the basis."""
import numpy as np
import pytest

from oracle import pyoracle as O
from qibojit_gb300.matrices import CustomMatrices
from tests.dense import apply_dense, random_unitary


def random_density_matrix(n, seed, dtype="complex128"):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((2**n, 2**n)) + 1j * rng.standard_normal((2**n, 2**n))
    rho = a @ a.conj().T
    return (rho / np.trace(rho)).astype(dtype)


def full_unitary(matrix, targets, controls, n):
    cols = [apply_dense(np.eye(2**n)[:, k], matrix, targets, controls, n) for k in range(2**n)]
    return np.stack(cols, axis=1)


CASES = [  # (n, targets, controls, kernel, matrix name)
    (3, [1], [], "apply_gate", "U"),
    (3, [0], [2], "apply_gate", "U"),
    (4, [2], [0, 3], "apply_x", "X"),
    (3, [2], [], "apply_y", "Y"),
    (3, [0], [1], "apply_y", "Y"),
    (3, [1], [], "apply_z", "Z"),
    (4, [3], [1], "apply_z_pow", "U1"),
    (4, [2, 0], [], "apply_two_qubit_gate", "U4"),
    (4, [1, 3], [0], "apply_two_qubit_gate", "U4"),
    (3, [0, 2], [], "apply_swap", "SWAP"),
    (4, [0, 2, 3], [], "multi", "U8"),
    (4, [3, 1, 2], [0], "multi", "U8"),
]


def _operands(name, seed):
    cm = CustomMatrices("complex128")
    if name == "U":
        m = random_unitary(2, seed)
        return m, m
    if name == "U4":
        m = random_unitary(4, seed)
        return m, m
    if name == "U8":
        m = random_unitary(8, seed)
        return m, m
    if name == "U1":
        theta = 0.3 + seed
        return cm.U1(theta), np.diag([1, np.exp(1j * theta)])
    if name == "SWAP":
        return None, np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=complex)
    dense = {"X": np.array([[0, 1], [1, 0]]), "Y": np.array([[0, -1j], [1j, 0]]), "Z": np.diag([1, -1])}[name]
    return getattr(cm, name), np.asarray(dense, dtype=complex)


@pytest.mark.parametrize("n,targets,controls,kernel,name", CASES)
def test_two_call_scheme_is_u_rho_udagger(n, targets, controls, kernel, name):
    operand, dense = _operands(name, 3)
    rho = random_density_matrix(n, 5)
    want = full_unitary(dense, targets, controls, n)
    want = want @ rho @ want.conj().T
    got = O.apply_gate_density_matrix(O.OracleBackend(), rho.copy(), n, targets, controls, kernel, operand)
    np.testing.assert_allclose(got, want, atol=1e-13)


def test_channel_is_the_kraus_sum():
    n = 3
    rho = random_density_matrix(n, 7)
    ob = O.OracleBackend()
    cm = CustomMatrices("complex128")
    u = random_unitary(4, 9)
    coeffs = [0.1, 0.2, 0.15]
    branches = [
        lambda r: O.apply_gate_density_matrix(ob, r, n, [1], [], "apply_x", cm.X),
        lambda r: O.apply_gate_density_matrix(ob, r, n, [2], [], "apply_y", cm.Y),
        lambda r: O.apply_gate_density_matrix(ob, r, n, [0, 2], [], "apply_two_qubit_gate", u),
    ]
    got = O.apply_channel_density_matrix(rho, coeffs, branches)
    x = full_unitary(np.array([[0, 1], [1, 0]]), [1], [], n)
    y = full_unitary(np.array([[0, -1j], [1j, 0]]), [2], [], n)
    w = full_unitary(u, [0, 2], [], n)
    want = (1 - sum(coeffs)) * rho + sum(c * k @ rho @ k.conj().T for c, k in zip(coeffs, (x, y, w)))
    np.testing.assert_allclose(got, want, atol=1e-14)
    assert abs(np.trace(got) - 1) < 1e-13


@pytest.mark.parametrize("qubits", [[0], [2], [1, 3], [3, 1], [0, 1, 2, 3], [2, 0, 3]])
def test_density_probabilities_definition(qubits):
    n = 4
    rho = random_density_matrix(n, 11)
    got = O.density_probabilities(rho, qubits, n)
    want = np.zeros(1 << len(qubits))
    for i in range(1 << n):
        o = 0
        for q in qubits:
            o = (o << 1) | ((i >> (n - 1 - q)) & 1)
        want[o] += rho[i, i].real
    np.testing.assert_allclose(got, want, atol=1e-15)


@pytest.mark.parametrize("qubits,shot", [([0], 1), ([2, 1], 2), ([3, 0, 2], 5)])
@pytest.mark.parametrize("normalize", [True, False])
def test_collapse_density_matrix_definition(qubits, shot, normalize):
    n = 4
    rho = random_density_matrix(n, 13)
    proj = np.zeros(1 << n)
    for i in range(1 << n):
        bits = [(i >> (n - 1 - q)) & 1 for q in qubits]
        proj[i] = float(bits == [(shot >> (len(qubits) - 1 - j)) & 1 for j in range(len(qubits))])
    p = np.diag(proj)
    want = p @ rho @ p
    if normalize:
        want = want / np.trace(want).real
    got = O.collapse_density_matrix(rho.copy(), qubits, shot, n, normalize)
    np.testing.assert_allclose(got, want, atol=1e-15)
