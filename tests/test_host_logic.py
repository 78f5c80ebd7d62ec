"""Host-side logic that needs no GPU: gate matrices, fused-gate matrices, circuit
builders and the reference energy formula."""
import numpy as np
import pytest

from qibojit_gb300 import circuits
from qibojit_gb300 import gates as G
from qibojit_gb300.batch import hea_batch, hea_circuit, tfim_energy_dense
from qibojit_gb300.fusion import SV_OP_DENSE, SV_OP_DIAG, lower, matrix_fused
from qibojit_gb300.matrices import CustomMatrices, Matrices
from tests.dense import apply_dense, random_state


def test_matrices_are_unitary():
    m = Matrices()
    rng = np.random.default_rng(0)
    for name in ["H", "X", "Y", "Z", "S", "SDG", "T", "TDG", "SX", "SXDG", "CNOT", "CZ", "SWAP", "TOFFOLI", "CCZ"]:
        u = getattr(m, name)
        np.testing.assert_allclose(u @ u.conj().T, np.eye(u.shape[0]), atol=1e-14)
    for name, k in [("RX", 1), ("RY", 1), ("RZ", 1), ("U1", 1), ("U2", 2), ("U3", 3), ("fSim", 2), ("CU3", 3)]:
        u = getattr(m, name)(*rng.uniform(0, 2 * np.pi, k))
        np.testing.assert_allclose(u @ u.conj().T, np.eye(u.shape[0]), atol=1e-14)


def test_u3_conventions():
    m = Matrices()
    # U3(t, -pi/2, pi/2) = RX(t); U3(t, 0, 0) = RY(t); U3(0, 0, l) = RZ(l) up to phase conventions
    t = 0.7
    np.testing.assert_allclose(m.U3(t, -np.pi / 2, np.pi / 2), m.RX(t), atol=1e-15)
    np.testing.assert_allclose(m.U3(t, 0, 0), m.RY(t), atol=1e-15)
    np.testing.assert_allclose(m.U3(0, 0, 0.3), m.RZ(0.3), atol=1e-15)


def test_custom_operands():
    cm = CustomMatrices()
    assert cm.U1(0.4).shape == ()
    assert np.isclose(cm.U1(0.4), np.exp(0.4j))
    f = cm.fSim(0.3, 0.2)
    assert f.shape == (5,) and np.isclose(f[4], np.exp(-0.2j))
    np.testing.assert_allclose(cm.CNOT, Matrices().X)


def test_lower_classifies_diagonals():
    c = G.Circuit(3)
    c.add([G.RZ(0, theta=0.1), G.CZ(0, 1), G.RY(1, theta=0.2), G.CNOT(1, 2), G.U1(2, theta=0.3)])
    kinds = [k for k, *_ in lower(c.queue)]
    assert kinds == [SV_OP_DIAG, SV_OP_DIAG, SV_OP_DENSE, SV_OP_DENSE, SV_OP_DIAG]


def test_matrix_fused_matches_sequential_application():
    rng = np.random.default_rng(1)
    n = 4
    fg = G.FusedGate(0, 1, 3)
    for g in [G.U3(0, *rng.uniform(0, 6, 3)), G.CNOT(3, 1), G.RY(1, theta=0.4), G.CZ(0, 3), G.SWAP(0, 3)]:
        fg.append(g)
    x = random_state(n, 2)
    want = x.copy()
    for g in fg.gates:
        want = apply_dense(want, g.base_matrix(), list(g.target_qubits), list(g.control_qubits), n)
    got = apply_dense(x, matrix_fused(fg), [0, 1, 3], [], n)
    np.testing.assert_allclose(got, want, atol=1e-14)


def test_brickwork_and_qft_shapes():
    c = circuits.brickwork(30, 20, 1234)
    assert len(c.queue) == 890
    assert sum(type(g).__name__ == "U3" for g in c.queue) == 600
    q = circuits.qft(20)
    assert len(q.queue) == 20 + 190 + 10


def test_hea_batch_distribution():
    specs = hea_batch(4096, seed=1234)
    ns = np.array([s[0] for s in specs])
    ls = np.array([s[1] for s in specs])
    assert ns.min() == 10 and ns.max() == 22 and ls.min() == 4 and ls.max() == 12
    n, L, p = specs[0]
    assert len(hea_circuit(n, L, p).queue) == L * (3 * n - 1)


@pytest.mark.parametrize("n", [2, 3, 5])
def test_tfim_energy_dense_matches_hamiltonian_matrix(n):
    I2, X, Z = np.eye(2), np.array([[0, 1], [1, 0]]), np.diag([1.0, -1.0])

    def op(single, q):
        out = np.array([[1.0]])
        for k in range(n):
            out = np.kron(out, single if k == q else I2)
        return out

    H = np.zeros((2**n, 2**n))
    for i in range(n - 1):
        H -= op(Z, i) @ op(Z, i + 1)
    for i in range(n):
        H -= 0.7 * op(X, i)
    x = random_state(n, 3)
    assert abs(tfim_energy_dense(x, n, 0.7) - np.real(np.vdot(x, H @ x))) < 1e-13


def test_lower_density_is_u_rho_udagger():
    """The 2n-qubit ops of a density-matrix program, applied densely to the row-major
    rho, give U rho U^dagger (row qubit q = qubit q, column qubit q = qubit q + n)."""
    from qibojit_gb300.fusion import lower_density

    rng = np.random.default_rng(3)
    n = 3
    c = G.Circuit(n)
    c.add([G.U3(0, *rng.uniform(0, 6, 3)), G.CNOT(2, 1), G.CU1(1, 0, theta=0.7), G.fSim(0, 2, 0.3, 0.4),
           G.Y(1), G.FanOut(0, 1, 2)])
    a = rng.standard_normal((8, 8)) + 1j * rng.standard_normal((8, 8))
    rho = a @ a.conj().T
    vec = rho.reshape(-1)
    ops = lower_density(c.queue, n)
    assert len(ops) == 2 * len(lower(c.queue))
    for kind, targets, controls, entries in ops:
        k = len(targets)
        m = np.diag(entries) if kind == SV_OP_DIAG else entries.reshape(2**k, 2**k)
        vec = apply_dense(vec, m, list(targets), list(controls), 2 * n)
    u = np.eye(8, dtype=complex)
    for g in c.queue:
        for t in (g.target_qubits if type(g).__name__ == "FanOut" else [None]):
            if t is None:
                cols = [apply_dense(u[:, j], g.base_matrix(), list(g.target_qubits), list(g.control_qubits), n)
                        for j in range(8)]
            else:
                cols = [apply_dense(u[:, j], Matrices().X, [t], list(g.control_qubits), n) for j in range(8)]
            u = np.stack(cols, axis=1)
    np.testing.assert_allclose(vec.reshape(8, 8), u @ rho @ u.conj().T, atol=1e-12)


def test_channels_expose_the_reference_attributes():
    ch = G.PauliNoiseChannel(1, px=0.1, pz=0.25)
    assert ch.coefficients == (0.1, 0.25) and [type(g).__name__ for g in ch.gates] == ["X", "Z"]
    assert abs(ch.coefficient_sum - 0.35) < 1e-15 and ch._all_unitary_operators and ch.qubits == (1,)
    u = G.UnitaryChannel([0.2, 0.3], [((0, 2), np.eye(4)), ((1,), np.eye(2))])
    assert [g.target_qubits for g in u.gates] == [(0, 2), (1,)] and u.qubits == (0, 1, 2)
    with pytest.raises(ValueError):
        G.UnitaryChannel([0.7, 0.6], [((0,), np.eye(2)), ((1,), np.eye(2))])
    with pytest.raises(ValueError):
        G.Channel([0.1], [])
    c = G.Circuit(3)
    c.add(ch)
    with pytest.raises(ValueError):
        c.add(G.PauliNoiseChannel(3, px=0.1))


@pytest.mark.parametrize("gate", [G.RX(0, 0.3), G.U3(1, 0.1, 0.2, 0.3), G.CU1(0, 1, 0.7), G.CRX(2, 0, 0.4),
                                  G.TOFFOLI(0, 1, 2), G.CCZ(2, 1, 0), G.fSim(0, 1, 0.2, 0.5), G.CU3(1, 2, 0.3, 0.2, 0.1)],
                         ids=lambda g: type(g).__name__)
def test_inverse_target_matrix(gate):
    """The inverse a density-matrix gate applies with inverse=True: controls kept, the
    target block inverted."""
    from qibojit_gb300.backend import _inverse_target_matrix

    u = gate.base_matrix()
    inv = _inverse_target_matrix(gate, None)
    np.testing.assert_allclose(inv @ u, np.eye(u.shape[0]), atol=1e-14)
    full = gate.matrix()
    controlled_inv = np.eye(full.shape[0], dtype=complex)
    controlled_inv[-u.shape[0]:, -u.shape[0]:] = inv
    np.testing.assert_allclose(controlled_inv, np.linalg.inv(full), atol=1e-14)


def test_circuit_fingerprint_follows_content():
    """execute_circuit's program cache is keyed by circuit content: equal circuits
    share a key, and any change of a gate's parameters, qubits or class (nested
    FusedGate components included) gives a new one."""
    from qibojit_gb300 import circuits
    from qibojit_gb300 import gates as G
    from qibojit_gb300.backend import _circuit_fingerprint as fp

    a, b = circuits.brickwork(8, 3, 5), circuits.brickwork(8, 3, 5)
    assert fp(a) == fp(b)
    b.queue[4].parameters = (0.1, 0.2, 0.3)
    assert fp(a) != fp(b)
    c = circuits.brickwork(8, 3, 5)
    c.queue[-1] = G.CZ(5, 6)
    assert fp(a) != fp(c)
    f1, f2 = G.Circuit(3), G.Circuit(3)
    for f, th in ((f1, 0.5), (f2, 0.6)):
        fg = G.FusedGate(0, 1)
        fg.append(G.RX(0, theta=th))
        fg.append(G.CNOT(0, 1))
        f.add(fg)
    assert fp(f1) != fp(f2)
