"""Fused execution (cache-blocked passes) against the per-gate path and the oracle."""
import numpy as np
import pytest

from oracle import pyoracle as O
from qibojit_gb300 import circuits
from tests.circuits_random import random_circuit
from tests.conftest import PARITY_ATOL
from tests.dense import random_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    return MetaBackend.load("gb300")


def _per_gate(backend, circ, state, dtype):
    s = backend.cast(state, dtype=dtype, copy=True)
    return backend.to_numpy(backend.execute_circuit(circ, s, fuse=False))


@pytest.mark.parametrize("tile_bits", [0, 8, 10])
@pytest.mark.parametrize("n,ngates,seed", [(8, 60, 1), (9, 80, 2), (12, 150, 3), (15, 200, 4), (18, 120, 5)])
def test_random_circuits_fused_vs_per_gate(backend, n, ngates, seed, tile_bits, dtype):
    circ = random_circuit(n, ngates, seed)
    state = random_state(n, seed + 100, dtype)
    want = _per_gate(backend, circ, state, dtype)
    prog = backend.compile(circ, dtype, tile_bits=min(tile_bits, n) if tile_bits else 0)
    got = backend.to_numpy(prog.run(backend.cast(state, dtype=dtype, copy=True)))
    st = prog.stats()
    assert st["fused_gates"] + st["unfused"] >= 1
    tol = PARITY_ATOL[dtype] * (10 if dtype == "complex64" else 1)
    np.testing.assert_allclose(got, want, rtol=0, atol=tol)


@pytest.mark.parametrize("n,depth", [(10, 20), (16, 12), (20, 6)])
def test_brickwork_fused_vs_oracle(backend, n, depth):
    circ = circuits.brickwork(n, depth, 7)
    state = random_state(n, 8)
    got = backend.to_numpy(backend.compile(circ, "complex128").run(backend.cast(state, copy=True)))
    ref = state.copy()
    ob = O.OracleBackend()
    cm = backend.custom_matrices
    for g in circ.queue:
        q = ob.qubits_tensor(n, g.target_qubits, g.control_qubits)
        if type(g).__name__ == "U3":
            ob._one_qubit_base(ref, n, g.target_qubits[0], "apply_gate", cm.U3(*g.parameters), q)
        else:
            ob._one_qubit_base(ref, n, g.target_qubits[0], "apply_z", None, q)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12)


def test_brickwork_plan_is_compact(backend):
    prog = backend.compile(circuits.brickwork(30, 20, 1234), "complex64")
    st = prog.stats()
    # engine ops after planning (edge qubits' consecutive U3s merge into one op; a
    # phase-folded plan writes each U3 as a real rotation plus carried diagonals)
    assert st["unfused"] == 0 and 850 <= st["fused_gates"] < 2 * 890
    assert st["passes"] < 890 // 8


@pytest.mark.parametrize("n", [10, 16, 20])
def test_qft_fused_is_ifft(backend, n):
    x = random_state(n, 9)
    got = backend.to_numpy(backend.execute_circuit(circuits.qft(n), x, fuse=True))
    np.testing.assert_allclose(got, np.sqrt(2**n) * np.fft.ifft(x), atol=1e-12)


def test_fused_program_rejects_wrong_state(backend):
    prog = backend.compile(circuits.brickwork(10, 2, 1), "complex128")
    with pytest.raises(ValueError):
        prog.run(backend.zero_state(11))
    with pytest.raises(TypeError):
        prog.run(backend.zero_state(10, dtype="complex64"))


def test_execute_circuit_cache_follows_circuit_content(backend):
    """Circuits built one after another (a freed circuit's id is reused by the next)
    and a circuit edited in place each run their own gates, with the program cache
    and its specialisation in between."""
    x = random_state(12, 3)
    for seed in range(5):
        c = circuits.brickwork(12, 3, seed)
        for _ in range(3):
            got = backend.to_numpy(backend.execute_circuit(c, x, fuse=True))
        want = backend.to_numpy(backend.execute_circuit(c, x, fuse=False))
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)
        del c
    c = circuits.brickwork(12, 3, 9)
    backend.execute_circuit(c, x)
    c.queue[0].parameters = (0.3, 0.2, 0.1)
    got = backend.to_numpy(backend.execute_circuit(c, x, fuse=True))
    want = backend.to_numpy(backend.execute_circuit(c, x, fuse=False))
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)
