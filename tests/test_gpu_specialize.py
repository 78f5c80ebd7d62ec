"""Pass kernels specialised at run time (sv_program_specialize) against the interpreting
tile kernel, the per-gate path and the oracle."""
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


@pytest.mark.parametrize("n,ngates,seed,tile_bits", [(9, 80, 2, 0), (12, 150, 3, 8), (15, 200, 4, 10),
                                                     (18, 120, 5, 0)])
def test_random_circuits_specialised_vs_interpreted(backend, n, ngates, seed, tile_bits, dtype):
    """Every gate family: controls on register, thread and tile bits, diagonals with
    table bits outside the registers, SWAP, fSim, three-target ops left unfused."""
    circ = random_circuit(n, ngates, seed)
    state = random_state(n, seed + 200, dtype)
    plain = backend.compile(circ, dtype, tile_bits=tile_bits)
    spec = backend.compile(circ, dtype, tile_bits=tile_bits, specialize=True)
    assert spec.specialized and not plain.specialized
    want = backend.to_numpy(plain.run(backend.cast(state, dtype=dtype, copy=True)))
    got = backend.to_numpy(spec.run(backend.cast(state, dtype=dtype, copy=True)))
    np.testing.assert_allclose(got, want, rtol=0, atol=PARITY_ATOL[dtype])
    per_gate = backend.to_numpy(backend.execute_circuit(circ, backend.cast(state, dtype=dtype, copy=True),
                                                        fuse=False))
    np.testing.assert_allclose(got, per_gate, rtol=0, atol=PARITY_ATOL[dtype] * (10 if dtype == "complex64" else 1))


@pytest.mark.parametrize("n,depth", [(10, 20), (20, 6)])
def test_brickwork_specialised_vs_oracle(backend, n, depth):
    circ = circuits.brickwork(n, depth, 17)
    state = random_state(n, 18)
    got = backend.to_numpy(backend.compile(circ, "complex128", specialize=True).run(backend.cast(state, copy=True)))
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


def test_qft_specialised_is_ifft(backend):
    n = 16
    x = random_state(n, 19)
    prog = backend.compile(circuits.qft(n), "complex128", specialize=True)
    got = backend.to_numpy(prog.run(backend.cast(x, copy=True)))
    np.testing.assert_allclose(got, np.sqrt(2**n) * np.fft.ifft(x), atol=1e-12)


def test_execute_circuit_specialises_repeated_programs(backend):
    n = 14
    circ = circuits.brickwork(n, 8, 21)
    x = random_state(n, 22, "complex64")
    first = backend.to_numpy(backend.execute_circuit(circ, x))
    key = next(iter(backend._programs))
    assert not backend._programs[key].specialized
    for _ in range(backend.specialize_after):
        again = backend.to_numpy(backend.execute_circuit(circ, x))
    prog = backend._programs[key]
    assert prog.specialized and prog.stats()["tile_bits"] == 13
    np.testing.assert_allclose(again, first, rtol=0, atol=PARITY_ATOL["complex64"])
    # complex128 programs stay interpreted in double-word arithmetic (compiled double-word
    # passes are slower) and are specialised in FP64 arithmetic
    y = random_state(n, 23)
    first128 = backend.to_numpy(backend.execute_circuit(circ, y))
    for _ in range(backend.specialize_after):
        again128 = backend.to_numpy(backend.execute_circuit(circ, y))
    assert not backend._programs[next(iter(backend._programs))].specialized
    np.testing.assert_allclose(again128, first128, rtol=0, atol=1e-13)
    backend.ctx.set_c128_arithmetic("fp64")
    try:
        for _ in range(backend.specialize_after):
            f64 = backend.to_numpy(backend.execute_circuit(circ, y))
        assert backend._programs[next(iter(backend._programs))].specialized
        np.testing.assert_allclose(f64, first128, rtol=0, atol=1e-13)
    finally:
        backend.ctx.set_c128_arithmetic("double-word")


@pytest.mark.parametrize("dt", ["complex64", "complex128"])
def test_large_brickwork_specialised_matches_interpreted(backend, dt):
    """n = 26: every pass of the full-depth brickwork; both paths from the same state,
    compared in FP64 on the device."""
    n = 26
    circ = circuits.brickwork(n, 20, 23)
    a = backend.zero_state(n, dtype=dt)
    b = backend.zero_state(n, dtype=dt)
    backend.compile(circ, dt).run(a)
    backend.compile(circ, dt, specialize=True).run(b)
    tol = 1e-6 if dt == "complex64" else 1e-13
    assert backend.max_abs_diff(a, b, n) < tol
    assert abs(backend.norm2(b, n) - 1) < (1e-5 if dt == "complex64" else 1e-12)


def _families(n, kind, seed):
    from qibojit_gb300 import gates as G

    rng = np.random.default_rng(seed)
    c = G.Circuit(n)
    for _ in range(6 * n):
        q = [int(x) for x in rng.permutation(n)]
        t = float(rng.uniform(0, 2 * np.pi))
        if kind == "diagonal":
            c.add([G.CZ(q[0], q[1]), G.RZ(q[0], t), G.CU1(q[0], q[1], t), G.T(q[0]), G.Z(q[0]),
                   G.CCZ(q[0], q[1], q[2])][int(rng.integers(6))])
        elif kind == "permutation":
            c.add([G.X(q[0]), G.CNOT(q[0], q[1]), G.SWAP(q[0], q[1]), G.TOFFOLI(q[0], q[1], q[2])][int(rng.integers(4))])
        else:  # real rotations and Hadamards
            c.add([G.RY(q[0], t), G.H(q[0])][int(rng.integers(2))])
    return c


@pytest.mark.parametrize("kind", ["diagonal", "permutation", "real"])
@pytest.mark.parametrize("n,tile_bits", [(8, 8), (13, 0)])
def test_special_gate_families_specialised(backend, kind, n, tile_bits, dtype):
    """Circuits of only diagonal, only permutation or only real gates (no folding
    material, sign tables only, runs of real rotations) at the smallest state a fused
    program takes (n = 8, one tile) and at n = 13."""
    circ = _families(n, kind, 31)
    state = random_state(n, 32, dtype)
    spec = backend.compile(circ, dtype, tile_bits=tile_bits, specialize=True)
    got = backend.to_numpy(spec.run(backend.cast(state, dtype=dtype, copy=True)))
    want = backend.to_numpy(backend.execute_circuit(circ, backend.cast(state, dtype=dtype, copy=True), fuse=False))
    np.testing.assert_allclose(got, want, rtol=0, atol=PARITY_ATOL[dtype] * (10 if dtype == "complex64" else 1))


def test_empty_circuit_specialised(backend):
    from qibojit_gb300 import gates as G

    x = random_state(10, 33, "complex64")
    prog = backend.compile(G.Circuit(10), "complex64", specialize=True)
    got = backend.to_numpy(prog.run(backend.cast(x, dtype="complex64", copy=True)))
    np.testing.assert_array_equal(got, x)
