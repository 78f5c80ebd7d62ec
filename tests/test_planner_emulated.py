"""The planner's output checked on the host: every pass block of a planned program is
run by a numpy restatement of the tile kernel (``tests/pass_emulator.py``) and the
result compared with the circuit applied gate by gate with dense matrices.  This
covers the plans the GPU runs (complex128 phase-folded, complex64 unfolded, and the
complex64 plan that specialisation re-folds: ``sv_program_specialize`` re-plans before
it needs a device, so on this machine it stops at device selection with the folded
plan in place) without a GPU."""
import ctypes

import numpy as np
import pytest

from qibojit_gb300 import _lib, circuits
from qibojit_gb300 import gates as G
from qibojit_gb300.matrices import Matrices
from tests import pass_emulator as E
from tests.circuits_random import random_circuit
from tests.dense import apply_dense, random_state
from tests.test_planner_cpu import _create

FUSABLE = ["one", "one_p", "two_c", "two_p", "swap", "fsim", "gfsim", "toffoli", "ccz", "deutsch", "u1q", "u2q",
           "cu1q", "cu2q", "fanout", "zc"]


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def dense_reference(circ, state):
    n = circ.nqubits
    out = np.array(state, dtype=np.complex128)
    for g in circ.queue:
        if type(g).__name__ == "FanOut":
            for t in g.target_qubits:
                out = apply_dense(out, Matrices().X, [t], list(g.control_qubits), n)
        elif type(g).__name__ == "Unitary":
            out = apply_dense(out, g.parameters[0], list(g.target_qubits), list(g.control_qubits), n)
        else:
            out = apply_dense(out, g.base_matrix(), list(g.target_qubits), list(g.control_qubits), n)
    return out


def emulate(lib, circ, dt, tile_bits, refold=False):
    rc, h, ctx, _ = _create(lib, circ, dt, tile_bits)
    assert rc == _lib.SV_OK, _lib.last_error()
    try:
        if refold:
            rc = lib.sv_program_specialize(ctypes.addressof(ctx), h)
            if rc == _lib.SV_ERR_UNSUPPORTED:
                pytest.skip(_lib.last_error())
            assert rc == _lib.SV_ERR_CUDA
        x = random_state(circ.nqubits, 11)
        return x, E.run_program(lib, h, _lib.DTYPE_CODES[dt], x)
    finally:
        lib.sv_program_destroy(h)


@pytest.mark.parametrize("dt,refold", [("complex128", False), ("complex64", False), ("complex64", True)],
                         ids=["c128-folded", "c64", "c64-refolded"])
@pytest.mark.parametrize("n,ngates,seed,tile_bits", [(9, 120, 1, 8), (10, 160, 2, 9), (12, 200, 3, 10),
                                                     (12, 200, 4, 12), (13, 220, 5, 11)])
def test_random_circuit_plans(lib, n, ngates, seed, tile_bits, dt, refold):
    circ = random_circuit(n, ngates, seed, families=FUSABLE)
    x, got = emulate(lib, circ, dt, tile_bits, refold)
    want = dense_reference(circ, x)
    np.testing.assert_allclose(got, want, atol=1e-11 if dt == "complex128" else 2e-5)


@pytest.mark.parametrize("dt,refold", [("complex128", False), ("complex64", True)], ids=["c128", "c64-refolded"])
@pytest.mark.parametrize("name", ["brickwork", "qft", "hea", "diagonal", "permutation"])
def test_structured_circuit_plans(lib, name, dt, refold):
    rng = np.random.default_rng(7)
    if name == "brickwork":
        circ = circuits.brickwork(12, 8, 3)
    elif name == "qft":
        circ = circuits.qft(11)
    elif name == "hea":
        circ = circuits.hea(11, 4)
    elif name == "diagonal":
        circ = G.Circuit(10)
        for _ in range(80):
            q = [int(v) for v in rng.permutation(10)]
            circ.add([G.RZ(q[0], float(rng.uniform(0, 6))), G.CU1(q[1], q[2], float(rng.uniform(0, 6))),
                      G.CZ(q[3], q[4]), G.CCZ(q[5], q[6], q[7])][int(rng.integers(4))])
    else:
        circ = G.Circuit(10)
        for _ in range(80):
            q = [int(v) for v in rng.permutation(10)]
            circ.add([G.X(q[0]), G.CNOT(q[1], q[2]), G.SWAP(q[3], q[4]), G.TOFFOLI(q[5], q[6], q[7])][int(rng.integers(4))])
    x, got = emulate(lib, circ, dt, 9, refold)
    want = dense_reference(circ, x)
    np.testing.assert_allclose(got, want, atol=1e-11 if dt == "complex128" else 2e-5)


class _HostContext:
    """What FusedProgram reads from a context; the planner never dereferences it."""

    def __init__(self, lib):
        self.lib = lib
        self._buf = ctypes.create_string_buffer(512)
        self.handle = ctypes.addressof(self._buf)


@pytest.mark.parametrize("dt", ["complex128", "complex64"])
@pytest.mark.parametrize("n,ngates,seed", [(4, 40, 21), (5, 70, 22), (6, 90, 23)])
def test_density_matrix_programs(lib, n, ngates, seed, dt):
    """execute_circuit's density-matrix plan (lower_density: U on the rows, conj(U) on the
    columns of the 2n-qubit vector of rho) gives U rho U^dagger."""
    from qibojit_gb300.fusion import FusedProgram, lower_density

    circ = random_circuit(n, ngates, seed, families=FUSABLE)
    prog = FusedProgram(_HostContext(lib), circ.queue, 2 * n, dt, 0, ops=lower_density(circ.queue, n))
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((2**n, 2**n)) + 1j * rng.standard_normal((2**n, 2**n))
    rho = a @ a.conj().T
    rho /= np.trace(rho)
    got = E.run_program(lib, prog._h, _lib.DTYPE_CODES[dt], rho.reshape(-1)).reshape(2**n, 2**n)
    u = np.stack([dense_reference(circ, np.eye(2**n)[:, k]) for k in range(2**n)], axis=1)
    np.testing.assert_allclose(got, u @ rho @ u.conj().T, atol=1e-11 if dt == "complex128" else 2e-5)


def test_qibo_fused_gates_are_planned_as_their_parts(lib):
    """A FusedGate (qibo's Circuit.fuse output) is lowered to its component gates."""
    from qibojit_gb300.fusion import FusedProgram, matrix_fused

    rng = np.random.default_rng(4)
    n = 9
    circ = G.Circuit(n)
    ref = G.Circuit(n)
    for k in range(12):
        q = sorted(int(v) for v in rng.choice(n, 3, replace=False))
        fg = G.FusedGate(*q)
        for g in [G.U3(q[0], *rng.uniform(0, 6, 3)), G.CNOT(q[0], q[2]), G.RY(q[1], float(rng.uniform(0, 6))),
                  G.CZ(q[1], q[2]), G.SWAP(q[0], q[1])]:
            fg.append(g)
        circ.add(fg)
        ref.add(G.Unitary(matrix_fused(fg), *q))
    prog = FusedProgram(_HostContext(lib), circ.queue, n, "complex128", 8)
    x = random_state(n, 5)
    np.testing.assert_allclose(E.run_program(lib, prog._h, _lib.SV_C128, x), dense_reference(ref, x), atol=1e-12)


def _tally(ps) -> float:
    """The arithmetic model restated over a decoded pass block (lane instructions per
    amplitude: complex 2x2 8, real 2x2 4, pivoted 2, complex 4x4 16, diagonal 4)."""
    total = 0.0
    for op in ps["ops"]:
        t = op["type"]

        def bases(targets):  # mask bits of pair (quadruple) bases: target bits clear
            return sum(1 for j in range(16) if not (j & targets) and (op["jmask"] >> j) & 1)

        one, two = 1 << op["u0"], (1 << op["u0"]) | (1 << op["u1"])
        cost = {E.FOP_D1RUN: 8.0 * op["nrun"], E.FOP_D1RUNR: 4.0 * op["nrun"], E.FOP_DIAGR: 4.0,
                E.FOP_DENSE1: bases(one), E.FOP_DENSE1R: 0.5 * bases(one), E.FOP_DENSE1P: 0.25 * bases(one),
                E.FOP_DENSE2: 4.0 * bases(two), E.FOP_DIAG: 0.25 * bases(0)}.get(t, 0.0)
        if t not in (E.FOP_D1RUN, E.FOP_D1RUNR, E.FOP_DIAGR):
            if op["flags"] & E.FLAG_OMASK:
                cost /= 2 ** bin(op["omask"]).count("1")
            if op["flags"] & E.FLAG_TMASK:
                cost /= 2 ** bin(op["tmask"]).count("1")
        total += cost
    return total


@pytest.mark.parametrize("dt,refold", [("complex128", False), ("complex64", False), ("complex64", True)])
@pytest.mark.parametrize("name", ["brickwork", "random"])
def test_arithmetic_count_matches_the_pass_blocks(lib, dt, refold, name):
    """sv_program_arith_per_amplitude against the same model evaluated on the decoded pass
    blocks; the bench circuit's specialised plan (n=30, 2^13 tiles) needs 2,064 FP32
    instructions per amplitude per step (582 pivoted real 2x2s, 195 diagonal tables, 30
    thread-bit diagonals), the count ncu's FFMA + FMUL figures confirm per pass."""
    n = 30 if name == "brickwork" else 12
    circ = circuits.brickwork(n, 20, 1234) if name == "brickwork" else random_circuit(n, 200, 9, families=FUSABLE)
    tile_bits = 13 if (name == "brickwork" and dt == "complex64") else 0
    rc, h, ctx, _ = _create(lib, circ, dt, tile_bits)
    assert rc == _lib.SV_OK, _lib.last_error()
    try:
        if refold:
            rc = lib.sv_program_specialize(ctypes.addressof(ctx), h)
            if rc == _lib.SV_ERR_UNSUPPORTED:
                pytest.skip(_lib.last_error())
        got = ctypes.c_double()
        _lib.check(lib.sv_program_arith_per_amplitude(h, ctypes.byref(got)))
        passes = ctypes.c_int()
        _lib.check(lib.sv_program_stats(h, ctypes.byref(passes), None, None, None))
        want = sum(_tally(E.read_pass(lib, h, i, _lib.DTYPE_CODES[dt])) for i in range(passes.value))
        assert got.value == pytest.approx(want, rel=1e-12)
        if name == "brickwork" and dt == "complex64" and refold:
            assert got.value == pytest.approx(2064.0)
    finally:
        lib.sv_program_destroy(h)
