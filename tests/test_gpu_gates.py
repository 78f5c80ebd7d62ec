"""Gate kernels on the GPU, checked the way qibojit's tests/test_gates.py checks its
backends (same placement tables), against two oracles:

* the reference's own kernel outputs (golden fixtures from the reference's Numba
  kernels run as Python) and the C restatement of those kernels, at the engine's
  parity bar: complex128 max-abs <= 1e-12, complex64 <= 1e-5;
* a dense numpy application of the gate's textbook matrix, at the reference
  suite's tolerances (ATOL 1e-10 / 1e-4, tests/test_gates.py:15).
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests import golden_cases
from tests.conftest import ATOL, PARITY_ATOL
from tests.dense import apply_dense, random_complex, random_state, random_unitary

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    return MetaBackend.load("gb300")


def _run(backend, fn, state, *args):
    s = backend.cast(state, dtype=str(state.dtype), copy=True)
    out = fn(s, *args)
    return backend.to_numpy(out)


# ------------------------------------------------ kernel-level parity (golden fixtures)
GOLDEN = [c for c in golden_cases.load() if c["family"] in ("one", "two", "multi")]


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: c["id"])
def test_kernels_match_reference_outputs(backend, case):
    n = case["nqubits"]
    targets = [int(t) for t in case["targets"]]
    state, gate, q = case["state"], case["gate"], case["qubits"]
    if case["family"] == "one":
        got = _run(backend, lambda s: backend._one_qubit_base(s, n, targets[0], case["kernel"], gate, q), state)
    elif case["family"] == "two":
        got = _run(backend, lambda s: backend._two_qubit_base(s, n, targets[0], targets[1], case["kernel"], gate, q),
                   state)
    else:
        got = _run(backend, lambda s: backend._multi_qubit_base(s, n, targets, gate, q), state)
    tol = PARITY_ATOL[str(state.dtype)]
    np.testing.assert_allclose(got, case["out"], rtol=0, atol=tol * _rounding_scale(case))


def _oracle_apply(case, state, gate):
    """The C oracle's kernel of a golden case on (state, gate)."""
    ob = O.OracleBackend()
    n, q, kernel = case["nqubits"], case["qubits"], case["kernel"]
    targets = [int(t) for t in case["targets"]]
    s = np.array(state, copy=True)
    if case["family"] == "one":
        return ob._one_qubit_base(s, n, targets[0], kernel, gate, q)
    if case["family"] == "two":
        return ob._two_qubit_base(s, n, targets[0], targets[1], kernel, gate, q)
    return ob._multi_qubit_base(s, n, targets, gate, q)


def _rounding_scale(case):
    """max(1, max over outputs of sum_j |g_ij| |x_j|): the magnitude that floating-point
    rounding of a gate row's dot product is proportional to.  The fixtures use
    un-normalised random operands (as the reference's tests do), whose outputs reach
    a few units; the absolute bar is applied relative to this scale."""
    gate = case["gate"]
    if gate is None or case["kernel"] in ("apply_x", "apply_y", "apply_z", "apply_swap"):
        return 1.0
    a = _oracle_apply(case, np.abs(case["state"]).astype(np.complex128), np.abs(gate).astype(np.complex128))
    return max(1.0, float(np.abs(a).max()))


UNITARY_CASES = [c for c in GOLDEN if c["kernel"] in ("apply_gate", "apply_two_qubit_gate", "apply_multi_qubit_gate")
                 or c["family"] == "multi"]


@pytest.mark.parametrize("case", UNITARY_CASES, ids=lambda c: c["id"])
def test_kernels_match_oracle_unitary_operands_unscaled(backend, case):
    """Every golden placement again with a normalised state and a random unitary
    operand, against the C oracle at the unscaled bar (complex128 1e-12, complex64
    1e-5 max-abs)."""
    n = case["nqubits"]
    targets = [int(t) for t in case["targets"]]
    dtype = str(case["state"].dtype)
    k = len(targets)
    gate = random_unitary(2**k, 1000 + len(case["id"]) + n).astype(dtype)
    state = random_state(n, 2000 + n + k, dtype)
    q = case["qubits"]
    if case["family"] == "one":
        got = _run(backend, lambda s: backend._one_qubit_base(s, n, targets[0], case["kernel"], gate, q), state)
    elif case["family"] == "two":
        got = _run(backend, lambda s: backend._two_qubit_base(s, n, targets[0], targets[1], case["kernel"], gate, q),
                   state)
    else:
        got = _run(backend, lambda s: backend._multi_qubit_base(s, n, targets, gate, q), state)
    want = _oracle_apply(case, state, gate)
    np.testing.assert_allclose(got, want, rtol=0, atol=PARITY_ATOL[dtype])


@pytest.mark.parametrize("use_qubits", [False, True])
@pytest.mark.parametrize(("nqubits", "target"), [(4, 1), (6, 5)])
def test_one_qubit_base(backend, nqubits, target, use_qubits, dtype):
    state = random_state(nqubits, 11, dtype)
    matrix = random_complex((2, 2), 12, dtype)
    qubits = O.OracleBackend.qubits_tensor(nqubits, [target]) if use_qubits else None
    got = _run(backend, lambda s: backend._one_qubit_base(s, nqubits, target, "apply_gate", matrix, qubits), state)
    want = apply_dense(state, matrix, [target], [], nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])


# --------------------------------------------------------- gate-level (dense oracle)
ONE_Q = [(5, 4, []), (4, 2, []), (3, 0, []), (8, 5, []), (3, 0, [1, 2]), (4, 3, [0, 1, 2]),
         (5, 3, [1]), (5, 2, [1, 4]), (6, 3, [0, 2, 5]), (6, 3, [0, 2, 4, 5])]


@pytest.mark.parametrize(("nqubits", "target", "controls"), ONE_Q)
def test_apply_gate(backend, nqubits, target, controls, dtype):
    from qibojit_gb300 import gates

    backend.set_dtype(dtype)
    state = random_state(nqubits, 10, dtype)
    matrix = random_unitary(2, 10).astype(dtype)
    gate = gates.Unitary(matrix, target).controlled_by(*controls)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = apply_dense(state, matrix, [target], controls, nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])


@pytest.mark.parametrize("pauli", ["X", "Y", "Z"])
@pytest.mark.parametrize(("nqubits", "target", "controls"),
                         [(3, 0, []), (4, 3, []), (5, 2, []), (3, 1, []), (3, 0, [1]), (4, 3, [0, 1]),
                          (5, 2, [1, 3, 4])])
def test_apply_pauli_gate(backend, nqubits, target, pauli, controls, dtype):
    from qibojit_gb300 import gates

    backend.set_dtype(dtype)
    state = random_state(nqubits, 3, dtype)
    gate = getattr(gates, pauli)(target).controlled_by(*controls)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = apply_dense(state, gate.base_matrix(), [target], controls, nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])


@pytest.mark.parametrize(("nqubits", "target", "controls"),
                         [(3, 0, []), (3, 2, [1]), (3, 2, [0, 1]), (6, 1, [0, 2, 4])])
def test_apply_zpow_gate(backend, nqubits, target, controls, dtype):
    from qibojit_gb300 import gates

    backend.set_dtype(dtype)
    state = random_state(nqubits, 4, dtype)
    gate = gates.U1(target, theta=0.1234).controlled_by(*controls)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = apply_dense(state, gate.base_matrix(), [target], controls, nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])


TWO_Q = [(5, [3, 4], []), (4, [2, 0], []), (2, [0, 1], []), (8, [6, 3], []), (3, [0, 1], [2]),
         (4, [1, 3], [0]), (5, [2, 3], [1, 4]), (5, [3, 1], [0, 2]), (6, [2, 5], [0, 1, 3, 4])]


@pytest.mark.parametrize(("nqubits", "targets", "controls"), TWO_Q)
def test_apply_two_qubit_gate(backend, nqubits, targets, controls, dtype):
    from qibojit_gb300 import gates

    backend.set_dtype(dtype)
    state = random_state(nqubits, 5, dtype)
    matrix = random_unitary(4, 6).astype(dtype)
    gate = gates.Unitary(matrix, *targets).controlled_by(*controls)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = apply_dense(state, matrix, targets, controls, nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])


@pytest.mark.parametrize("use_qubits", [False, True])
@pytest.mark.parametrize(("nqubits", "targets"), [(5, [3, 4]), (4, [2, 0])])
def test_apply_two_qubit_base(backend, nqubits, targets, use_qubits, dtype):
    state = random_state(nqubits, 7, dtype)
    matrix = random_complex((4, 4), 8, dtype)
    qubits = O.OracleBackend.qubits_tensor(nqubits, targets) if use_qubits else None
    got = _run(backend, lambda s: backend._two_qubit_base(s, nqubits, targets[0], targets[1],
                                                          "apply_two_qubit_gate", matrix, qubits), state)
    np.testing.assert_allclose(got, apply_dense(state, matrix, targets, [], nqubits), atol=ATOL[dtype])


@pytest.mark.parametrize("gatename", ["CY", "CH", "CSX", "CSXDG"])
@pytest.mark.parametrize(("nqubits", "targets"),
                         [(2, [0, 1]), (3, [0, 2]), (4, [1, 3]), (3, [1, 2]), (4, [0, 2]), (4, [2, 3]),
                          (5, [3, 4]), (6, [1, 4])])
def test_apply_control_single_qubit_gate(backend, gatename, nqubits, targets, dtype):
    from qibojit_gb300 import gates

    backend.set_dtype(dtype)
    state = random_state(nqubits, 9, dtype)
    gate = getattr(gates, gatename)(*targets)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = apply_dense(state, gate.base_matrix(), [targets[1]], [targets[0]], nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])


@pytest.mark.parametrize(("nqubits", "target", "controls"), [(3, 2, [0, 1]), (4, 2, [1, 3])])
def test_apply_ccz(backend, nqubits, target, controls, dtype):
    from qibojit_gb300 import gates

    backend.set_dtype(dtype)
    state = random_state(nqubits, 13, dtype)
    gate = gates.CCZ(*controls, target)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = apply_dense(state, gate.base_matrix(), [target], controls, nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])


@pytest.mark.parametrize(("nqubits", "targets"),
                         [(3, [0, 1, 2]), (4, [1, 2, 3]), (4, [0, 2, 3]), (4, [2, 3, 1]), (5, [3, 4, 2]),
                          (6, [1, 2, 4])])
def test_apply_deutsch(backend, nqubits, targets, dtype):
    from qibojit_gb300 import gates

    backend.set_dtype(dtype)
    state = random_state(nqubits, 14, dtype)
    gate = gates.DEUTSCH(*targets, 0.3817)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = apply_dense(state, gate.base_matrix(), [targets[2]], targets[:2], nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])


@pytest.mark.parametrize(("nqubits", "targets", "controls"),
                         [(2, [0, 1], []), (3, [0, 2], []), (4, [1, 3], []), (3, [1, 2], [0]),
                          (4, [0, 2], [1]), (4, [2, 3], [0]), (5, [3, 4], [1, 2]), (6, [1, 4], [0, 2, 5])])
def test_apply_swap(backend, nqubits, targets, controls, dtype):
    from qibojit_gb300 import gates

    backend.set_dtype(dtype)
    state = random_state(nqubits, 15, dtype)
    gate = gates.SWAP(*targets).controlled_by(*controls)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = apply_dense(state, gate.base_matrix(), targets, controls, nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])


@pytest.mark.parametrize(("nqubits", "targets", "controls"),
                         [(3, [0, 1], []), (4, [2, 0], []), (3, [1, 2], [0]), (4, [0, 1], [2]), (5, [0, 1], [2]),
                          (5, [3, 4], [2]), (4, [0, 3], [1]), (4, [3, 2], [0]), (5, [1, 4], [2]),
                          (6, [1, 3], [0, 4]), (6, [5, 0], [1, 2, 3])])
def test_apply_fsim(backend, nqubits, targets, controls, dtype):
    from qibojit_gb300 import gates

    backend.set_dtype(dtype)
    state = random_state(nqubits, 16, dtype)
    matrix = random_complex((2, 2), 17, dtype)
    gate = gates.GeneralizedfSim(*targets, matrix, 0.4321).controlled_by(*controls)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = apply_dense(state, gate.base_matrix(), targets, controls, nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype])


@pytest.mark.parametrize("nqubits", [2, 3, 4])
def test_apply_fanout(backend, nqubits):
    from qibojit_gb300 import gates

    backend.set_dtype("complex128")
    state = random_state(nqubits, 18)
    gate = gates.FanOut(*range(nqubits))
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = state.copy()
    for t in range(1, nqubits):
        want = apply_dense(want, np.array([[0, 1], [1, 0]]), [t], [0], nqubits)
    np.testing.assert_allclose(got, want, atol=1e-12)


MULTI = [(3, [0, 1, 2], []), (4, [2, 1, 3], []), (5, [0, 2, 3], []), (8, [2, 6, 3], []),
         (5, [0, 2, 3, 4], []), (8, [0, 4, 2, 5, 7], []), (7, [0, 2, 4, 3, 6, 5], []),
         (8, [0, 4, 2, 3, 5, 7, 1], []), (4, [2, 1, 3], [0]), (5, [0, 2, 3], [1]), (8, [2, 6, 3], [4, 7]),
         (5, [0, 2, 3, 4], [1]), (8, [0, 4, 2, 5, 7], [1, 3]), (10, [9, 1, 5, 3, 7, 0, 8, 2], []),
         (12, [3, 11, 0, 6, 9, 1, 4, 10, 7, 2], [5])]


@pytest.mark.parametrize(("nqubits", "targets", "controls"), MULTI)
def test_apply_multiqubit_gate(backend, nqubits, targets, controls, dtype):
    from qibojit_gb300 import gates

    backend.set_dtype(dtype)
    state = random_state(nqubits, 19, dtype)
    rank = 2 ** len(targets)
    matrix = random_complex((rank, rank), 20, dtype)
    gate = gates.Unitary(matrix, *targets).controlled_by(*controls)
    got = backend.to_numpy(backend.apply_gate(gate, backend.cast(state, copy=True), nqubits))
    want = apply_dense(state, matrix, targets, controls, nqubits)
    np.testing.assert_allclose(got, want, atol=ATOL[dtype] * rank)


@pytest.mark.parametrize(("nqubits", "targets", "controls"),
                         [(10, [0, 4, 2, 5, 9], [1, 3, 7, 8]), (20, [10, 8, 13], []), (20, [11, 19, 13, 4], []),
                          (20, [12, 14, 2, 5, 17], []), (20, [12, 17, 3], [10]), (20, [19, 6, 13], [14, 7]),
                          (20, [0, 19, 3, 14], [1]), (20, [0, 4, 18, 5, 17], [10, 3])])
def test_apply_multiqubit_gate_large(backend, nqubits, targets, controls, dtype):
    """tests/test_gates.py:332-346 sizes, checked against the C oracle kernels."""
    state = random_state(nqubits, 21, dtype)
    rank = 2 ** len(targets)
    matrix = random_complex((rank, rank), 22, dtype)
    q = O.OracleBackend.qubits_tensor(nqubits, targets, controls)
    got = _run(backend, lambda s: backend._multi_qubit_base(s, nqubits, targets, matrix, q), state)
    want = O.OracleBackend()._multi_qubit_base(state.copy(), nqubits, targets, matrix, q)
    np.testing.assert_allclose(got, want, rtol=0, atol=PARITY_ATOL[dtype] * rank)


@pytest.mark.parametrize(("nqubits", "targets", "controls"),
                         [(12, [9, 10, 11], []), (12, [11, 10, 9], []), (20, [16, 17, 18, 19], []),
                          (20, [19, 17, 16, 18], []), (8, [4, 5, 6, 7], []), (9, [6, 7, 8], [0]),
                          (20, [18, 19, 16, 17], [3])])
def test_multi_target_gate_on_lowest_bits(backend, nqubits, targets, controls, dtype):
    """3 and 4 targets on the lowest bits without controls (any target order) take the
    coalesced warp-regrouping kernel once there is at least one warp of groups; with
    fewer groups or with controls the per-thread kernel runs.  Unitary operands, so the
    bar is unscaled."""
    state = random_state(nqubits, 31, dtype)
    matrix = random_unitary(2 ** len(targets), 32).astype(dtype)
    q = O.OracleBackend.qubits_tensor(nqubits, targets, controls)
    got = _run(backend, lambda s: backend._multi_qubit_base(s, nqubits, targets, matrix, q), state)
    want = O.OracleBackend()._multi_qubit_base(state.copy(), nqubits, targets, matrix, q)
    np.testing.assert_allclose(got, want, rtol=0, atol=PARITY_ATOL[dtype])


@pytest.mark.parametrize("use_qubits", [False, True])
@pytest.mark.parametrize(("nqubits", "targets"), [(5, [2, 3, 4]), (4, [2, 0, 1])])
def test_apply_multi_qubit_base(backend, nqubits, targets, use_qubits, dtype):
    state = random_state(nqubits, 23, dtype)
    matrix = random_complex((8, 8), 24, dtype)
    qubits = O.OracleBackend.qubits_tensor(nqubits, targets) if use_qubits else None
    got = _run(backend, lambda s: backend._multi_qubit_base(s, nqubits, targets, matrix, qubits), state)
    np.testing.assert_allclose(got, apply_dense(state, matrix, targets, [], nqubits), atol=ATOL[dtype] * 8)


@pytest.mark.parametrize("gatename", ["H", "X", "Y", "Z", "S", "T", "SX"])
def test_gates_on_circuit(backend, gatename):
    from qibojit_gb300 import gates

    backend.set_dtype("complex128")
    state = random_state(1, 25)
    c = gates.Circuit(1)
    c.add(getattr(gates, gatename)(0))
    got = backend.to_numpy(backend.execute_circuit(c, state))
    np.testing.assert_allclose(got, c.queue[0].base_matrix() @ state, atol=1e-12)


@pytest.mark.parametrize("gatename,params",
                         [("CRX", {"theta": 0.1}), ("CRY", {"theta": 0.1}), ("CRZ", {"theta": 0.1}),
                          ("CU1", {"theta": 0.1}), ("CU2", {"phi": 0.1, "lam": 0.2}),
                          ("CU3", {"theta": 0.1, "phi": 0.2, "lam": 0.3}), ("fSim", {"theta": 0.1, "phi": 0.2})])
def test_parametrized_gates_on_circuit(backend, gatename, params):
    from qibojit_gb300 import gates

    backend.set_dtype("complex128")
    state = random_state(2, 26)
    c = gates.Circuit(2)
    c.add(getattr(gates, gatename)(0, 1, **params))
    got = backend.to_numpy(backend.execute_circuit(c, state))
    np.testing.assert_allclose(got, c.queue[0].matrix() @ state, atol=1e-12)


@pytest.mark.parametrize("dt", ["float64", "float32"])
def test_real_dtypes(backend, dt):
    """float32/float64 states with real gates (the reference compiles all four dtypes)."""
    n = 6
    rng = np.random.default_rng(27)
    state = rng.standard_normal(2**n).astype(dt)
    h = (np.array([[1, 1], [1, -1]]) / np.sqrt(2)).astype(dt)
    s = backend.cast(state, dtype=dt, copy=True)
    backend._one_qubit_base(s, n, 2, "apply_gate", h, None)
    backend._one_qubit_base(s, n, 4, "apply_x", None, O.OracleBackend.qubits_tensor(n, [4], [0]))
    backend._one_qubit_base(s, n, 1, "apply_z", None, None)
    backend._two_qubit_base(s, n, 0, 5, "apply_swap", None, None)
    want = state.copy()
    O.apply_gate_kernel(want, h, 1 << (n - 1), n - 2 - 1)
    O.multicontrol_apply_x_kernel(want, None, O.OracleBackend.qubits_tensor(n, [4], [0]), 1 << (n - 2), n - 4 - 1)
    O.apply_z_kernel(want, None, 1 << (n - 1), n - 1 - 1)
    O.apply_swap_kernel(want, None, 1 << (n - 2), 0, n - 1)
    np.testing.assert_allclose(backend.to_numpy(s), want, atol=PARITY_ATOL[dt])


def test_errors_map_to_reference_exceptions(backend):
    n = 4
    s = backend.zero_state(n)
    with pytest.raises(ValueError):
        backend._one_qubit_base(s, n, 7, "apply_x", None, None)
    with pytest.raises(ValueError):
        backend._multi_qubit_base(s, n, [0, 0, 1], np.eye(8), None)
    with pytest.raises(ValueError):
        backend._multi_qubit_base(backend.zero_state(12), 12, list(range(11)), np.eye(2048), None)
    with pytest.raises(ValueError):  # size mismatch is caught before any launch
        backend._one_qubit_base(s, n + 1, 0, "apply_x", None, None)
    r = backend.cast(np.zeros(2**n), dtype="float64")
    with pytest.raises(NotImplementedError):
        backend._one_qubit_base(r, n, 0, "apply_y", None, None)
