"""complex128 one- and two-target dense gates in double-word arithmetic (pairs of
floats on the FP32 pipe) against the FP64 kernels and the oracle: every gate family
that takes the path (apply_gate, apply_z_pow, apply_two_qubit_gate, apply_fsim), with
and without controls, at states whose amplitudes span many magnitudes."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.conftest import PARITY_ATOL
from tests.dense import random_state, random_unitary

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    b = MetaBackend.load("gb300")
    yield b
    b.ctx.set_c128_arithmetic("double-word")


def _run(backend, mode, state, fn):
    backend.ctx.set_c128_arithmetic(mode)
    s = backend.cast(state, dtype="complex128", copy=True)
    out = backend.to_numpy(fn(s))
    backend.ctx.set_c128_arithmetic("double-word")
    return out


def _wide_state(n, seed):
    """Normalised state whose amplitudes range over ~30 orders of magnitude."""
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(2**n) + 1j * rng.standard_normal(2**n)) * 10.0 ** rng.uniform(-30, 0, 2**n)
    return x / np.linalg.norm(x)


def _row_scale(apply, state, gate):
    """sum_j |g_ij| |x_j| for every output: the magnitude the rounding of a gate row is
    proportional to (computed by the oracle's kernel on absolute values)."""
    return np.abs(apply(np.abs(state).astype(np.complex128), np.abs(np.asarray(gate)).astype(np.complex128)))


ONE = [(12, 0, []), (12, 11, []), (14, 5, [2]), (14, 13, [0, 7]), (20, 9, []), (20, 19, [3, 4, 5])]


@pytest.mark.parametrize("n,target,controls", ONE)
@pytest.mark.parametrize("kernel", ["apply_gate", "apply_z_pow"])
def test_one_target_double_word_vs_oracle_and_fp64(backend, n, target, controls, kernel):
    ob = O.OracleBackend()
    q = ob.qubits_tensor(n, [target], controls)
    gate = random_unitary(2, n + target) if kernel == "apply_gate" else np.array(np.exp(0.7j))
    oracle = lambda x, g: ob._one_qubit_base(x.copy(), n, target, kernel, g, q)  # noqa: E731
    for state in (random_state(n, 3 + n), _wide_state(n, 4 + n)):
        fn = lambda s: backend._one_qubit_base(s, n, target, kernel, gate, q)  # noqa: E731
        dwr = _run(backend, "double-word", state, fn)
        f64 = _run(backend, "fp64", state, fn)
        want = oracle(state, gate)
        np.testing.assert_allclose(dwr, want, rtol=0, atol=PARITY_ATOL["complex128"])
        np.testing.assert_allclose(dwr, f64, rtol=0, atol=1e-13)
        # every output within 2^-43 of its row scale (amplitudes above the 2^-103 floor)
        assert np.all(np.abs(dwr - want) <= 1.2e-13 * _row_scale(oracle, state, gate) + 1e-28)


TWO = [(10, 0, 1, []), (10, 9, 3, []), (14, 2, 11, [5]), (16, 15, 0, [3, 8]), (20, 4, 17, [])]


@pytest.mark.parametrize("n,t1,t2,controls", TWO)
@pytest.mark.parametrize("kernel", ["apply_two_qubit_gate", "apply_fsim"])
def test_two_target_double_word_vs_oracle_and_fp64(backend, n, t1, t2, controls, kernel):
    ob = O.OracleBackend()
    q = ob.qubits_tensor(n, [t1, t2], controls)
    if kernel == "apply_two_qubit_gate":
        gate = random_unitary(4, n + t1 + t2)
    else:
        u = random_unitary(2, n)
        gate = np.array([u[0, 0], u[0, 1], u[1, 0], u[1, 1], np.exp(-0.3j)])
    oracle = lambda x, g: ob._two_qubit_base(x.copy(), n, t1, t2, kernel, g, q)  # noqa: E731
    for state in (random_state(n, 5 + n), _wide_state(n, 6 + n)):
        fn = lambda s: backend._two_qubit_base(s, n, t1, t2, kernel, gate, q)  # noqa: E731
        dwr = _run(backend, "double-word", state, fn)
        f64 = _run(backend, "fp64", state, fn)
        want = oracle(state, gate)
        np.testing.assert_allclose(dwr, want, rtol=0, atol=PARITY_ATOL["complex128"])
        np.testing.assert_allclose(dwr, f64, rtol=0, atol=1e-13)
        assert np.all(np.abs(dwr - want) <= 1.2e-13 * _row_scale(oracle, state, gate) + 1e-28)


MULTI = [(12, [0, 5, 11], []), (12, [9, 10, 11], []), (14, [3, 7, 1, 12], []), (16, [15, 12, 13, 14], [2]),
         (14, [6, 0, 13], [4, 9]), (13, [0, 2, 4, 6, 8], []), (14, [13, 12, 11, 10, 9, 8], [1]),
         (12, [5, 1, 9, 3, 11, 7, 0], [])]


@pytest.mark.parametrize("n,targets,controls", MULTI)
def test_multi_target_double_word_vs_oracle_and_fp64(backend, n, targets, controls):
    """3 to 7 targets (any bits, with and without controls) in double-word arithmetic,
    against the oracle and the FP64 kernels, on states spanning many magnitudes."""
    ob = O.OracleBackend()
    q = ob.qubits_tensor(n, targets, controls)
    gate = random_unitary(2 ** len(targets), n + len(targets))
    oracle = lambda x, g: ob._multi_qubit_base(x.copy(), n, targets, g, q)  # noqa: E731
    for state in (random_state(n, 7 + n), _wide_state(n, 8 + n)):
        fn = lambda s: backend._multi_qubit_base(s, n, targets, gate, q)  # noqa: E731
        dwr = _run(backend, "double-word", state, fn)
        f64 = _run(backend, "fp64", state, fn)
        want = oracle(state, gate)
        np.testing.assert_allclose(dwr, want, rtol=0, atol=PARITY_ATOL["complex128"])
        np.testing.assert_allclose(dwr, f64, rtol=0, atol=1e-13)
        assert np.all(np.abs(dwr - want) <= 1.2e-13 * _row_scale(oracle, state, gate) + 1e-28)


def test_double_word_circuit_depth(backend):
    """A 300-gate circuit of dense one- and two-target gates at n=18, gate by gate in
    double-word arithmetic, against the oracle: the per-gate errors stay far below the
    1e-12 bar after many gates."""
    from qibojit_gb300 import gates as G
    from qibojit_gb300.fusion import _target_matrix

    n = 18
    rng = np.random.default_rng(9)
    c = G.Circuit(n)
    for _ in range(300):
        if rng.random() < 0.6:
            c.add(G.U3(int(rng.integers(n)), *rng.uniform(0, 2 * np.pi, 3)))
        else:
            a, b = (int(v) for v in rng.permutation(n)[:2])
            c.add(G.Unitary(random_unitary(4, int(rng.integers(1 << 30))), a, b))
    x = random_state(n, 10)
    backend.set_dtype("complex128")
    got = backend.to_numpy(backend.execute_circuit(c, x, fuse=False))
    ob = O.OracleBackend()
    ref = x.copy()
    for g in c.queue:
        t = list(g.target_qubits)
        ref = ob._multi_qubit_base(ref, n, t, _target_matrix(g), ob.qubits_tensor(n, t))
    np.testing.assert_allclose(got, ref, rtol=0, atol=PARITY_ATOL["complex128"])


def test_double_word_mode_is_rejected_when_unknown(backend):
    with pytest.raises(ValueError):
        backend.ctx.set_c128_arithmetic("fp32")


@pytest.mark.parametrize("specialize", [False, True])
def test_fused_program_double_word_vs_fp64(backend, specialize):
    """The fused complex128 passes in double-word arithmetic (tile converted to float
    pairs in shared memory once per pass) against the same program in FP64, on a
    random circuit of every fusable family and on the brickwork."""
    from qibojit_gb300 import circuits
    from tests.circuits_random import random_circuit

    for circ in (random_circuit(14, 160, 3), circuits.brickwork(16, 12, 4)):
        n = circ.nqubits
        x = random_state(n, 12)
        outs = {}
        for mode in ("double-word", "fp64"):
            backend.ctx.set_c128_arithmetic(mode)
            prog = backend.compile(circ, "complex128", specialize=specialize)
            outs[mode] = backend.to_numpy(prog.run(backend.cast(x, dtype="complex128", copy=True)))
        backend.ctx.set_c128_arithmetic("double-word")
        np.testing.assert_allclose(outs["double-word"], outs["fp64"], rtol=0, atol=PARITY_ATOL["complex128"])


@pytest.mark.parametrize("specialize", [False, True])
def test_batched_circuits_double_word_vs_fp64(backend, specialize):
    """Batched complex128 circuits (the arithmetic is fixed when the batch is created)
    in double-word arithmetic against the same batch in FP64: every state and every
    TFIM energy."""
    from qibojit_gb300.batch import BatchedCircuits, hea_batch, hea_circuit

    specs = hea_batch(24, seed=29, nmin=8, nmax=14, lmin=2, lmax=5)
    circs = [hea_circuit(n, L, p) for n, L, p in specs]
    states, energies = {}, {}
    for mode in ("double-word", "fp64"):
        backend.ctx.set_c128_arithmetic(mode)
        batch = BatchedCircuits(backend, circs, "complex128")
        backend.ctx.set_c128_arithmetic("double-word")
        if specialize:
            batch.specialize()
        batch.run()
        states[mode] = [backend.to_numpy(batch.state(i)) for i in range(len(circs))]
        energies[mode] = np.asarray(batch.tfim_energies(1.0))
        del batch
    for a, b in zip(states["double-word"], states["fp64"]):
        np.testing.assert_allclose(a, b, rtol=0, atol=PARITY_ATOL["complex128"])
    np.testing.assert_allclose(energies["double-word"], energies["fp64"], rtol=0, atol=1e-11)
