"""Pin the CPU oracle against the reference's own outputs and known answers.

The fixtures were produced by running the reference kernels
(src/qibojit/custom_operators/gates.py, ops.py) unchanged in NUMBA_DISABLE_JIT mode
(tests/golden/make_golden.py).  With one OpenMP thread the oracle uses the same
arithmetic order, so gate kernels are required to match bit for bit; Metropolis
frequencies must match exactly for any thread count.
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests import golden_cases

ALL = golden_cases.load()


def _one_thread():
    O.set_threads(1)


@pytest.mark.parametrize("case", [c for c in ALL if c["family"] in ("one", "two", "multi")],
                         ids=lambda c: c["id"])
def test_gate_kernels_bitexact(case):
    _one_thread()
    n = case["nqubits"]
    state = case["state"].copy()
    gate, q = case["gate"], case["qubits"]
    targets = [int(t) for t in case["targets"]]
    be = O.OracleBackend()
    if case["family"] == "one":
        out = be._one_qubit_base(state, n, targets[0], case["kernel"], gate, q)
    elif case["family"] == "two":
        out = be._two_qubit_base(state, n, targets[0], targets[1], case["kernel"], gate, q)
    else:
        out = be._multi_qubit_base(state, n, targets, gate, q)
    if case["family"] == "multi" and len(targets) > 5:
        # the reference's generic kernel sums with np.dot (BLAS order)
        np.testing.assert_allclose(out, case["out"], rtol=0, atol=1e-13 if out.dtype == np.complex128 else 2e-6)
    elif case.get("kernel") == "apply_z_pow":
        # the U1 operand is a 0-d array, so the reference's product goes through
        # NumPy's vectorised complex loop, which may contract to FMA: one rounding
        _ulp_close(out, case["out"])
    else:
        np.testing.assert_array_equal(out, case["out"])


def _ulp_close(a, b, nulp=2):
    eps = np.finfo(a.real.dtype).eps
    np.testing.assert_allclose(a, b, rtol=nulp * eps, atol=nulp * eps * np.abs(b).max())


@pytest.mark.parametrize("case", [c for c in ALL if c["family"] == "collapse"], ids=lambda c: c["id"])
def test_collapse_bitexact(case):
    _one_thread()
    state = case["state"].copy()
    fn = O.collapse_state_normalized if case["normalize"] else O.collapse_state
    out = fn(state, case["qubits"], case["result"], case["nqubits"])
    if case["normalize"]:
        # NumPy's complex abs (used for the norm) may differ from C's hypot in the
        # last bit; everything else is bit-identical
        _ulp_close(out, case["out"], nulp=4)
    else:
        np.testing.assert_array_equal(out, case["out"])


@pytest.mark.parametrize("case", [c for c in ALL if c["family"] == "init"], ids=lambda c: c["id"])
def test_initial_state(case):
    s = O.initial_state_vector(np.full(case["out"].shape, 3, dtype=case["out"].dtype))
    np.testing.assert_array_equal(s, case["out"])


@pytest.mark.parametrize("case", [c for c in ALL if c["family"] == "freq"], ids=lambda c: c["id"])
@pytest.mark.parametrize("threads", [1, 4])
def test_measure_frequencies_exact(case, threads):
    O.set_threads(threads)
    f = O.measure_frequencies(np.zeros(2 ** case["nqubits"], dtype=np.int64), case["probs"],
                              case["nshots"], case["nqubits"], case["seed"], case["nthreads"])
    np.testing.assert_array_equal(f, case["out"])


def test_known_answer_vector():
    """tests/test_ops.py:236-256 of the reference, verbatim numbers."""
    for realtype in ("float32", "float64"):
        for inttype in ("int32", "int64"):
            probs = np.ones(16, dtype=realtype) / 16
            f = O.measure_frequencies(np.zeros(16, dtype=inttype), probs, 1000, 4, 1234, 4)
            assert f.sum() == 1000
            np.testing.assert_array_equal(
                f, np.array([72, 65, 63, 54, 57, 55, 67, 50, 53, 67, 69, 68, 64, 68, 66, 62]))


def test_mt_stream_matches_numpy_legacy():
    rs = np.random.RandomState(4321)
    ref = [rs.randint(0, 1 << 20) if i % 2 == 0 else rs.random() for i in range(2000)]
    a = O.mt_stream(4321, "word", 1)  # warm the library
    assert a.shape == (1,)
    # interleaved stream: randint words then two words per random()
    rs2 = np.random.RandomState(4321)
    words = rs2.randint(0, 2**32, size=3000, dtype=np.uint32).astype(np.uint64)
    got = []
    k = 0
    for i in range(2000):
        if i % 2 == 0:
            got.append(int(words[k] & ((1 << 20) - 1)))
            k += 1
        else:
            a, b = int(words[k]) >> 5, int(words[k + 1]) >> 6
            got.append((a * 67108864.0 + b) / 9007199254740992.0)
            k += 2
    assert got == ref
    np.testing.assert_array_equal(O.mt_stream(4321, "word", 3000), words.astype(np.float64))
    np.testing.assert_array_equal(O.chain_seeds(1234, 3),
                                  [np.random.RandomState(1234).randint(0, int(1e8)) for _ in range(1)] +
                                  list(O.chain_seeds(1234, 3)[1:]))


def test_qft_closed_form():
    """QFT (H + CU1 + SWAPs, benchmarks/abstract.py:86-104) equals sqrt(N) * ifft."""
    be = O.OracleBackend()
    n = 10
    rng = np.random.default_rng(3)
    x = rng.standard_normal(2**n) + 1j * rng.standard_normal(2**n)
    x /= np.linalg.norm(x)
    s = x.copy()
    h = np.array([[1, 1], [1, -1]], dtype=complex) / np.sqrt(2)
    for i1 in range(n):
        s = be._one_qubit_base(s, n, i1, "apply_gate", h, be.qubits_tensor(n, [i1]))
        for i2 in range(i1 + 1, n):
            phase = np.exp(1j * np.pi / 2 ** (i2 - i1))
            s = be._one_qubit_base(s, n, i1, "apply_z_pow", phase, be.qubits_tensor(n, [i1], [i2]))
    for i in range(n // 2):
        s = be._two_qubit_base(s, n, i, n - i - 1, "apply_swap", None, be.qubits_tensor(n, [i, n - i - 1]))
    np.testing.assert_allclose(s, np.sqrt(2**n) * np.fft.ifft(x), atol=1e-13)


def test_probabilities_semantics():
    """Marginal |psi|^2 with qubits[0] the most significant output bit."""
    n = 5
    rng = np.random.default_rng(1)
    x = rng.standard_normal(2**n) + 1j * rng.standard_normal(2**n)
    x /= np.linalg.norm(x)
    t = np.abs(x.reshape((2,) * n)) ** 2
    for qubits in ([0], [3, 1], [4, 0, 2], [0, 1, 2, 3, 4], [2, 4, 1, 0, 3]):
        unmeasured = tuple(i for i in range(n) if i not in qubits)
        p = t.sum(axis=unmeasured)
        kept = [i for i in range(n) if i in qubits]
        p = np.transpose(p, [kept.index(q) for q in qubits]).ravel()
        np.testing.assert_allclose(O.probabilities(x, qubits, n), p, atol=1e-15)


@pytest.mark.parametrize("nbits,nshots,seed,pdt", [(3, 50, 1, "float64"), (10, 999, 2, "float64"),
                                                   (12, 5000, 3, "float32"), (16, 99999, 4, "float64")])
def test_sample_shots_restatement_is_numpy_choice(nbits, nshots, seed, pdt):
    """The direct-sampling oracle reproduces numpy.random.choice(N, nshots, p) (qibo's
    sample_shots) draw for draw from the same global-stream uniforms, zeros included."""
    rng = np.random.default_rng(seed)
    p = rng.random(2**nbits)
    p[rng.random(2**nbits) < 0.3] = 0
    p = (p / p.sum()).astype(pdt)
    p = p / p.sum()
    np.random.seed(seed)
    want = np.random.choice(range(len(p)), size=nshots, p=p)
    np.random.seed(seed)
    got = O.sample_shots(p, np.random.random_sample(nshots))
    np.testing.assert_array_equal(got, want)
    assert np.all(p[got] > 0)
