"""State creation, collapse, probabilities and Metropolis sampling on the GPU,
following qibojit's tests/test_ops.py, with the reference's own outputs (golden
fixtures) and the C oracle as checkers."""
import itertools

import numpy as np
import pytest

from oracle import pyoracle as O
from tests import golden_cases
from tests.conftest import PARITY_ATOL
from tests.dense import random_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    return MetaBackend.load("gb300")


@pytest.mark.parametrize("dt", ["complex128", "complex64", "float64", "float32"])
@pytest.mark.parametrize("n", [1, 2, 4, 11])
def test_zero_state(backend, dt, n):
    s = backend.zero_state(n, dtype=dt)
    want = np.zeros(2**n, dtype=dt)
    want[0] = 1
    np.testing.assert_array_equal(backend.to_numpy(s), want)


@pytest.mark.parametrize("case", [c for c in golden_cases.load() if c["family"] == "init"], ids=lambda c: c["id"])
def test_zero_state_golden(backend, case):
    s = backend.zero_state(case["nqubits"], dtype=str(case["out"].dtype))
    np.testing.assert_array_equal(backend.to_numpy(s), case["out"])


@pytest.mark.parametrize("case", [c for c in golden_cases.load() if c["family"] == "collapse"],
                         ids=lambda c: c["id"])
def test_collapse_matches_reference_outputs(backend, case):
    n = case["nqubits"]
    state = case["state"]
    s = backend.cast(state, dtype=str(state.dtype), copy=True)
    # the fixture stores the measured qubits sorted and the outcome MSB-first, as the
    # reference backend receives them (tests/test_ops.py:73-82)
    targets = [int(t) for t in np.atleast_1d(case["targets"])]
    backend.collapse_state(s, targets, int(case["result"]), n, bool(case["normalize"]))
    tol = PARITY_ATOL[str(state.dtype)]
    np.testing.assert_allclose(backend.to_numpy(s), case["out"], rtol=0, atol=tol)


@pytest.mark.parametrize("normalize", [True, False])
@pytest.mark.parametrize("nqubits,targets,results",
                         [(2, [0], [1]), (2, [1], [0]), (3, [1], [1]), (4, [1, 3], [1, 0]), (5, [1, 2, 4], [0, 1, 1]),
                          (15, [4, 7], [0, 0]), (16, [8, 12, 15], [1, 0, 1]), (20, [0, 1, 2, 3], [1, 0, 1, 1])])
def test_collapse_state(backend, nqubits, targets, results, normalize, dtype):
    """tests/test_ops.py:52-83: analytic slicing oracle."""
    atol = 1e-7 if dtype == "complex64" else 1e-14
    state = random_state(nqubits, 31, dtype)
    slicer = [slice(None)] * nqubits
    for t, r in zip(targets, results):
        slicer[t] = r
    init = state.reshape((2,) * nqubits).astype(np.complex128)
    target = np.zeros_like(init)
    target[tuple(slicer)] = init[tuple(slicer)]
    target = target.ravel()
    if normalize:
        target = target / np.sqrt((np.abs(target) ** 2).sum())
    result = int(np.array(results).dot(2 ** np.arange(len(results) - 1, -1, -1)))
    s = backend.cast(state, dtype=dtype, copy=True)
    backend.collapse_state(s, sorted(targets), np.array([result]), nqubits, normalize)
    np.testing.assert_allclose(backend.to_numpy(s), target, atol=atol)


def test_collapse_norm_is_fp64(backend):
    """complex64 state, normalisation computed in FP64: |psi|^2 sums to 1 within c64 rounding."""
    n = 22
    state = random_state(n, 32, "complex64")
    s = backend.cast(state, dtype="complex64", copy=True)
    backend.collapse_state(s, [3, 9], 2, n, True)
    out = backend.to_numpy(s).astype(np.complex128)
    assert abs((np.abs(out) ** 2).sum() - 1) < 1e-6


@pytest.mark.parametrize("out_dtype", ["float64", "float32"])
@pytest.mark.parametrize("qubits", [[0], [3, 1], [4, 0, 2], list(range(12)), [11, 0, 5, 7], [2, 9, 1, 0, 3, 11, 6],
                                    list(range(11, -1, -1)), [5, 6, 7, 8, 9, 10, 11]])
def test_probabilities(backend, qubits, out_dtype, dtype):
    n = 12
    state = random_state(n, 33, dtype)
    s = backend.cast(state, dtype=dtype)
    p = backend.to_numpy(backend.calculate_probabilities(s, qubits, n, out_dtype=out_dtype))
    assert p.dtype == np.dtype(out_dtype)
    want = O.probabilities(state, qubits, n)
    tol = 1e-14 if (out_dtype == "float64" and dtype == "complex128") else 2e-7
    np.testing.assert_allclose(p, want, rtol=0, atol=tol)


@pytest.mark.parametrize("n,qubits", [(24, [0, 1, 2]), (24, [23, 5]), (26, list(range(10))), (22, [21])])
def test_probabilities_large_marginals(backend, n, qubits):
    state = random_state(n, 34)
    p = backend.to_numpy(backend.calculate_probabilities(backend.cast(state), qubits, n))
    np.testing.assert_allclose(p, O.probabilities(state, qubits, n), rtol=1e-12, atol=1e-15)
    assert abs(p.sum() - 1) < 1e-12


def test_probabilities_default_dtype(backend, dtype):
    n = 6
    s = backend.cast(random_state(n, 35, dtype), dtype=dtype)
    p = backend.calculate_probabilities(s, [0, 1], n)
    assert str(p.dtype).endswith("float64" if dtype == "complex128" else "float32")


@pytest.mark.parametrize("realtype", ["float32", "float64"])
@pytest.mark.parametrize("inttype", ["int32", "int64"])
@pytest.mark.parametrize("nthreads", [None, 4])
def test_measure_frequencies(backend, realtype, inttype, nthreads):
    """tests/test_ops.py:236-256, including its known-answer vector (exact)."""
    probs = np.ones(16, dtype=realtype) / 16
    frequencies = np.zeros(16, dtype=inttype)
    if nthreads is None:
        nthreads = backend.nthreads
    frequencies = backend.measure_frequencies_op(frequencies, probs, nshots=1000, nqubits=4, seed=1234,
                                                 nthreads=nthreads)
    assert np.sum(frequencies) == 1000
    if nthreads == 4:
        target = np.array([72, 65, 63, 54, 57, 55, 67, 50, 53, 67, 69, 68, 64, 68, 66, 62], dtype=inttype)
        np.testing.assert_array_equal(frequencies, target)


@pytest.mark.parametrize("case", [c for c in golden_cases.load() if c["family"] == "freq"], ids=lambda c: c["id"])
def test_measure_frequencies_golden(backend, case):
    f = np.zeros(2 ** case["nqubits"], dtype=np.int64)
    f = backend.measure_frequencies_op(f, case["probs"], case["nshots"], case["nqubits"], case["seed"],
                                       case["nthreads"])
    np.testing.assert_array_equal(f, case["out"])


@pytest.mark.parametrize("nthreads", [1, 7, 64, 1000])
def test_measure_frequencies_vs_oracle(backend, nthreads):
    """Bit-exact against the C oracle on a 2^16-bin distribution from a random state."""
    n = 16
    probs = np.abs(random_state(n, 36)) ** 2
    want = O.measure_frequencies(np.zeros(2**n, dtype=np.int64), probs, 200000, n, 987, nthreads)
    got = backend.measure_frequencies_op(np.zeros(2**n, dtype=np.int64), probs, 200000, n, 987, nthreads)
    np.testing.assert_array_equal(got, want)


NONZERO = list(itertools.combinations(range(8), r=1))
NONZERO.extend(itertools.combinations(range(8), r=2))
NONZERO.extend(itertools.combinations(range(8), r=3))
NONZERO.extend(itertools.combinations(range(8), r=4))
NSHOTS = (len(NONZERO) // 2 + 1) * [1000, 200000]


@pytest.mark.parametrize("nonzero,nshots", list(zip(NONZERO, NSHOTS)))
def test_measure_frequencies_sparse_probabilities(backend, nonzero, nshots):
    probs = np.zeros(8, dtype=np.float64)
    for i in nonzero:
        probs[i] = 1
    probs = probs / np.sum(probs)
    frequencies = backend.sample_frequencies(probs, nshots)
    assert sum(frequencies.values()) == nshots
    for i, freq in frequencies.items():
        assert freq != 0
        assert i in nonzero


def _sampling_probs(nbits, seed, pdt, zeros=0.3):
    rng = np.random.default_rng(seed)
    p = rng.random(2**nbits)
    p[rng.random(2**nbits) < zeros] = 0
    p = (p / p.sum()).astype(pdt)
    return p / p.sum()


@pytest.mark.parametrize("pdt", ["float64", "float32"])
@pytest.mark.parametrize("nbits,nshots,seed", [(1, 10, 1), (5, 1000, 2), (12, 20000, 3), (20, 99999, 4)])
def test_sample_shots_is_numpy_choice(backend, nbits, nshots, seed, pdt):
    """Below SHOT_METROPOLIS_THRESHOLD the reference samples with numpy.random.choice
    (cpu.py:384-385 -> qibo sample_shots): same global-stream draws, same outcomes."""
    p = _sampling_probs(nbits, seed, pdt)
    np.random.seed(seed)
    want = np.random.choice(range(len(p)), size=nshots, p=p)
    np.random.seed(seed)
    got = backend.to_numpy(backend.sample_shots(backend.cast(p, dtype=pdt), nshots))
    np.testing.assert_array_equal(got, want)


def test_sample_frequencies_below_threshold_match_numpy(backend):
    from collections import Counter

    p = _sampling_probs(14, 5, "float64")
    np.random.seed(77)
    want = Counter(np.random.choice(range(len(p)), size=50000, p=p).tolist())
    np.random.seed(77)
    got = backend.sample_frequencies(backend.cast(p, dtype="float64"), 50000)
    assert got == want


def _two_level_cdf(p, block=4096):
    """Normalised FP64 CDF summed per block, with the block offsets added by Neumaier's
    compensated sum: rounding far below the plain cumsum's (~1e-14 against ~1e-13)."""
    inner = np.cumsum(p.astype(np.float64).reshape(-1, block), axis=1)
    off = np.zeros(inner.shape[0])
    s = c = 0.0
    for b in range(1, inner.shape[0]):
        x = float(inner[b - 1, -1])
        t = s + x
        c += (s - t) + x if abs(s) >= abs(x) else (x - t) + s
        s = t
        off[b] = s + c
    cdf = (inner + off[:, None]).ravel()
    return cdf / cdf[-1]


def test_sample_shots_large_state_vs_oracle(backend):
    """2^26 outcomes (CDF over 16384 blocks) and 10^6 draws against the oracle's FP64
    cumsum search.  The two cumulative sums add in different orders and differ by
    rounding only (the oracle's plain cumsum drifts by up to ~1e-12 over 2^26 terms):
    a draw lands in a neighbouring bin only when its uniform lies between the two
    CDF values of the boundary between those bins.  Every mismatch must be such a
    boundary case, and their number must stay within the Poisson bound of its
    expectation, draws * sum_k |cdf_oracle(k) - cdf_exact(k)|."""
    n = 26
    p = _sampling_probs(n, 6, "float32", zeros=0.5)
    u = np.random.default_rng(7).random(1000000)
    want = O.sample_shots(p, u)
    d = backend.cast(p, dtype="float32")
    import ctypes

    from qibojit_gb300 import _lib

    torch = pytest.importorskip("torch")
    out = torch.empty(len(u), dtype=torch.int64, device="cuda")
    freqs = torch.zeros(2**n, dtype=torch.int64, device="cuda")
    _lib.check(backend.lib.sv_sample_cdf(backend.ctx.handle, d.data_ptr(), _lib.SV_F32, n,
                                         u.ctypes.data_as(ctypes.c_void_p), len(u), freqs.data_ptr(), out.data_ptr()))
    got = out.cpu().numpy()
    bad = np.nonzero(got != want)[0]
    cdf = np.cumsum(p.astype(np.float64))
    cdf /= cdf[-1]
    exact = _two_level_cdf(p)
    for i in bad:
        lo, hi = sorted((int(got[i]), int(want[i])))
        assert np.all(p[lo + 1:hi] == 0), "a mismatch skips a non-empty bin"
        assert abs(u[i] - cdf[lo]) <= abs(cdf[lo] - exact[lo]) + 1e-14, "a mismatch away from a bin boundary"
    expected = len(u) * float(np.abs(cdf - exact).sum())
    assert len(bad) <= 3 * expected + 5, (len(bad), expected)
    assert np.all(p[got] > 0)
    assert int(freqs.sum()) == len(u)
    np.testing.assert_array_equal(np.bincount(got, minlength=2**n), freqs.cpu().numpy())


def test_host_buffer_is_pinned_and_zero(backend):
    buf = backend.host_buffer(12, "complex64")
    assert buf.is_pinned() and buf.numel() == 4096 and str(buf.dtype) == "torch.complex64"
    assert not bool(buf.abs().max() > 0)
    d = backend.cast(buf, dtype="complex64")
    assert d.is_cuda and d.numel() == 4096
