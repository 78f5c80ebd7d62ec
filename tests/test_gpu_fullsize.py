"""Size-independent properties at the benchmark's full sizes (n=28-30): norm
preservation with FP64 reductions, complex64 vs complex128 agreement, fused vs per-gate
agreement, collapse and probability invariants, and exact sampling against the oracle
on a large distribution."""
import numpy as np
import pytest

from oracle import pyoracle as O
from qibojit_gb300 import circuits
from tests.circuits_random import random_circuit

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    return MetaBackend.load("gb300")


@pytest.fixture(scope="module")
def brickwork30(backend):
    import torch

    circ = circuits.brickwork(30, 20, 1234)
    s64 = backend.compile(circ, "complex64").run(backend.zero_state(30, dtype="complex64"))
    s128 = backend.compile(circ, "complex128").run(backend.zero_state(30, dtype="complex128"))
    torch.cuda.synchronize()
    yield s64, s128
    del s64, s128
    torch.cuda.empty_cache()


def test_brickwork30_precision(backend, brickwork30):
    s64, s128 = brickwork30
    n = 30
    assert abs(backend.norm2(s128, n) - 1) < 1e-12
    assert abs(backend.norm2(s64, n) - 1) < 2e-6
    ip = backend.inner_product(s128, s64, n)
    assert 1 - abs(ip) ** 2 < 2e-6
    assert backend.max_abs_diff(s64, s128, n) < 1e-8
    assert abs(backend.expectation_z(s64, [0, 1], n) - backend.expectation_z(s128, [0, 1], n)) < 1e-5


def test_brickwork30_collapse_and_probabilities(backend, brickwork30):
    _, s128 = brickwork30
    n = 30
    p = backend.to_numpy(backend.calculate_probabilities(s128, [0, 1, 2, 3], n))
    assert abs(p.sum() - 1) < 1e-12
    s = s128.clone()
    backend.collapse_state(s, [0, 1, 2, 3], 5, n, True)
    assert abs(backend.norm2(s, n) - 1) < 1e-12
    pc = backend.to_numpy(backend.calculate_probabilities(s, [0, 1, 2, 3], n))
    assert abs(pc[5] - 1) < 1e-12 and np.abs(np.delete(pc, 5)).max() == 0.0
    # the kept amplitudes are the old ones divided by sqrt(p[5])
    blk = 1 << (n - 4)
    old = backend.to_numpy(s128[5 * blk: 5 * blk + 4096])
    new = backend.to_numpy(s[5 * blk: 5 * blk + 4096])
    np.testing.assert_allclose(new, old / np.sqrt(p[5]), rtol=1e-12, atol=1e-18)


def test_random_circuit_n28_fused_vs_per_gate(backend):
    n = 28
    circ = random_circuit(n, 80, 77, families=["one", "one_p", "two_c", "two_p", "swap", "fsim", "u2q", "zc", "ccz",
                                               "toffoli", "u3q"])
    a = backend.execute_circuit(circ, backend.zero_state(n), fuse=True)
    b = backend.execute_circuit(circ, backend.zero_state(n), fuse=False)
    assert backend.max_abs_diff(a, b, n) < 1e-12
    assert abs(backend.norm2(a, n) - 1) < 1e-11


def test_sampling_large_distribution_exact(backend):
    n = 24
    rng = np.random.default_rng(5)
    probs = rng.random(2**n)
    probs /= probs.sum()
    want = O.measure_frequencies(np.zeros(2**n, dtype=np.int64), probs, 100000, n, 2024, 16)
    got = backend.measure_frequencies_op(np.zeros(2**n, dtype=np.int64), probs, 100000, n, 2024, 16)
    np.testing.assert_array_equal(got, want)
