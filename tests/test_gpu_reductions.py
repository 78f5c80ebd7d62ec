"""FP64 reductions (inner product, max difference, Z-string expectations)."""
import numpy as np
import pytest

from tests.dense import random_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from qibojit_gb300 import MetaBackend

    return MetaBackend.load("gb300")


@pytest.mark.parametrize("da,db", [("complex128", "complex128"), ("complex64", "complex128"),
                                   ("complex64", "complex64"), ("float64", "complex128")])
def test_inner_product_and_maxdiff(backend, da, db):
    n = 16
    a = random_state(n, 1).astype(da) if da.startswith("complex") else np.abs(random_state(n, 1)).astype(da)
    b = random_state(n, 2).astype(db)
    ta, tb = backend.cast(a, dtype=da), backend.cast(b, dtype=db)
    got = backend.inner_product(ta, tb, n)
    want = np.vdot(a.astype(np.complex128), b.astype(np.complex128))
    assert abs(got - want) < 1e-13
    md = backend.max_abs_diff(ta, tb, n)
    assert abs(md - np.abs(a.astype(np.complex128) - b).max()) < 1e-15


@pytest.mark.parametrize("qubits", [[], [0], [0, 1], [3, 7, 11], [15]])
def test_expectation_z(backend, qubits, dtype):
    n = 16
    x = random_state(n, 3, dtype)
    got = backend.expectation_z(backend.cast(x, dtype=dtype), qubits, n)
    p = np.abs(x.astype(np.complex128)) ** 2
    idx = np.arange(2**n)
    sign = np.ones(2**n)
    for q in qubits:
        sign *= 1 - 2 * ((idx >> (n - 1 - q)) & 1)
    assert abs(got - (sign * p).sum()) < 1e-13


def test_zz_sign_pattern(backend):
    """<Z0 Z1> is +1/-1/-1/+1 on the four top-bit quarters (|00>, |01>, |10>, |11> on qubits 0, 1)."""
    n = 12
    for k, want in enumerate([1, -1, -1, 1]):
        x = np.zeros(2**n, dtype=np.complex128)
        x[k << (n - 2)] = 1
        assert backend.expectation_z(backend.cast(x), [0, 1], n) == want
