"""Dense numpy application of a gate, the role qibo's NumpyBackend plays as the
reference suite's oracle (tests/test_gates.py of qibojit): the target matrix is
applied with tensordot on the slice where every control qubit is 1."""
import numpy as np


def apply_dense(state, matrix, targets, controls, nqubits):
    psi = np.array(state, dtype=np.complex128).reshape((2,) * nqubits)
    k = len(targets)
    u = np.asarray(matrix, dtype=np.complex128).reshape((2,) * (2 * k))
    sl = [slice(None)] * nqubits
    for c in controls:
        sl[c] = 1
    sl = tuple(sl)
    sub = psi[sl]
    # axes of the remaining tensor after slicing away the controls
    remaining = [q for q in range(nqubits) if q not in controls]
    axes = [remaining.index(t) for t in targets]
    out = np.tensordot(u, sub, axes=(list(range(k, 2 * k)), axes))
    out = np.moveaxis(out, list(range(k)), axes)
    psi = psi.copy()
    psi[sl] = out
    return psi.ravel()


def random_state(n, seed, dtype="complex128"):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(2**n) + 1j * rng.standard_normal(2**n)
    return (x / np.linalg.norm(x)).astype(dtype)


def random_unitary(d, seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def random_complex(shape, seed, dtype="complex128"):
    rng = np.random.default_rng(seed)
    return (rng.random(shape) + 1j * rng.random(shape)).astype(dtype)
